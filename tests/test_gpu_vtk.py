"""VTK output from the GPU state (life_case_get_vtk_fields, formed on the
device in VTK point order; markers and FEM nodes from their getters) against
the files the reference wrote for the same cases (tests/golden/make_vtk.py).

Lattice-only and rigid-body cases are bit-identical to the reference on the
GPU, so every file (Fluid.vti, IBM.vtp at t = 0, nSteps/2, nSteps) must be
byte for byte the reference's. For flexible bodies the XML part must be
identical and the raw numbers within the flexible-body tolerances of
tests/test_gpu_fsi.py (the trigonometry differs in the last bit)."""
import hashlib
import os

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


@pytest.mark.parametrize("name", ["cavity_cm", "cylinder_rigid_cm"])
def test_gpu_vtk_byte_identical(name, tmp_path):
    from life_gb300 import vtk
    from life_gb300.lib import Case
    p, b = golden_cases()[name]
    g = np.load(os.path.join(GOLD, f"vtk_{name}.npz"))
    with Case(p, b) as c:
        for t in (0, p.nSteps // 2, p.nSteps):
            c.step(t - c.t)
            paths = vtk.write_vtk(c, str(tmp_path))
            for path in paths:
                fname = os.path.basename(path)
                key = fname.replace(".", "_")
                data = open(path, "rb").read()
                assert len(data) == int(g["size_" + key]), fname
                assert hashlib.sha256(data).hexdigest() == str(g["sha_" + key]), fname


def _split(data: bytes):
    k = data.index(b"_", data.index(b"<AppendedData")) + 1
    return data[:k], data[k:]


@pytest.mark.parametrize("name", ["filament_flex_deflect", "honami_like_cm"])
def test_gpu_vtk_flexible_bodies(name, tmp_path):
    from life_gb300 import vtk
    from life_gb300.lib import Case
    p, b = golden_cases()[name]
    g = np.load(os.path.join(GOLD, f"vtk_{name}.npz"))
    with Case(p, b) as c:
        c.step(p.nSteps)
        paths = vtk.write_vtk(c, str(tmp_path), fem=True)
    assert sorted(os.path.basename(x) for x in paths) == sorted(
        [f"Fluid.{p.nSteps}.vti", f"IBM.{p.nSteps}.vtp", f"FEM.{p.nSteps}.vtp"])
    for path in paths:
        key = os.path.basename(path).replace(".", "_")
        got, ref = open(path, "rb").read(), g["bytes_" + key].tobytes()
        gh, graw = _split(got)
        rh, rraw = _split(ref)
        assert gh == rh and len(graw) == len(rraw), key
        # raw blocks: a UInt64 byte count, then Float64 / Int64 data; the
        # Int64 connectivity is identical, the Float64 data within tolerance
        a = np.frombuffer(graw[:-len(b"\n\t</AppendedData>\n</VTKFile>\n")], dtype=np.uint8)
        r = np.frombuffer(rraw[:-len(b"\n\t</AppendedData>\n</VTKFile>\n")], dtype=np.uint8)
        assert a.size == r.size and a.size % 8 == 0
        af, rf = a.view(np.float64), r.view(np.float64)
        same = a.view(np.int64) == r.view(np.int64)
        scale = np.abs(rf[np.isfinite(rf)]).max()
        assert np.all(same | (np.abs(af - rf) <= 1e-11 * scale)), key
