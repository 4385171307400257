"""The C++ drop-in driver (life_gb300/host/life_main.cpp) builds against an
unmodified LIFE case directory (its params.h + input/geometry.config), and on
the GPU writes a Fluid.restart equal to the reference's own dump."""
import os
import subprocess

import numpy as np
import pytest

from cases import golden_cases
from life_gb300.case import geometry_config_text
from life_gb300.restart import read_fluid_restart

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def build_driver(tmp_path, name):
    from life_gb300.build import build
    lib = build()
    p, bodies = golden_cases()[name]
    case = tmp_path / name
    (case / "input").mkdir(parents=True)
    (case / "params.h").write_text(p.to_params_h())
    if bodies:
        (case / "input" / "geometry.config").write_text(geometry_config_text(bodies))
    exe = case / "LIFE_gb300"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-O2", "-std=c++17", "-include", str(case / "params.h"),
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "include", "life_ref_defs"),
                    os.path.join(ROOT, "life_gb300", "host", "life_main.cpp"), "-L", libdir, "-llife_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return case, exe


@pytest.mark.parametrize("name", ["cavity_bgk", "cylinder_rigid_cm"])
def test_driver_builds_against_case_params(tmp_path, name):
    case, exe = build_driver(tmp_path, name)
    assert exe.exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["channel_convective_freeslip_cm", "cylinders_uni_bgk"])
def test_driver_restart_dump_matches_reference(tmp_path, name):
    import hashlib
    case, exe = build_driver(tmp_path, name)
    res = subprocess.run([str(exe)], cwd=case, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:]
    assert "MLUPS" in res.stdout
    r = read_fluid_restart(str(case / "Results" / "Restart" / "Fluid.restart"))
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    assert r.t == int(g["t"])
    if "sha_textbook_f" in g and "ibm_pos" in g:
        dig = lambda a: hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()  # noqa: E731
        assert dig(r.f) == str(g["sha_textbook_f"])
        assert dig(r.u) == str(g["sha_textbook_u"])
    else:
        assert np.array_equal(r.f, g["f"])
        assert np.array_equal(r.u, g["u"])
        assert np.array_equal(r.rho, g["rho"])
