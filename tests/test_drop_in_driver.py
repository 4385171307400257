"""The C++ drop-in driver (life_gb300/host/life_main.cpp) builds against an
unmodified LIFE case directory (its params.h + input/geometry.config), and on
the GPU writes a Fluid.restart equal to the reference's own dump. Run twice in
one directory it resumes from its own restart set, as the reference's main
does, and ends where one uninterrupted run of twice the steps ends."""
import os
import subprocess

import numpy as np
import pytest

from cases import golden_cases
from life_gb300.case import geometry_config_text
from life_gb300.restart import read_fluid_restart

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def build_driver(tmp_path, name, params=None, tag=""):
    from life_gb300.build import build
    lib = build()
    p, bodies = golden_cases()[name]
    if params is not None:
        p = params
    case = tmp_path / (name + tag)
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


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cylinder_rigid_cm", "filament_flex_deflect", "honami_like_cm"])
def test_driver_resumes_from_its_restart_set(tmp_path, name):
    import dataclasses
    p, _ = golden_cases()[name]
    n = 30
    half = dataclasses.replace(p, nSteps=n, tRestart=n, tinfo=n, tVTK=n)
    full = dataclasses.replace(p, nSteps=2 * n, tRestart=2 * n, tinfo=2 * n, tVTK=2 * n)
    case_a, exe_a = build_driver(tmp_path, name, half, "_half")
    for _ in range(2):
        res = subprocess.run([str(exe_a)], cwd=case_a, capture_output=True, text=True)
        assert res.returncode == 0, res.stdout[-2000:]
    assert "Restarting from time step 30" in res.stdout
    case_b, exe_b = build_driver(tmp_path, name, full, "_full")
    res = subprocess.run([str(exe_b)], cwd=case_b, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:]
    for fn in ("Fluid.restart", "IBM.restart", "FEM.restart"):
        fa, fb = case_a / "Results" / "Restart" / fn, case_b / "Results" / "Restart" / fn
        assert fa.exists() == fb.exists(), fn
        if fa.exists():
            assert fa.read_bytes() == fb.read_bytes(), fn
    assert (case_a / "Results" / "Restart" / "FEM.restart").exists() == (name != "cylinder_rigid_cm")
