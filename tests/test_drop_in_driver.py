"""The C++ drop-in driver (life_gb300/host/life_main.cpp over the
reference-interface classes of include/life_ref_shim, implemented in
life_gb300/host/ref_shim.cpp) builds against an unmodified LIFE case
directory (its params.h + input/geometry.config), and so does the
reference's own src/main.cpp, unchanged, when the reference tree is present.

On the GPU the driver writes a Fluid.restart equal to the reference's own
dump, VTK files byte-identical to the reference's, and the reference's
TotalForces.out; run twice in one directory it resumes from its own restart
set, as the reference's main does, and ends where one uninterrupted run of
twice the steps ends."""
import os
import subprocess

import numpy as np
import pytest

from cases import golden_cases
from life_gb300.case import geometry_config_text
from life_gb300.restart import read_fluid_restart

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


REF = os.environ.get("LIFE_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
SHIM_FLAGS = ["-I", os.path.join(ROOT, "include", "life_ref_shim"), "-I", os.path.join(ROOT, "include"),
              "-I", os.path.join(ROOT, "include", "life_ref_defs")]


def write_case(tmp_path, name, params=None, tag=""):
    p, bodies = golden_cases()[name]
    if params is not None:
        p = params
    case = tmp_path / (name + tag)
    (case / "input").mkdir(parents=True)
    (case / "params.h").write_text(p.to_params_h())
    if bodies:
        (case / "input" / "geometry.config").write_text(geometry_config_text(bodies))
    return case


def build_driver(tmp_path, name, params=None, tag="", main=None):
    from life_gb300.build import build
    lib = build()
    case = write_case(tmp_path, name, params, tag)
    exe = case / "LIFE_gb300"
    libdir = os.path.dirname(lib)
    main = main or os.path.join(ROOT, "life_gb300", "host", "life_main.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(case), *SHIM_FLAGS, main,
                    os.path.join(ROOT, "life_gb300", "host", "ref_shim.cpp"), "-L", libdir, "-llife_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return case, exe


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "src", "main.cpp")), reason="reference tree not present")
def test_reference_main_compiles_unchanged_against_the_shim(tmp_path):
    """The reference's main.cpp includes "../inc/Grid.h", "../inc/Objects.h"
    and "../inc/Utils.h": in a copy of its tree where inc/ holds the shim's
    headers and the case's params.h, the unchanged file compiles and links
    against the GB300 library."""
    import shutil
    src, inc = tmp_path / "ref" / "src", tmp_path / "ref" / "inc"
    src.mkdir(parents=True)
    inc.mkdir()
    shutil.copyfile(os.path.join(REF, "src", "main.cpp"), src / "main.cpp")
    for h in ("Grid.h", "Objects.h", "Utils.h"):
        shutil.copyfile(os.path.join(ROOT, "include", "life_ref_shim", h), inc / h)
    p, _ = golden_cases()["cylinder_rigid_cm"]
    (inc / "params.h").write_text(p.to_params_h())
    from life_gb300.build import build
    libdir = os.path.dirname(build())
    exe = tmp_path / "LIFE"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-I", str(inc), "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "include", "life_ref_defs"), str(src / "main.cpp"),
                    os.path.join(ROOT, "life_gb300", "host", "ref_shim.cpp"), "-L", libdir, "-llife_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    assert exe.exists()


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
    assert "READ IN RESTART DATA" in res.stdout and "Restarting from time step 30" in res.stdout
    case_b, exe_b = build_driver(tmp_path, name, full, "_full")
    res = subprocess.run([str(exe_b)], cwd=case_b, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:]
    for fn in ("Fluid.restart", "IBM.restart", "FEM.restart"):
        fa, fb = case_a / "Results" / "Restart" / fn, case_b / "Results" / "Restart" / fn
        assert fa.exists() == fb.exists(), fn
        if fa.exists():
            assert fa.read_bytes() == fb.read_bytes(), fn
    assert (case_a / "Results" / "Restart" / "FEM.restart").exists() == (name != "cylinder_rigid_cm")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cylinder_rigid_cm", "filament_flex_deflect"])
def test_driver_writes_the_reference_vtk_and_forces(tmp_path, name):
    """With VTK, VTK_FEM, FORCES and TIPS on, the driver's output files are
    the reference's: VTK byte for byte for the rigid case (bit-identical on
    the GPU), within the flexible-body tolerance otherwise; TotalForces.out to
    its printed digits."""
    import hashlib
    from life_gb300.observables import parse_table
    p, _ = golden_cases()[name]
    p = p.replace(vtk=True, vtk_fem=True, tVTK=p.nSteps // 2)
    case, exe = build_driver(tmp_path, name, p, "_vtk")
    res = subprocess.run([str(exe)], cwd=case, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:]
    g = np.load(os.path.join(GOLD, f"vtk_{name}.npz"))
    vdir = case / "Results" / "VTK"
    assert sorted(os.listdir(vdir)) == sorted(str(x) for x in g["names"])
    for fname in os.listdir(vdir):
        data = (vdir / fname).read_bytes()
        key = fname.replace(".", "_")
        assert len(data) == int(g["size_" + key]), fname
        if name == "cylinder_rigid_cm":
            assert hashlib.sha256(data).hexdigest() == str(g["sha_" + key]), fname
        elif "bytes_" + key in g:
            ref = g["bytes_" + key].tobytes()
            k = data.index(b"_", data.index(b"<AppendedData")) + 1
            assert data[:k] == ref[:k], fname
    gt = np.load(os.path.join(GOLD, f"{name}.npz"))
    a = parse_table((case / "Results" / "TotalForces.out").read_text())
    r = parse_table(str(gt["total_forces_text"]))
    assert a.shape == r.shape and np.array_equal(a[:, :2], r[:, :2])
    tol = (1e-9 if name == "cylinder_rigid_cm" else 1e-7) * np.abs(r[:, 2:])
    assert np.all(np.abs(a[:, 2:] - r[:, 2:]) <= tol), (a, r)
