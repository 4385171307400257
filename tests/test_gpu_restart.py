"""Restart sets on the GPU: a case stopped after N1 steps is written as the
reference's Fluid.restart / IBM.restart / FEM.restart (life_gb300.restart.
save_case), loaded into a fresh case of the same geometry (load_case: the
reference's readRestart rules -- fields, markers by body ID with support, ds
and epsilon recomputed, FEM vectors, element lengths and angles with their
transforms recomputed, nodes, Aitken factor), and continued N2 steps. In FP64
the continuation equals the uninterrupted run bit for bit. In FP32 the load
re-forms the stored populations from the FP64 restart fields, so the
continuation is held to 1e-6 relative velocity.
"""
import dataclasses

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu
NAMES = ["cavity_cm", "channel_convective_freeslip_cm", "cylinder_rigid_cm", "cylinders_uni_bgk",
         "filament_flex_deflect", "turek_like_uni", "honami_like_cm", "filament_supported_and_rigid",
         "womersley_gravity_cm", "pressure_ywalls_convective_cm"]
N1, N2 = 40, 33


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


def _state(c):
    out = dict(c.fields())
    if c.n_markers:
        mk = c.markers()
        out["marker_pos"], out["marker_force"], out["eps"] = mk["pos"], mk["force"], mk["epsilon"]
    for k in range(c.n_flex):
        d = c.fem(k)
        out[f"fem{k}_U"], out[f"fem{k}_pos"] = d["U"], d["pos"]
    return out


@pytest.mark.parametrize("prec", [0, 1], ids=["f64", "f32"])
@pytest.mark.parametrize("name", NAMES)
def test_restart_set_continues_the_run(name, prec, tmp_path):
    from life_gb300.lib import Case
    from life_gb300.restart import load_case, save_case
    p, b = golden_cases()[name]
    p = dataclasses.replace(p, precision=prec)
    with Case(p, b) as A:
        A.step(N1)
        save_case(A, str(tmp_path))
        A.step(N2)
        ref = _state(A)
    with Case(p, b) as B:
        assert load_case(B, str(tmp_path)) == N1
        B.step(N2)
        assert B.t == N1 + N2
        got = _state(B)
    for key in ref:
        if prec == 0:
            assert np.array_equal(got[key], ref[key]), key
        elif key == "u":
            err = np.abs(got[key] - ref[key]).max() / np.abs(ref[key]).max()
            assert err < 1e-6, (key, err)


def test_restart_files_round_trip(tmp_path):
    from life_gb300.lib import Case
    from life_gb300.restart import read_fem_restart, read_ibm_restart, save_case
    p, b = golden_cases()["filament_supported_and_rigid"]
    with Case(p, b) as A:
        A.step(20)
        save_case(A, str(tmp_path))
        mk, bo = A.markers(), A.bodies()
        fem = A.fem(0)
        relax = A.relax()
    ir = read_ibm_restart(str(tmp_path / "IBM.restart"))
    assert ir.ids == [int(x) for x in bo["ids"]]
    assert np.array_equal(np.vstack(ir.pos), mk["pos"]) and np.array_equal(np.vstack(ir.force), mk["force"])
    fr = read_fem_restart(str(tmp_path / "FEM.restart"))
    assert fr.relax == relax and len(fr.bodies) == 1
    assert np.array_equal(fr.bodies[0].U, fem["U"]) and np.array_equal(fr.bodies[0].pos0, fem["pos0"])
