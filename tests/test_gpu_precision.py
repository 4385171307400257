"""Reduced-precision storage forms against the FP64 reference dumps.

The FP32 form stores shifted populations f - w and collides in FP32; the
FP16 form stores (f - w)/s_v with power-of-two per-direction scales. Both must
stay within a stated velocity error of the reference's FP64 result after the
full golden run (hundreds of steps). Tolerances (relative to max |u|):
FP32 <= 1e-5, FP16 <= 1e-2 (measured worst case 5.5e-3, on the slowest flow).

One case has a looser FP32 bound. With pressure conditions on both y walls
and fluid crossing them, a uniform vertical velocity is a neutral mode of the
flow: the walls take it from their neighbours (zero-gradient extrapolation)
and nothing damps it. The FP32 rounding therefore accumulates in that mode
instead of decaying. On pressure_ywalls_convective_cm the FP32 velocity error
grows about linearly (6.6e-8 per step, at the top wall next to the outlet) to
2.0e-5 after the 300 steps. The same case with solid y walls stays at 1.7e-6.
"""
import os

import numpy as np
import pytest

from cases import golden_cases
from life_gb300.case import PREC_F16, PREC_F32

pytestmark = pytest.mark.gpu
CASES = golden_cases()
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {PREC_F32: 1e-5, PREC_F16: 1e-2}
TOL_CASE = {("pressure_ywalls_convective_cm", PREC_F32): 3e-5}
NAMES = [k for k, (_, b) in CASES.items() if not any(getattr(x, "flexible", False) for x in b)]


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


@pytest.mark.parametrize("prec", [PREC_F32, PREC_F16], ids=["f32", "f16"])
@pytest.mark.parametrize("name", NAMES)
def test_velocity_error_vs_reference(name, prec):
    from life_gb300.lib import Case
    p, b = CASES[name]
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    with Case(p.replace(precision=prec), b) as c:
        c.step(p.nSteps)
        fl = c.fields(("rho", "u"))
    scale = np.abs(g["u"]).max()
    err = np.abs(fl["u"] - g["u"]).max() / scale
    assert err <= TOL_CASE.get((name, prec), TOL[prec]), err
    assert np.abs(fl["rho"] - g["rho"]).max() < 50 * TOL[prec]


def test_fp32_interior_matches_fp64_one_step_from_same_state():
    """One step from an identical (FP32-representable) state: the FP32 fast
    path and the FP64 path agree to FP32 rounding."""
    from life_gb300.lib import Case
    p, b = CASES["cavity_cm"]
    with Case(p, b) as c64:
        c64.step(50)
        st = c64.fields()
    f = st["f"]
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    f32 = (f - w).astype(np.float32).astype(np.float64) + w
    with Case(p, b) as a, Case(p.replace(precision=PREC_F32), b) as q:
        a.set_fields(50, st["rho"], st["u"], f32, st["force_ibm"])
        q.set_fields(50, st["rho"], st["u"], f32, st["force_ibm"])
        a.step(1)
        q.step(1)
        ua, uq = a.fields(("u",))["u"], q.fields(("u",))["u"]
    assert np.abs(ua - uq).max() / np.abs(ua).max() < 2e-6


def test_fp32_body_forces_and_tip_vs_fp64():
    """The immersed-body observables the FP32 form is stated for: drag and
    lift of the 1000 x 400 rigid cylinder (central moments, D = 40, Re = 100)
    over 4000 steps, and the tip displacement of the 1200 x 400 clamped
    filament (80 corotational elements, FEM/epsilon/Aitken in FP64) over 600
    steps, both against the FP64 form (bit-identical to the reference).
    Tolerances: Cd within 1e-3 relative at every sample, Cl within 1e-3 of
    the mean drag, tip within 1e-6 L (measured over 50,000 and 2,000 steps:
    7.9e-4, 3.5e-3 of the lift amplitude, 8.2e-8 L)."""
    import bench
    r = {prec: bench.cylinder_forces(prec, 4000, every=100) for prec in (0, PREC_F32)}
    a, q = r[0], r[PREC_F32]
    assert len(a["cd"]) == 40
    cd_scale = float(np.abs(a["cd"]).mean())
    assert cd_scale > 0.5
    assert np.abs(q["cd"] - a["cd"]).max() <= 1e-3 * cd_scale
    assert np.abs(q["cl"] - a["cl"]).max() <= 1e-3 * cd_scale
    t64 = bench.filament_tip(0, 600, every=100)["tip"]
    t32 = bench.filament_tip(PREC_F32, 600, every=100)["tip"]
    assert abs(t64[0]) > 1e-3  # the seeded deflection is visible
    assert np.abs(t32 - t64).max() <= 1e-6
