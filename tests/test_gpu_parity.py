"""GPU FP64 path against the reference (golden dumps) and the oracle.

All calls go through the C-ABI (life_gb300.lib). Lattice-only cases must
match the reference's own dumps bit for bit. Cases with rigid bodies use the
textbook-order LU at start-up, so they must match the oracle (and the
reference built against the textbook LAPACK shim) bit for bit.
"""
import hashlib
import os

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu

CASES = golden_cases()
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LATTICE = [k for k, (_, b) in CASES.items() if not b]
RIGID = [k for k, (_, b) in CASES.items() if b and not any(getattr(x, "flexible", False) for x in b)]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


@pytest.mark.parametrize("name", LATTICE)
def test_lattice_bit_exact_vs_reference(name):
    from life_gb300.lib import Case
    p, b = CASES[name]
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    with Case(p, b) as c:
        c.step(p.nSteps)
        assert c.t == int(g["t"])
        fl = c.fields()
    for key in ("f", "rho", "u", "force_ibm"):
        assert np.array_equal(fl[key], g[key]), (key, np.abs(fl[key] - g[key]).max())


@pytest.mark.parametrize("name", RIGID)
def test_rigid_bodies_bit_exact(name):
    from life_gb300.lib import Case
    p, b = CASES[name]
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    with Case(p, b) as c:
        c.step(p.nSteps)
        fl, mk = c.fields(), c.markers()
    got = dict(f=fl["f"], rho=fl["rho"], u=fl["u"], force_ibm=fl["force_ibm"], ibm_pos=mk["pos"],
               ibm_vel=mk["vel"], ibm_force=mk["force"])
    for key, arr in got.items():
        assert digest(arr) == str(g["sha_textbook_" + key]), key
    # and close to the reference's own OpenBLAS numerics
    err = np.abs(fl["u"] - g["u"]).max() / np.abs(g["u"]).max()
    assert err < 1e-12, err


def test_initial_state_export_matches_oracle():
    from life_gb300.lib import Case
    from oracle.pyoracle import Oracle
    p, b = CASES["channel_convective_freeslip_cm"]
    o = Oracle(p, b)
    with Case(p, b) as c:
        a, r = c.fields(), o.fields()
        for key in ("f", "rho", "u"):
            assert np.array_equal(a[key], r[key]), key
        for n in (1, 2, 7):
            c.step(n)
            o.step(n)
            a, r = c.fields(), o.fields()
            for key in ("f", "rho", "u"):
                assert np.array_equal(a[key], r[key]), (key, c.t)


@pytest.mark.parametrize("name", ["velocity_walls_shear", "channel_pressure_ramp"])
def test_restart_roundtrip_matches_uninterrupted_run(name):
    """set_fields (GridClass::readRestart) then stepping equals one long run.

    A restart file holds f and u, which is all the next step reads, including
    the convective outlet (f_n and u of the previous step)."""
    from life_gb300.lib import Case
    p, b = CASES[name]
    with Case(p, b) as c1:
        c1.step(60)
        mid = c1.fields()
        c1.step(40)
        end = c1.fields()
    with Case(p, b) as c2:
        c2.set_fields(60, mid["rho"], mid["u"], mid["f"], mid["force_ibm"])
        again = c2.fields()
        assert np.array_equal(again["f"], mid["f"])
        c2.step(40)
        end2 = c2.fields()
    for key in ("f", "rho", "u"):
        assert np.array_equal(end[key], end2[key]), key


def test_max_velocity_matches_fields():
    from life_gb300.lib import Case
    p, b = CASES["cavity_bgk"]
    with Case(p, b) as c:
        c.step(37)
        m, nan = c.max_velocity()
        u = c.fields(("u",))["u"]
    assert not nan
    assert m == np.sqrt(u[:, 0] ** 2 + u[:, 1] ** 2).max()


def test_fields_into_caller_buffers():
    """fields(out=...) fills the caller's arrays with exactly what the
    allocating call returns, and rejects arrays of the wrong shape or type."""
    from life_gb300.lib import Case
    p, b = CASES["cylinder_rigid_cm"]
    with Case(p, b) as c:
        c.step(11)
        ref = c.fields()
        n = p.Nx * p.Ny
        out = {"rho": np.full(n, np.nan), "u": np.full((n, 2), np.nan), "f": np.full((n, 9), np.nan),
               "force_ibm": np.full((n, 2), np.nan)}
        got = c.fields(out=out)
        for key in ("rho", "u", "f", "force_ibm"):
            assert got[key] is out[key]
            assert np.array_equal(out[key], ref[key]), key
        with pytest.raises(ValueError):
            c.fields(("u",), out={"u": np.zeros((n, 3))})
        with pytest.raises(ValueError):
            c.fields(("u",), out={"u": np.zeros((n, 2), dtype=np.float32)})
