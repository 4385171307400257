"""Flexible bodies (corotational FEM + Newmark + Aitken FSI) on the GPU.

Start-up (static pre-deflection, support, ds, epsilon) runs on the host with
the textbook-order LU and must equal the oracle bit for bit. Time stepping
runs the FEM on the device in FP64; its trigonometric functions (atan2, sin,
cos) are CUDA's, which can differ from the C library's in the last bit, and
the Aitken factor (a ratio of differences of successive iterates) magnifies
such differences, so parity after N steps is a tolerance:
  lattice fields  <= 1e-11 relative, IBM forces <= 1e-9 relative,
  marker / FEM node positions <= 1e-11 absolute (lattice units).
(measured worst cases on these fixtures: 2.3e-12, 2.1e-11, well below 1e-12).
The reference's own dumps (OpenBLAS LU) are held to the same bounds.
"""
import os

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu
CASES = golden_cases()
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLEX = [k for k, (_, b) in CASES.items() if any(getattr(x, "flexible", False) for x in b)]


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name", FLEX)
def test_startup_state_bit_exact(name):
    from life_gb300.lib import Case
    from oracle.pyoracle import Oracle
    p, b = CASES[name]
    o = Oracle(p, b)
    with Case(p, b) as c:
        mg, mo = c.markers(), o.markers()
        for key in ("pos", "vel", "epsilon", "ds"):
            assert np.array_equal(mg[key], mo[key]), key
        for k in range(c.n_flex):
            fg, fo = c.fem(k), o.fem(k)
            for key in ("U", "pos", "angle", "el_L", "el_angle"):
                assert np.array_equal(fg[key], fo[key]), (k, key)


@pytest.mark.parametrize("name", FLEX)
def test_fsi_run_matches_oracle_and_reference(name):
    from life_gb300.lib import Case
    from oracle.pyoracle import Oracle
    p, b = CASES[name]
    g = np.load(os.path.join(GOLD, f"{name}.npz"))
    o = Oracle(p, b)
    o.step(p.nSteps)
    with Case(p, b) as c:
        c.step(p.nSteps)
        fl, mk = c.fields(), c.markers()
        fem = [c.fem(k) for k in range(c.n_flex)]
        st = c.status()
    fo, mo = o.fields(), o.markers()
    femo = [o.fem(k) for k in range(o.n_flex)]
    report = {}
    for ref_name, F, Mk, FE in (("oracle", fo, mo, femo),
                                ("reference", g, {"force": g["ibm_force"], "pos": g["ibm_pos"]}, None)):
        for key in ("f", "rho", "u"):
            report[(ref_name, key)] = rel(fl[key], F[key])
            assert report[(ref_name, key)] < 1e-11, (ref_name, key, report[(ref_name, key)])
        report[(ref_name, "force_ibm")] = rel(fl["force_ibm"], F["force_ibm"])
        assert report[(ref_name, "force_ibm")] < 1e-9
        report[(ref_name, "marker_force")] = rel(mk["force"], Mk["force"])
        assert report[(ref_name, "marker_force")] < 1e-9
        assert np.abs(mk["pos"] - Mk["pos"]).max() < 1e-11
    pos = np.vstack([x["pos"] for x in fem])
    assert np.abs(pos - g["fem_pos"]).max() < 1e-11
    for k in range(len(fem)):
        assert np.abs(fem[k]["pos"] - femo[k]["pos"]).max() < 1e-11
    assert st.code == 0
    print(name, {f"{a}:{b}": f"{v:.2e}" for (a, b), v in report.items()}, "subits", st.last_subits)


def test_graph_loop_equals_host_driven_loop():
    """The FSI loop replayed as a CUDA graph (WHILE node set from the device)
    gives the same bits as the host-driven loop that reads the flag each
    subiteration."""
    import subprocess
    import sys
    code = ("import sys, numpy as np; sys.path.insert(0, 'tests/golden'); sys.path.insert(0, '.');"
            "from cases import golden_cases; from life_gb300.lib import Case;"
            "p, b = golden_cases()['honami_like_cm']; c = Case(p, b); c.step(60);"
            "f = c.fields(); m = c.markers();"
            "np.save(sys.argv[1], np.concatenate([f['f'].ravel(), m['pos'].ravel(), m['force'].ravel()]))")
    import os
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with tempfile.TemporaryDirectory() as td:
        a, h = os.path.join(td, "graph.npy"), os.path.join(td, "host.npy")
        subprocess.run([sys.executable, "-c", code, a], cwd=root, check=True)
        subprocess.run([sys.executable, "-c", code, h], cwd=root, check=True,
                       env=dict(os.environ, LIFE_FSI_HOSTLOOP="1"))
        assert np.array_equal(np.load(a), np.load(h))
