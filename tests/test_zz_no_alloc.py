"""life_ibm_epsilon_noalloc: the epsilon solve for callers that cannot call
cudaMalloc (their device memory comes from another allocator's pool, or the
implicit synchronisation of cudaMalloc/cudaFree is not allowed where they
run). Its scratch is a static device array inside the library, shared by all
calls. Calls in a row on different marker sets must each give exactly the
result of the allocating entry point life_ibm_epsilon; a marker set above the
static maximum (256) must be refused before any work is launched.

The marker sets are closed rings (cylinders). A ring's first and last markers
are neighbours, so its epsilon system is as wide as the ring and is solved as
a dense system in the static array, not in shared memory; the 256-marker ring
fills the array to its limit.

This file is collected last so a run that stops at the first failure has run
every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu


def _ring_case(radius, n_lat):
    from life_gb300.case import CONVECTIVE, VELOCITY, Circle
    from cases import lattice_case
    c = n_lat / 2.0
    p = lattice_case(n_lat, n_lat + 1, 1.0 / 0.56, 1, wall_left=VELOCITY, wall_right=CONVECTIVE,
                     uxInlet_p=0.04, ref_L=2 * radius)
    return p, [Circle(x=c, y=c + 0.3, radius=radius, ID=0)]


def _inputs(p, b):
    import torch
    from life_gb300.lib import Case
    with Case(p, b) as c:
        mk, sp = c.markers(), c.support()
        Dx = c.info().Dx
    t = lambda a, dt: torch.tensor(a, dtype=dt, device="cuda")  # noqa: E731
    dev = dict(pos=t(mk["pos"], torch.float64), nsupp=t(sp["nsupp"], torch.int32), si=t(sp["si"], torch.int32),
               sj=t(sp["sj"], torch.int32), sd=t(sp["sd"], torch.float64), ds=t(mk["ds"], torch.float64))
    return dev, len(mk["ds"]), Dx


def _run(fn, dev, n, Dx):
    import torch
    out = torch.full((max(n, 1),), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = fn(*[C.c_void_p(dev[k].data_ptr()) for k in ("pos", "nsupp", "si", "sj", "sd", "ds")], n, Dx,
            C.c_void_p(out.data_ptr()), None)
    return rc, out[:n].cpu().numpy()


def test_noalloc_epsilon_matches_allocating_entry_point_two_calls():
    from life_gb300.build import build
    build()
    from life_gb300.lib import lib
    L = lib()
    # 256 markers (the static maximum: floor(2 pi 40.8) = 256), then 125, then
    # 37: each call reuses the array the previous, larger call left behind.
    rings = [_ring_case(40.8, 120), _ring_case(20.0, 64), golden_cases()["cylinder_rigid_cm"]]
    sizes = []
    for p, b in rings:
        dev, n, Dx = _inputs(p, b)
        sizes.append(n)
        rc, ref = _run(L.life_ibm_epsilon, dev, n, Dx)
        assert rc == 0, L.life_last_error()
        rc, got = _run(L.life_ibm_epsilon_noalloc, dev, n, Dx)
        assert rc == 0, L.life_last_error()
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, ref), (n, np.abs(got - ref).max())
    assert sizes == [256, 125, 37], sizes


def test_noalloc_epsilon_rejects_oversized_marker_set():
    from life_gb300.build import build
    build()
    from life_gb300.lib import lib
    L = lib()
    rc = L.life_ibm_epsilon_noalloc(None, None, None, None, None, None, 257, 1.0, None, None)
    assert rc != 0
    assert b"257" in L.life_last_error() and b"256" in L.life_last_error()
