"""life_ibm_epsilon_noalloc: the epsilon solve for callers that cannot call
cudaMalloc (their device memory comes from another allocator's pool, or the
implicit synchronisation of cudaMalloc/cudaFree is not allowed where they
run). Its scratch is a static device array inside the library, shared by all
calls. Two calls in a row on different marker sets must each give exactly the
result of the allocating entry point life_ibm_epsilon; a marker set above the
static maximum (256) must be refused before any work is launched.

This file is collected last so a run that stops at the first failure has run
every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu


def _inputs(name):
    import torch
    from life_gb300.lib import Case
    p, b = golden_cases()[name]
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
    for name in ("cylinder_rigid_cm", "filament_supported_and_rigid"):
        dev, n, Dx = _inputs(name)
        assert 0 < n <= 256
        rc, ref = _run(L.life_ibm_epsilon, dev, n, Dx)
        assert rc == 0, L.life_last_error()
        rc, got = _run(L.life_ibm_epsilon_noalloc, dev, n, Dx)
        assert rc == 0, L.life_last_error()
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, ref), (name, np.abs(got - ref).max())


def test_noalloc_epsilon_rejects_oversized_marker_set():
    from life_gb300.build import build
    build()
    from life_gb300.lib import lib
    L = lib()
    rc = L.life_ibm_epsilon_noalloc(None, None, None, None, None, None, 257, 1.0, None, None)
    assert rc != 0
    assert b"257" in L.life_last_error() and b"256" in L.life_last_error()
