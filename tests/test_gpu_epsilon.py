"""life_ibm_epsilon on caller-owned device buffers reproduces the epsilon
weights a case computed for its markers (same textbook-order LU, bit for bit)."""
import ctypes as C

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu


def device_inputs(case):
    import torch
    mk, sp = case.markers(), case.support()
    dev = {
        "pos": torch.tensor(mk["pos"], dtype=torch.float64, device="cuda"),
        "nsupp": torch.tensor(sp["nsupp"], dtype=torch.int32, device="cuda"),
        "si": torch.tensor(sp["si"], dtype=torch.int32, device="cuda"),
        "sj": torch.tensor(sp["sj"], dtype=torch.int32, device="cuda"),
        "sd": torch.tensor(sp["sd"], dtype=torch.float64, device="cuda"),
        "ds": torch.tensor(mk["ds"], dtype=torch.float64, device="cuda"),
        "eps": torch.zeros(len(mk["ds"]), dtype=torch.float64, device="cuda"),
    }
    return mk, dev


def call_epsilon(fn, dev, n, Dx):
    import torch
    torch.cuda.synchronize()
    rc = fn(C.c_void_p(dev["pos"].data_ptr()), C.c_void_p(dev["nsupp"].data_ptr()),
            C.c_void_p(dev["si"].data_ptr()), C.c_void_p(dev["sj"].data_ptr()),
            C.c_void_p(dev["sd"].data_ptr()), C.c_void_p(dev["ds"].data_ptr()), n, Dx,
            C.c_void_p(dev["eps"].data_ptr()), None)
    return rc


@pytest.mark.parametrize("name", ["cylinder_rigid_cm", "filament_flex_deflect"])
def test_epsilon_entry_point_matches_case(name):
    from life_gb300.build import build
    build()
    from life_gb300.lib import Case, lib
    p, b = golden_cases()[name]
    with Case(p, b) as c:
        mk, dev = device_inputs(c)
        rc = call_epsilon(lib().life_ibm_epsilon, dev, c.n_markers, c.info().Dx)
        assert rc == 0, lib().life_last_error()
        got = dev["eps"].cpu().numpy()
    assert np.array_equal(got, mk["epsilon"])
