"""The device's correctly rounded trigonometry (crtrig.h) gives the host's
results bit for bit (the host side is checked against 300-bit arithmetic in
tests/test_crtrig.py): sin and cos on the FEM's angle range and beyond,
atan2 over all quadrants and its special operands."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_trig_equals_host_bit_for_bit():
    from life_gb300.build import build
    build()
    from life_gb300.lib import lib
    from oracle.pyoracle import build as build_oracle, lib as oracle_lib
    build_oracle()
    H = oracle_lib("cr")
    L = lib()
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-math.pi, math.pi, 200000), rng.uniform(-4e5, 4e5, 20000),
                        np.array([0.0, -0.0, 5e-324, 1e-300, math.pi / 2, -math.pi, 1e-8])])
    y = np.concatenate([rng.uniform(-2, 2, x.size - 10),
                        np.array([0.0, -0.0, 1.0, -1.0, math.inf, -math.inf, 1e-200, 3.0, -0.0, 0.0])])
    xa = np.concatenate([rng.uniform(-2, 2, x.size - 10),
                         np.array([1.0, -1.0, 0.0, -0.0, math.inf, -math.inf, 1.0, -1e-12, -2.0, -0.0])])
    dp = C.POINTER(C.c_double)
    for op, host in ((0, H.oracle_cr_sin), (1, H.oracle_cr_cos)):
        out = np.empty_like(x)
        assert L.life_selftest_trig(op, x.size, x.ctypes.data_as(dp), None, out.ctypes.data_as(dp)) == 0
        ref = np.array([host(float(v)) for v in x])
        assert np.array_equal(out.view(np.uint64), ref.view(np.uint64)), op
    out = np.empty_like(y)
    assert L.life_selftest_trig(2, y.size, xa.ctypes.data_as(dp), y.ctypes.data_as(dp), out.ctypes.data_as(dp)) == 0
    ref = np.array([H.oracle_cr_atan2(float(a), float(b)) for a, b in zip(y, xa)])
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))
