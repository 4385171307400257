"""The FEM band solve divides by a pivot whose correctly rounded reciprocal it
already holds, with Markstein's method (q = a*y and two fused-multiply-add
corrections). It must give exactly the IEEE quotient: the self-test compares
it with a / b on the device for seeded random operands (exponents mostly near
1, one pair in eight anywhere in the normal range, which also exercises the
guarded fallback)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20260101, 987654321])
def test_division_by_reciprocal_is_correctly_rounded(seed):
    from life_gb300.build import build
    build()
    from life_gb300.lib import _check, lib
    bad = C.c_int64(-1)
    _check(lib().life_selftest_division(1 << 26, seed, C.byref(bad)))
    assert bad.value == 0
