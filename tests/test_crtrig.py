"""The correctly rounded sin, cos and atan2 of the FEM element update
(life_gb300/csrc/crtrig.h), called on the host through the oracle built with
them (liblife_oracle_cr.so), against 300-bit arithmetic (mpmath): every result
must be the double nearest the exact value (error <= 0.5 units in the last
place), on the angles the FEM produces (all of [-pi, pi]), near multiples of
pi/2, on tiny and larger operands, and on atan2's special operands (C99 Annex
F.9.1.4, compared with the C library, which follows it exactly).

The device evaluates the same header; tests/test_gpu_trig.py checks that its
results equal these bit for bit.
"""
import math
import random

import pytest

mpmath = pytest.importorskip("mpmath")


@pytest.fixture(scope="module")
def L():
    from oracle.pyoracle import build, lib
    build()
    return lib("cr")


def ulp_error(got, exact):
    if got == 0.0:
        return float("inf") if exact != 0 else 0.0
    return float(abs((mpmath.mpf(got) - exact) / math.ulp(got)))


def sin_cos_args(n, seed):
    rng = random.Random(seed)
    xs = [rng.uniform(-math.pi, math.pi) for _ in range(n)]
    for k in range(-8, 9):
        x = k * math.pi / 2
        xs += [x, math.nextafter(x, math.inf), math.nextafter(x, -math.inf), x + 1e-9, x - 1e-13]
    xs += [1e-300, 5e-324, 1e-8, -1e-20, 3.0, 1e5, 123456.789, -524287.9, 0.5, -0.7853981633974483]
    return xs


def test_sin_cos_correctly_rounded(L):
    mpmath.mp.prec = 300
    worst = 0.0
    for x in sin_cos_args(20000, 1):
        for got, f in ((L.oracle_cr_sin(x), mpmath.sin), (L.oracle_cr_cos(x), mpmath.cos)):
            e = ulp_error(got, f(mpmath.mpf(x)))
            worst = max(worst, e)
            assert e <= 0.5, (x, got, e)
    assert L.oracle_cr_sin(0.0) == 0.0 and math.copysign(1.0, L.oracle_cr_sin(-0.0)) == -1.0
    assert L.oracle_cr_cos(0.0) == 1.0
    print(f"sin/cos worst error {worst:.6f} ulp")


def test_atan2_correctly_rounded(L):
    mpmath.mp.prec = 300
    rng = random.Random(2)
    pairs = [(rng.uniform(-2, 2), rng.uniform(-2, 2)) for _ in range(20000)]
    pairs += [(1e-3 * rng.uniform(-1, 1), rng.uniform(-2, 2)) for _ in range(2000)]
    pairs += [(rng.uniform(-2, 2), 1e-3 * rng.uniform(-1, 1)) for _ in range(2000)]
    pairs += [(1.0, 1.0), (-1.0, -1.0), (1e-200, 1.0), (1.0, 1e-200), (3.0, -1e-12), (0.5, -0.5)]
    worst = 0.0
    for y, x in pairs:
        got = L.oracle_cr_atan2(y, x)
        e = ulp_error(got, mpmath.atan2(mpmath.mpf(y), mpmath.mpf(x)))
        worst = max(worst, e)
        assert e <= 0.5, (y, x, got, e)
    print(f"atan2 worst error {worst:.6f} ulp")


def test_atan2_special_operands(L):
    inf, nan = math.inf, math.nan
    cases = [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (0.0, 0.0), (-0.0, 0.0), (0.0, -0.0),
             (-0.0, -0.0), (1.0, 0.0), (-1.0, -0.0), (inf, 1.0), (-inf, 1.0), (inf, inf), (inf, -inf),
             (-inf, -inf), (1.0, inf), (-1.0, inf), (1.0, -inf), (-1.0, -inf), (-0.0, -2.0)]
    for y, x in cases:
        a, b = L.oracle_cr_atan2(y, x), math.atan2(y, x)
        assert a == b and math.copysign(1.0, a) == math.copysign(1.0, b), (y, x, a, b)
    assert math.isnan(L.oracle_cr_atan2(nan, 1.0)) and math.isnan(L.oracle_cr_atan2(1.0, nan))
