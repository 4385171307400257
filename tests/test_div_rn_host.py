"""The FP64 quotient routine of the lattice kernels and the FEM band solve
(``life_gb300/csrc/div_rn.cuh``: one correctly rounded reciprocal y = RN(1/b)
per divisor, each quotient finished with two FMA residual corrections, the
hardware division outside a safe exponent window) must give the bits of IEEE
division for every pair of operands. The same function is compiled here for
the host (nvcc, host code only: no GPU is used) and compared with a / b on
millions of seeded operand pairs: normal operands near 1 and over the whole
exponent range, signed-zero numerators (the velocity of a site at rest),
subnormal, infinite and NaN operands (which take the hardware path), and
quotients that overflow or underflow. The device build is checked the same
way by ``life_selftest_division`` (``tests/test_gpu_division.py``).
"""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "life_gb300", "csrc")

DRIVER = r"""
#include "div_rn.cuh"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static uint64_t mix(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
static double from_bits(uint64_t u) {
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
}
static uint64_t bits(double d) {
    uint64_t u;
    std::memcpy(&u, &d, sizeof u);
    return u;
}
// an operand: mostly a normal number near 1, sometimes anywhere in the
// normal range, sometimes a special value
static double operand(uint64_t r, uint64_t w) {
    const int kind = (int)(w & 63);
    if (kind == 0) return (r & 1) ? -0.0 : 0.0;
    if (kind == 1) return from_bits((r & 0x800fffffffffffffull));                      // subnormal (or zero)
    if (kind == 2) return (r & 1) ? -__builtin_inf() : __builtin_inf();
    if (kind == 3) return from_bits(0x7ff8000000000000ull | (r & 0xfffffull));         // NaN
    const int span = (kind < 12) ? 2046 : 80;
    long long e = 1023 + (long long)((w >> 8) % (uint64_t)span) - span / 2;
    if (e < 1) e = 1;
    if (e > 2046) e = 2046;
    return from_bits((r & 0x800fffffffffffffull) | ((uint64_t)e << 52));
}

int main(int argc, char** argv) {
    const uint64_t seed = strtoull(argv[1], nullptr, 10);
    const long long n = atoll(argv[2]);
    long long bad = 0, checked = 0, fast = 0;
    for (long long q = 0; q < n; q++) {
        const uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(2 * q + 1);
        const double a = operand(mix(z), mix(z ^ 0x5851f42d4c957f2dull));
        const double b = operand(mix(z + 0x9e3779b97f4a7c15ull), mix(z ^ 0x2545f4914f6cdd1dull));
        const double y = 1.0 / b;
        const double ref = a / b;
        const double got = life::div_rn_recip(a, b, y);
        checked++;
        const int ea = (int)(bits(a) >> 52) & 0x7ff, eb = (int)(bits(b) >> 52) & 0x7ff;
        if (eb > 200 && eb < 1800 && ((bits(a) << 1) == 0 || (ea > 200 && ea < 1800))) fast++;
        if (bits(ref) != bits(got) && !(ref != ref && got != got)) {
            if (bad < 5) printf("mismatch a=%a b=%a ref=%a got=%a\n", a, b, ref, got);
            bad++;
        }
    }
    printf("%lld %lld %lld\n", checked, fast, bad);
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver():
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    d = tempfile.mkdtemp(prefix="div_rn_")
    src, exe = os.path.join(d, "div_rn_host.cu"), os.path.join(d, "div_rn_host")
    with open(src, "w") as fh:
        fh.write(DRIVER)
    cmd = [nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
           "-Xcompiler", "-ffp-contract=off", "-I", CSRC, src, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    yield exe
    shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("seed", [1, 20251204, 987654321])
def test_host_build_of_the_quotient_routine_equals_ieee_division(driver, seed):
    res = subprocess.run([driver, str(seed), "2000000"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    checked, fast, bad = map(int, res.stdout.split()[-3:])
    assert checked == 2000000
    assert fast > checked // 2  # most pairs take the reciprocal path, not the fallback
    assert bad == 0, res.stdout
