"""The FP64 density and momentum sums of the lattice kernels
(``moment_sums`` in ``life_gb300/csrc/lbm_device.cuh``) skip the terms whose
lattice-velocity component is 0, add +-f for a component of +-1, start each
sum at its first term instead of at +0, and clear a negative-zero result on
the bits. Each of these is claimed to give the bits of the reference's
literal sums (GridClass::macroscopic, src/Grid.cpp:285-293: rho += f_v,
rhoU += c_v f_v from +0, over v = 0..8). The same function is compiled here
for the host (nvcc, host code only: no GPU is used) and compared with the
literal sums on every population whose entries come from {+0, -0, x} (all
signed-zero patterns; a sum started at its first term ends at -0 only when
all of its terms are -0) and on millions of seeded populations built to
stress the other edge cases: exact cancellations (equal and opposite
populations), tiny and huge magnitudes, and ordinary values.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "life_gb300", "csrc")

DRIVER = r"""
#include "lbm_device.cuh"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static uint64_t mix(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
static uint64_t bits(double d) {
    uint64_t u;
    std::memcpy(&u, &d, sizeof u);
    return u;
}
// one population: a small pool of values (so that equal and opposite values,
// hence exact cancellations, are frequent), signed zeros, or a random double
static double pop(uint64_t r) {
    static const double pool[] = {0.0, -0.0, 0.25, -0.25, 1.0 / 9.0, -1.0 / 9.0, 1e-300, -1e-300,
                                  4.9e-324, -4.9e-324, 1e300, -1e300, 0.4444444444444444, 3.0};
    const int kind = (int)(r & 7);
    if (kind < 5) return pool[(r >> 3) % (sizeof pool / sizeof pool[0])];
    double d;
    uint64_t u = mix(r);
    u = (u & 0x800fffffffffffffull) | ((uint64_t)(1023 - 40 + (int)((r >> 8) % 60)) << 52);
    std::memcpy(&d, &u, sizeof d);
    return d;
}

static long long bad = 0;
static void check(const double f[9]) {
    // the reference's literal sums from +0
    double r0 = 0.0, mx0 = 0.0, my0 = 0.0;
    for (int v = 0; v < 9; v++) {
        r0 += f[v];
        mx0 += (double)life::cx_of(v) * f[v];
        my0 += (double)life::cy_of(v) * f[v];
    }
    double r, mx, my;
    life::moment_sums(f, r, mx, my);
    const bool same = (bits(r) == bits(r0) || (r != r && r0 != r0)) &&
                      (bits(mx) == bits(mx0) || (mx != mx && mx0 != mx0)) &&
                      (bits(my) == bits(my0) || (my != my && my0 != my0));
    if (!same) {
        if (bad < 5) printf("mismatch r %a/%a mx %a/%a my %a/%a\n", r, r0, mx, mx0, my, my0);
        bad++;
    }
}

int main(int argc, char** argv) {
    const uint64_t seed = strtoull(argv[1], nullptr, 10);
    const long long n = atoll(argv[2]);
    long long negzero_seen = 0;
    // every population with entries from {+0, -0, x}: all signed-zero patterns
    // (a sum started at its first term ends at -0 only when all its terms are)
    long long exhaustive = 0;
    for (double x : {0.25, -0.25, 1e-300}) {
        const double vals[3] = {0.0, -0.0, x};
        for (int code = 0; code < 19683; code++) {
            double f[9];
            int c = code;
            for (int v = 0; v < 9; v++, c /= 3) f[v] = vals[c % 3];
            check(f);
            exhaustive++;
        }
    }
    for (long long q = 0; q < n; q++) {
        double f[9];
        for (int v = 0; v < 9; v++) f[v] = pop(mix(seed * 0x9e3779b97f4a7c15ull + (uint64_t)q * 9 + v));
        if (bits(f[0]) == 0x8000000000000000ull || bits(f[1]) == 0x8000000000000000ull) negzero_seen++;
        check(f);
    }
    printf("%lld %lld %lld %lld\n", exhaustive, n, negzero_seen, bad);
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver():
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    d = tempfile.mkdtemp(prefix="moment_sums_")
    src, exe = os.path.join(d, "moment_sums_host.cu"), os.path.join(d, "moment_sums_host")
    with open(src, "w") as fh:
        fh.write(DRIVER)
    inc = os.path.join(os.path.dirname(CSRC), "..", "include")
    cmd = [nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
           "-Xcompiler", "-ffp-contract=off", "-I", CSRC, "-I", inc, src, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    yield exe
    shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("seed", [3, 777, 20251204])
def test_host_build_of_moment_sums_equals_the_reference_sums(driver, seed):
    res = subprocess.run([driver, str(seed), "2000000"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    exhaustive, n, negzero, bad = map(int, res.stdout.split()[-4:])
    assert exhaustive == 3 * 3 ** 9 and n == 2000000
    assert negzero > 10000  # signed-zero leading terms among the random populations too
    assert bad == 0, res.stdout
