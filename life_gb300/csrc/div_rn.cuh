// Correctly rounded FP64 division through a reciprocal, shared by the lattice
// kernels (the velocity of every site) and the FEM band solve.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

namespace life {

// the bits of a double (device intrinsic, or a copy on the host)
__host__ __device__ __forceinline__ unsigned long long div_bits(double x) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long u;
    std::memcpy(&u, &x, sizeof u);
    return u;
#endif
}

// a / b correctly rounded (round to nearest), given y = RN(1/b): Markstein's
// method (P. Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et al.,
// Handbook of Floating-Point Arithmetic, "Markstein's theorem"): q0 = RN(a y)
// is within 1.5 ulp of a/b, one correction q1 = RN(q0 + RN(a - b q0) y)
// brings it within one ulp, and then the residual a - b q1 is exact and
// RN(q1 + (a - b q1) y) = RN(a/b). The theorem needs the intermediates in the
// normal range, so operands outside a safe exponent window (tested on the
// bits, with integer operations) take the hardware division.
// life_selftest_division checks this function against a / b on the device,
// and the host build of the same function is checked against IEEE division
// by the CPU tests.
__host__ __device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
    const unsigned long long ba = div_bits(a);
    const unsigned long long bb = div_bits(b);
    const int ea = (int)(ba >> 52) & 0x7ff, eb = (int)(bb >> 52) & 0x7ff;
    // a zero numerator runs the same steps (every intermediate is a zero) and
    // then takes q0 = a * y, the signed zero a / b (y has the sign of b): the
    // cost of a site does not depend on its velocity being zero
    const bool a_zero = (ba << 1) == 0ull;
    const bool a_ok = a_zero || (ea > 200 && ea < 1800 && ea - eb > -700 && ea - eb < 700);
    const bool b_ok = eb > 200 && eb < 1800;
    if (!(a_ok && b_ok)) return a / b;
    const double q0 = a * y;
    const double r0 = fma(-b, q0, a);
    const double q1 = fma(r0, y, q0);
    const double r1 = fma(-b, q1, a);
    const double q = fma(r1, y, q1);
    return a_zero ? q0 : q;
}

}  // namespace life
