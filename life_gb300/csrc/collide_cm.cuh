// Central-moments collision in FP64 (De Rosis 2019), the reference's
// CENTRAL_MOMENTS branch of GridClass::streamCollide.
#pragma once
#include "lbm_device.cuh"

namespace life {

// Inverse central-moment transform (De Rosis 2019), term order as in the
// reference (src/Grid.cpp:109-223); FP64 parity depends on that order.
template <bool UNF>
__device__ __forceinline__ void collide_cm(const double f[9], double rho, double ux, double uy, double Fx, double Fy,
                           double omega, double cs, double fs[9]) {
    // the two sums start at their first term rather than at +0 (see
    // moment_sums: equal up to the sign of a zero, which pos_zero restores)
    double k4Pre, k5Pre;
#pragma unroll
    for (int v = 0; v < 9; v++) {
        double cx = cx_of(v) - ux;
        double cy = cy_of(v) - uy;
        const double t4 = f[v] * (LSQ(cx) - LSQ(cy)), t5 = f[v] * cx * cy;
        k4Pre = v == 0 ? t4 : k4Pre + t4;
        k5Pre = v == 0 ? t5 : k5Pre + t5;
    }
    k4Pre = pos_zero(k4Pre);
    k5Pre = pos_zero(k5Pre);
    const double k0 = rho;
    const double k1 = 0.5 * Fx;
    const double k2 = 0.5 * Fy;
    const double k3 = 2.0 * rho * LSQ(cs);
    const double k4 = (1.0 - omega) * k4Pre;
    const double k5 = (1.0 - omega) * k5Pre;
    const double k6 = 0.5 * Fy * LSQ(cs);
    const double k7 = 0.5 * Fx * LSQ(cs);
    const double k8 = rho * LQU(cs);
    const double X2 = LSQ(ux), Y2 = LSQ(uy);
    // The force moments k1, k2, k6, k7 are exact zeros when Fx = Fy = 0 (a
    // value the whole launch shares); their terms are then not formed, and
    // every other term is added in the reference's order.
    const bool forced = !UNF && (Fx != 0.0 || Fy != 0.0);
    {
        double a = (X2 * Y2 - X2 - Y2 + 1.0) * k0;
        if (forced) a = a + ((2.0 * ux * Y2 - 2.0 * ux) * k1);
        if (forced) a = a + ((2.0 * uy * X2 - 2.0 * uy) * k2);
        a = a + ((0.5 * X2 + 0.5 * Y2 - 1.0) * k3);
        a = a + ((0.5 * Y2 - 0.5 * X2) * k4);
        a = a + (4.0 * ux * uy * k5);
        if (forced) a = a + (2.0 * uy * k6);
        if (forced) a = a + (2.0 * ux * k7);
        a = a + (k8);
        fs[0] = a;
    }
    {
        double a = (0.5 * X2 - 0.5 * (X2 * Y2) - 0.5 * (ux * Y2) + 0.5 * ux) * k0;
        if (forced) a = a + ((ux - ux * Y2 - 0.5 * Y2 + 0.5) * k1);
        if (forced) a = a + ((-uy * X2 - uy * ux) * k2);
        a = a + ((-0.25 * X2 - 0.25 * ux - 0.25 * Y2 + 0.25) * k3);
        a = a + ((0.25 * X2 + 0.25 * ux - 0.25 * Y2 + 0.25) * k4);
        a = a + ((-uy - 2.0 * ux * uy) * k5);
        if (forced) a = a + ((-uy) * k6);
        if (forced) a = a + ((-ux - 0.5) * k7);
        a = a - (0.5 * k8);
        fs[1] = a;
    }
    {
        double a = (-0.5 * (X2 * Y2) + 0.5 * X2 + 0.5 * (ux * Y2) - 0.5 * ux) * k0;
        if (forced) a = a + ((ux - ux * Y2 + 0.5 * Y2 - 0.5) * k1);
        if (forced) a = a + ((-uy * X2 + uy * ux) * k2);
        a = a + ((-0.25 * X2 + 0.25 * ux - 0.25 * Y2 + 0.25) * k3);
        a = a + ((0.25 * X2 - 0.25 * ux - 0.25 * Y2 + 0.25) * k4);
        a = a + ((uy - 2.0 * ux * uy) * k5);
        if (forced) a = a + ((-uy) * k6);
        if (forced) a = a + ((0.5 - ux) * k7);
        a = a - (0.5 * k8);
        fs[2] = a;
    }
    {
        double a = (0.5 * Y2 - 0.5 * (X2 * uy) - 0.5 * (X2 * Y2) + 0.5 * uy) * k0;
        if (forced) a = a + ((-ux * Y2 - ux * uy) * k1);
        if (forced) a = a + ((uy - X2 * uy - 0.5 * X2 + 0.5) * k2);
        a = a + ((-0.25 * X2 - 0.25 * Y2 - 0.25 * uy + 0.25) * k3);
        a = a + ((0.25 * X2 - 0.25 * Y2 - 0.25 * uy - 0.25) * k4);
        a = a + ((-ux - 2.0 * ux * uy) * k5);
        if (forced) a = a + ((-uy - 0.5) * k6);
        if (forced) a = a + ((-ux) * k7);
        a = a - (0.5 * k8);
        fs[3] = a;
    }
    {
        double a = (-0.5 * (X2 * Y2) + 0.5 * (X2 * uy) + 0.5 * Y2 - 0.5 * uy) * k0;
        if (forced) a = a + ((-ux * Y2 + ux * uy) * k1);
        if (forced) a = a + ((uy - X2 * uy + 0.5 * X2 - 0.5) * k2);
        a = a + ((-0.25 * X2 - 0.25 * Y2 + 0.25 * uy + 0.25) * k3);
        a = a + ((0.25 * X2 - 0.25 * Y2 + 0.25 * uy - 0.25) * k4);
        a = a + ((ux - 2.0 * ux * uy) * k5);
        if (forced) a = a + ((0.5 - uy) * k6);
        if (forced) a = a + ((-ux) * k7);
        a = a - (0.5 * k8);
        fs[4] = a;
    }
    {
        double a = (0.25 * (X2 * Y2) + 0.25 * (X2 * uy) + 0.25 * (ux * Y2) + 0.25 * (ux * uy)) * k0;
        if (forced) a = a + ((0.25 * uy + 0.5 * (ux * uy) + 0.5 * (ux * Y2) + 0.25 * Y2) * k1);
        if (forced) a = a + ((0.25 * ux + 0.5 * (ux * uy) + 0.5 * (X2 * uy) + 0.25 * X2) * k2);
        a = a + ((0.125 * X2 + 0.125 * ux + 0.125 * Y2 + 0.125 * uy) * k3);
        a = a + ((-0.125 * X2 - 0.125 * ux + 0.125 * Y2 + 0.125 * uy) * k4);
        a = a + ((0.5 * ux + 0.5 * uy + ux * uy + 0.25) * k5);
        if (forced) a = a + ((0.5 * uy + 0.25) * k6);
        if (forced) a = a + ((0.5 * ux + 0.25) * k7);
        a = a + (0.25 * k8);
        fs[5] = a;
    }
    {
        double a = (0.25 * (X2 * Y2) - 0.25 * (X2 * uy) - 0.25 * (ux * Y2) + 0.25 * (ux * uy)) * k0;
        if (forced) a = a + ((0.25 * uy - 0.5 * (ux * uy) + 0.5 * (ux * Y2) - 0.25 * Y2) * k1);
        if (forced) a = a + ((0.25 * ux - 0.5 * (ux * uy) + 0.5 * (X2 * uy) - 0.25 * X2) * k2);
        a = a + ((0.125 * X2 - 0.125 * ux + 0.125 * Y2 - 0.125 * uy) * k3);
        a = a + ((-0.125 * X2 + 0.125 * ux + 0.125 * Y2 - 0.125 * uy) * k4);
        a = a + ((ux * uy - 0.5 * uy - 0.5 * ux + 0.25) * k5);
        if (forced) a = a + ((0.5 * uy - 0.25) * k6);
        if (forced) a = a + ((0.5 * ux - 0.25) * k7);
        a = a + (0.25 * k8);
        fs[6] = a;
    }
    {
        double a = (0.25 * (X2 * Y2) - 0.25 * (X2 * uy) + 0.25 * (ux * Y2) - 0.25 * (ux * uy)) * k0;
        if (forced) a = a + ((0.5 * (ux * Y2) - 0.5 * (ux * uy) - 0.25 * uy + 0.25 * Y2) * k1);
        if (forced) a = a + ((0.5 * (ux * uy) - 0.25 * ux + 0.5 * (X2 * uy) - 0.25 * X2) * k2);
        a = a + ((0.125 * X2 + 0.125 * ux + 0.125 * Y2 - 0.125 * uy) * k3);
        a = a + ((-0.125 * X2 - 0.125 * ux + 0.125 * Y2 - 0.125 * uy) * k4);
        a = a + ((0.5 * uy - 0.5 * ux + ux * uy - 0.25) * k5);
        if (forced) a = a + ((0.5 * uy - 0.25) * k6);
        if (forced) a = a + ((0.5 * ux + 0.25) * k7);
        a = a + (0.25 * k8);
        fs[7] = a;
    }
    {
        double a = (0.25 * (X2 * Y2) + 0.25 * (X2 * uy) - 0.25 * (ux * Y2) - 0.25 * (ux * uy)) * k0;
        if (forced) a = a + ((0.5 * (ux * uy) - 0.25 * uy + 0.5 * (ux * Y2) - 0.25 * Y2) * k1);
        if (forced) a = a + ((0.5 * (X2 * uy) - 0.5 * (ux * uy) - 0.25 * ux + 0.25 * X2) * k2);
        a = a + ((0.125 * X2 - 0.125 * ux + 0.125 * Y2 + 0.125 * uy) * k3);
        a = a + ((-0.125 * X2 + 0.125 * ux + 0.125 * Y2 + 0.125 * uy) * k4);
        a = a + ((0.5 * ux - 0.5 * uy + ux * uy - 0.25) * k5);
        if (forced) a = a + ((0.5 * uy + 0.25) * k6);
        if (forced) a = a + ((0.5 * ux - 0.25) * k7);
        a = a + (0.25 * k8);
        fs[8] = a;
    }
}

}  // namespace life
