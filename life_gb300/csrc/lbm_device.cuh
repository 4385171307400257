// Device-side lattice primitives shared by the lattice, IBM and export
// kernels: D2Q9 constants, site classification, the pull gather, macroscopic
// moments, the regularised / convective boundary conditions and the BGK and
// central-moment collisions in FP64.
//
// State convention. The device keeps P_t: the post-collision populations of
// step t, before streaming, in structure-of-arrays layout
//   P[v*S + j*pitch + i]   (x fastest; S = pitch*Ny).
// The reference's state after step t (post-stream f, rho, u; reference
// GridClass::lbmKernel, src/Grid.cpp:36-100) is a pure function of P_t plus a
// few per-step scalars, and site_state() computes it for any site. Every
// kernel that needs rho/u/f at a site (the fused step kernel, boundary sites,
// IBM interpolation, field export) calls the same function, so all of them see
// bit-identical values.
//
// FP64 translation units are compiled with --fmad=false and keep the
// reference's operation order, so a + b*c is rounded twice as g++ does on x86.
#pragma once
#include <cuda_fp16.h>
#include "div_rn.cuh"

#include <cstdint>

#include "life_types.h"

namespace life {

__host__ __device__ constexpr int cx_of(int v) { return v == 1 || v == 5 || v == 7 ? 1 : (v == 2 || v == 6 || v == 8 ? -1 : 0); }
__host__ __device__ constexpr int cy_of(int v) { return v == 3 || v == 5 || v == 8 ? 1 : (v == 4 || v == 6 || v == 7 ? -1 : 0); }
__host__ __device__ constexpr int opp_of(int v) { return v == 0 ? 0 : (v % 2 == 1 ? v + 1 : v - 1); }

// Lattice weights exactly as GridClass::GridClass builds them (4/9, 1/9, 1/36).
__device__ __forceinline__ double wgt(int v) {
    return v == 0 ? 4.0 / 9.0 : (v < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
}

#define LSQ(x) ((x) * (x))
#define LQU(x) ((x) * (x) * (x) * (x))

// Storage forms of the populations. load() returns f_v in FP64, save()
// stores an FP64 f_v back.
//   F64: f_v itself (the plain form).
//   F32: the shifted deviation g_v = f_v - w_v (rest density 1), so the
//        stored bits resolve the small departure from rest, not w_v.
//   F16: g_v / s_v with a per-direction power-of-two scale s_v close to w_v
//        (1/2, 1/8, 1/32), so scaling adds no rounding of its own.
__device__ __forceinline__ float h16_scale(int v) { return v == 0 ? 0.5f : (v < 5 ? 0.125f : 0.03125f); }
__device__ __forceinline__ float h16_inv(int v) { return v == 0 ? 2.0f : (v < 5 ? 8.0f : 32.0f); }
__device__ __forceinline__ float wgt_f(int v) { return v == 0 ? 4.0f / 9.0f : (v < 5 ? 1.0f / 9.0f : 1.0f / 36.0f); }

// float -> double, the exact value. On GB300 the hardware conversion issues
// to the narrow FP64 pipe; for normal floats the double's fields are the
// float's, rebiased, so integer operations give the same bits. Zeros,
// subnormals, infinities and NaNs take the hardware conversion.
__device__ __forceinline__ double f2d(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    return __longlong_as_double((long long)(((unsigned long long)(b >> 31) << 63) |
                                            ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                            ((unsigned long long)(b & 0x7fffffu) << 29)));
}

struct StoreF64 {
    using T = double;
    static constexpr int prec = LIFE_PREC_F64;
    __device__ static __forceinline__ double load(T x, int) { return x; }
    __device__ static __forceinline__ T save(double f, int) { return f; }
};
struct StoreF32 {
    using T = float;
    static constexpr int prec = LIFE_PREC_F32;
    __device__ static __forceinline__ double load(T x, int v) { return f2d(x) + wgt(v); }
    __device__ static __forceinline__ T save(double f, int v) { return (float)(f - wgt(v)); }
    __device__ static __forceinline__ float dev(T x, int) { return x; }      // g_v
    __device__ static __forceinline__ T put(float g, int) { return g; }
    // the stored value as a float and its deviation (here the same)
    static constexpr bool SCALED = false;
    __device__ static __forceinline__ float raw(T x) { return x; }
    __device__ static __forceinline__ float scaled(float r, int) { return r; }
    __device__ static __forceinline__ T put_raw(float r) { return r; }
};
struct StoreF16 {
    using T = __half;
    static constexpr int prec = LIFE_PREC_F16;
    __device__ static __forceinline__ double load(T x, int v) {
        return f2d(__half2float(x) * h16_scale(v)) + wgt(v);
    }
    __device__ static __forceinline__ T save(double f, int v) {
        return __float2half_rn((float)(f - wgt(v)) * h16_inv(v));
    }
    __device__ static __forceinline__ float dev(T x, int v) { return __half2float(x) * h16_scale(v); }
    __device__ static __forceinline__ T put(float g, int v) { return __float2half_rn(g * h16_inv(v)); }
    // the stored value as a float (the deviation divided by the direction's
    // power-of-two scale) and its deviation
    static constexpr bool SCALED = true;
    __device__ static __forceinline__ float raw(T x) { return __half2float(x); }
    __device__ static __forceinline__ float scaled(float r, int v) { return r * h16_scale(v); }
    __device__ static __forceinline__ T put_raw(float r) { return __float2half_rn(r); }
};

// Site type from the wall configuration; y walls override x walls at the
// corners (reference src/Grid.cpp:925-951).
__device__ __forceinline__ int site_type(const LatDev& L, int i, int j) {
    int t = LIFE_FLUID;
    if (i == 0) t = L.wall[0];
    else if (i == L.Nx - 1) t = L.wall[1];
    if (j == 0) t = L.wall[2];
    else if (j == L.Ny - 1) t = L.wall[3];
    return t;
}

// Outward-facing normal into the fluid and its direction
// (GridClass::getNormalVector, src/Grid.cpp:498-545). Corners next to a
// periodic wall become edges. A corner surrounded by periodic sites is
// rejected when the case is created.
__device__ __forceinline__ void site_normal(const LatDev& L, int i, int j, int& nx, int& ny, int& nd) {
    nx = 0; ny = 0; nd = 0;
    if (i == 0) { nx = 1; nd = 0; }
    else if (i == L.Nx - 1) { nx = -1; nd = 0; }
    if (j == 0) { ny = 1; nd = 1; }
    else if (j == L.Ny - 1) { ny = -1; nd = 1; }
    if (nx != 0 && ny != 0) {
        int tx = site_type(L, i + nx, j), ty = site_type(L, i, j + ny);
        if (tx == LIFE_FLUID && ty != LIFE_FLUID) { nd = 0; ny = 0; }
        else if (ty == LIFE_FLUID && tx != LIFE_FLUID) { nd = 1; nx = 0; }
    }
}

// Pull gather: the post-stream population v at (i,j) is the post-collision
// population v of the upwind site (i-cx, j-cy), with periodic wrap
// (the push index of src/Grid.cpp:229,240 read backwards).
template <class S>
__device__ __forceinline__ void gather(const typename S::T* __restrict__ P, const LatDev& L, int i, int j,
                                       double f[9]) {
#pragma unroll
    for (int v = 0; v < 9; v++) {
        int si = i - cx_of(v), sj = j - cy_of(v);
        si = si < 0 ? si + L.Nx : (si >= L.Nx ? si - L.Nx : si);
        sj = sj < 0 ? sj + L.Ny : (sj >= L.Ny ? sj - L.Ny : sj);
        f[v] = S::load(P[(size_t)v * L.S + (size_t)sj * L.pitch + si], v);
    }
}

// Terms of the reference's sums that multiply a population or velocity by a
// lattice-velocity component of 0 are exact zeros: adding one leaves a sum
// unchanged (the sums start at +0 and never hold -0), so the FP64 code below
// does not form them. A component of +-1 multiplies exactly. The remaining
// terms keep the reference's order. (After unrolling, the component tests are
// compile-time constants.)
__host__ __device__ __forceinline__ double add_c(double acc, int c, double x) {
    return c == 0 ? acc : (c > 0 ? acc + x : acc - x);
}

// 1/rho of the reduced-precision forms: the hardware approximation
// (rcp.approx.ftz.f32) refined by one Newton-Raphson step, y + y (1 - rho y)
// in two fused multiply-adds (the textbook iteration for a reciprocal). For
// the densities of a flow (rho near 1) the result is within one unit in the
// last place of 1/rho, and every kernel that forms a site's velocity in
// FP32 uses this function, so they agree bit for bit.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_lowp(float rho) {
    const float y = rcp_approx(rho);
    return fmaf(y, fmaf(-rho, y, 1.0f), y);
}

// -0 -> +0, tested on the bits (integer operations, not the FP64 unit)
__host__ __device__ __forceinline__ double pos_zero(double s) {
    return div_bits(s) == 0x8000000000000000ull ? 0.0 : s;
}

// The reference's density and momentum sums (src/Grid.cpp:285-293) start at
// +0. Here each starts at its first term instead (+-f, one FP64 add fewer
// per sum). The two running sums then differ at most in the sign of a zero:
// a round-to-nearest sum is -0 only when both of its terms are, so the
// reference's sums are never -0, and where this sum holds -0 the
// reference's holds +0, while any nonzero term makes them equal again.
// pos_zero() on the result gives the reference's bits. (Also built for the
// host, where the CPU tests compare it with the reference's literal sums.)
__host__ __device__ __forceinline__ void moment_sums(const double f[9], double& r, double& mx, double& my) {
    r = f[0];
    mx = 0.0;
    my = 0.0;
    bool hx = false, hy = false;
#pragma unroll
    for (int v = 1; v < 9; v++) {
        r = r + f[v];
        const int cx = cx_of(v), cy = cy_of(v);
        if (cx != 0) {
            mx = hx ? add_c(mx, cx, f[v]) : (cx > 0 ? f[v] : -f[v]);
            hx = true;
        }
        if (cy != 0) {
            my = hy ? add_c(my, cy, f[v]) : (cy > 0 ? f[v] : -f[v]);
            hy = true;
        }
    }
    r = pos_zero(r);
    mx = pos_zero(mx);
    my = pos_zero(my);
}

// GridClass::macroscopic (src/Grid.cpp:282-299)
__device__ __forceinline__ void macroscopic(const double f[9], double Fx, double Fy, double& rho,
                                            double& ux, double& uy) {
    double r, mx, my;
    moment_sums(f, r, mx, my);
    rho = r;
    // (m + F/2) / rho, both quotients through one correctly rounded reciprocal
    const double y = __drcp_rn(r);
    ux = div_rn_recip(mx + 0.5 * Fx, r, y);
    uy = div_rn_recip(my + 0.5 * Fy, r, y);
}

// macroscopic() for a zero force: m + 0.5 * (+-0) is m itself, since the
// momentum sums start at +0 and a round-to-nearest sum is -0 only when both
// of its terms are, so they are never -0.
__device__ __forceinline__ void macroscopic_unforced(const double f[9], double& rho, double& ux, double& uy) {
    double r, mx, my;
    moment_sums(f, r, mx, my);
    rho = r;
    const double y = __drcp_rn(r);
    ux = div_rn_recip(mx, r, y);
    uy = div_rn_recip(my, r, y);
}

// IBMNodeClass::updateMacroscopic form (src/IBMNode.cpp:113-122): the IBM
// force enters the velocity at support sites.
__device__ __forceinline__ void macroscopic_ibm(const double f[9], double Fx, double Fy, double Ix,
                                                double Iy, double& rho, double& ux, double& uy) {
    double r, mx, my;
    moment_sums(f, r, mx, my);
    rho = r;
    const double y = __drcp_rn(r);
    ux = div_rn_recip(mx + 0.5 * (Fx + Ix), r, y);
    uy = div_rn_recip(my + 0.5 * (Fy + Iy), r, y);
}

// GridClass::equilibrium (src/Grid.cpp:249-264): 2nd-order Hermite (BGK) or
// the 4th-order product form used with central moments.
// c . u without its zero-component products (c of a D2Q9 direction)
__device__ __forceinline__ double cdot_d(int cx, int cy, double ux, double uy) {
    if (cx == 0) return cy == 0 ? 0.0 : cy * uy;
    return cy == 0 ? cx * ux : cx * ux + cy * uy;
}

template <bool CM>
__device__ __forceinline__ double equilibrium(int v, double rho, double ux, double uy) {
    const int cx = cx_of(v), cy = cy_of(v);
    if (CM) {
        // (9 c^2 u^2 + 6 c u - 3 u^2 + 2) per axis; for c = 0 the first two
        // terms are exact zeros
        const double ax = cx == 0 ? -3.0 * LSQ(ux) + 2.0 : 9.0 * LSQ(cx) * LSQ(ux) + 6.0 * cx * ux - 3.0 * LSQ(ux) + 2.0;
        const double ay = cy == 0 ? -3.0 * LSQ(uy) + 2.0 : 9.0 * LSQ(cy) * LSQ(uy) + 6.0 * cy * uy - 3.0 * LSQ(uy) + 2.0;
        return 0.25 * rho * wgt(v) * ax * ay;
    }
    double s = 1.0 + 3.0 * cdot_d(cx, cy, ux, uy);
    s = s + 4.5 * (LSQ(ux) * (LSQ(cx) - 1.0 / 3.0) + LSQ(uy) * (LSQ(cy) - 1.0 / 3.0));
    if (cx != 0 && cy != 0) s = s + 9.0 * cx * cy * ux * uy;
    return rho * wgt(v) * s;
}

// GridClass::latticeForce (src/Grid.cpp:267-279), Guo forcing for BGK.
__device__ __forceinline__ double lattice_force(int v, double ux, double uy, double Fx, double Fy) {
    const int cx = cx_of(v), cy = cy_of(v);
    const double cu = cdot_d(cx, cy, ux, uy);
    const double tx = cx == 0 ? -ux : (cx - ux) + cx * 3.0 * cu;
    const double ty = cy == 0 ? -uy : (cy - uy) + cy * 3.0 * cu;
    return 3.0 * wgt(v) * (Fx * tx + Fy * ty);
}

// BGK collision (src/Grid.cpp:236-244).
// With no force at all (Fx = Fy = 0, a value the whole launch shares) the
// forcing term is an exact zero added to a nonzero sum, so it is not formed;
// UNF = true states that at compile time (no comparison at run time).
// The equilibria are those of equilibrium<false>, value for value, with the
// products that opposite directions share formed once: for c_w = -c_v,
// c_w.u = -(c_v.u) and 3 (c_w.u) = -(3 c_v.u) exactly (negation commutes
// with round-to-nearest), and 1 + 3 c.u adds the same operands either way (a
// zero of either sign gives 1); the diagonal term 9 cx cy ux uy is
// (9 ux) uy or its negative.
template <bool UNF = false>
__device__ __forceinline__ void collide_bgk(const double f[9], double rho, double ux, double uy, double Fx,
                                            double Fy, double omega, double fs[9]) {
    const bool forced = !UNF && (Fx != 0.0 || Fy != 0.0);
    const double px = 3.0 * ux, py = 3.0 * uy;
    const double pa = 3.0 * (ux + uy), pb = 3.0 * (ux - uy);
    const double d9 = 9.0 * ux * uy;
    const double X2 = LSQ(ux), Y2 = LSQ(uy);
    const double h00 = 4.5 * (X2 * (0.0 - 1.0 / 3.0) + Y2 * (0.0 - 1.0 / 3.0));
    const double h10 = 4.5 * (X2 * (1.0 - 1.0 / 3.0) + Y2 * (0.0 - 1.0 / 3.0));
    const double h01 = 4.5 * (X2 * (0.0 - 1.0 / 3.0) + Y2 * (1.0 - 1.0 / 3.0));
    const double h11 = 4.5 * (X2 * (1.0 - 1.0 / 3.0) + Y2 * (1.0 - 1.0 / 3.0));
    const double r0 = rho * (4.0 / 9.0), r1 = rho * (1.0 / 9.0), r2 = rho * (1.0 / 36.0);
    double feq[9];
    feq[0] = r0 * (1.0 + h00);
    feq[1] = r1 * ((1.0 + px) + h10);
    feq[2] = r1 * ((1.0 + -px) + h10);
    feq[3] = r1 * ((1.0 + py) + h01);
    feq[4] = r1 * ((1.0 + -py) + h01);
    feq[5] = r2 * (((1.0 + pa) + h11) + d9);
    feq[6] = r2 * (((1.0 + -pa) + h11) + d9);
    feq[7] = r2 * (((1.0 + pb) + h11) + -d9);
    feq[8] = r2 * (((1.0 + -pb) + h11) + -d9);
#pragma unroll
    for (int v = 0; v < 9; v++) {
        const double a = f[v] + omega * (feq[v] - f[v]);
        fs[v] = forced ? a + (1.0 - 0.5 * omega) * lattice_force(v, ux, uy, Fx, Fy) : a;
    }
}

// Central-moments collision (De Rosis 2019; src/Grid.cpp:106-233), in collide_cm.cuh.
template <bool UNF = false>
__device__ __forceinline__ void collide_cm(const double f[9], double rho, double ux, double uy, double Fx,
                                           double Fy, double omega, double cs, double fs[9]);

// force_xy_at in float for the FP32 kernels (values rounded on the host).
__device__ __forceinline__ void force_xy_at_f(const LatDev& L, int t, float& Fx, float& Fy) {
    if (L.womersley) {
        const StepScalars& s = L.steps[t % L.steps_cap];
        Fx = s.fx_f;
        Fy = s.fy_f;
    } else {
        Fx = L.Fx0_f;
        Fy = L.Fy0_f;
    }
}

// force_xy of step t in float at a site whose density after step t-1 was
// rho_n (per-site force; reduced-precision kernels, constants rounded on the
// host).
__device__ __forceinline__ void force_xy_site_f(const LatDev& L, int t, float rho_n, float& Fx, float& Fy) {
    const StepScalars& s = L.steps[t % L.steps_cap];
    Fx = fmaf(rho_n * L.Drho_f, L.gx_f, s.ax_f) * L.fscdm_f;
    Fy = fmaf(rho_n * L.Drho_f, L.gy_f, s.ay_f) * L.fscdm_f;
}

// Whether this case has a step force at all (a value every thread of a
// launch shares): a Womersley pressure gradient or a gravity that is not
// +-0, tested on the bits (no FP64 comparison).
__device__ __forceinline__ bool lattice_forced_d(const LatDev& L) {
    return L.womersley || ((unsigned long long)__double_as_longlong(L.Fx0) << 1) != 0ull ||
           ((unsigned long long)__double_as_longlong(L.Fy0) << 1) != 0ull;
}

// Step index of a launch: its argument, or the device counter in a graph.
__device__ __forceinline__ int step_t(const LatDev& L, int t) { return L.t_dev ? *L.t_dev + L.t_off : t; }

// One time step's scalars: the inlet ramp used by the boundary conditions of
// step t and the uniform pressure-gradient force of step t (Womersley).
__device__ __forceinline__ void force_xy_at(const LatDev& L, int t, double& Fx, double& Fy) {
    if (L.womersley) {
        const StepScalars& s = L.steps[t % L.steps_cap];
        Fx = s.fx;
        Fy = s.fy;
    } else {
        Fx = L.Fx0;
        Fy = L.Fy0;
    }
}

// force_xy of step t at a site whose density after step t-1 was rho_n, with
// gravity beside the Womersley term (GridClass::lbmKernel,
// src/Grid.cpp:59-60, in its operation order).
__device__ __forceinline__ void force_xy_site(const LatDev& L, int t, double rho_n, double& Fx, double& Fy) {
    const StepScalars& s = L.steps[t % L.steps_cap];
    Fx = (rho_n * L.Drho * L.gx + s.ax) * L.fsc / L.Dm;
    Fy = (rho_n * L.Drho * L.gy + s.ay) * L.fsc / L.Dm;
}

// force_xy of step t at site (i, j): the step's value, or with a per-site
// force the value formed from the site's density after step t-1.
__device__ __forceinline__ void force_xy_of(const LatDev& L, int t, int i, int j, double& Fx, double& Fy) {
    if (L.site_force) force_xy_site(L, t, L.rho_prev[(size_t)j * L.pitch + i], Fx, Fy);
    else force_xy_at(L, t, Fx, Fy);
}

// force_xy of step t+1 at a site whose density after step t is rho (the
// force the collision of the next step uses).
__device__ __forceinline__ void force_xy_next(const LatDev& L, int t_next, double rho, double& Fx, double& Fy) {
    if (L.site_force) force_xy_site(L, t_next, rho, Fx, Fy);
    else force_xy_at(L, t_next, Fx, Fy);
}

// Slot of a pressure-boundary corner site in LatDev::corner_prev/next, or -1.
// A corner is a site with a normal in both directions (site_normal).
__device__ __forceinline__ int pressure_corner(int type, int nx, int ny, int i, int j) {
    if (type != LIFE_PRESSURE || nx == 0 || ny == 0) return -1;
    return (i == 0 ? 0 : 1) + (j == 0 ? 0 : 2);
}

// Post-macroscopic moments of a fluid site of step t (read by boundary sites:
// Utils::extrapolate / zeroGradient, inc/Utils.h:137-217), with the site's
// own force_xy.
template <class S>
__device__ __forceinline__ void fluid_moments(const typename S::T* __restrict__ P, const LatDev& L, int t, int i,
                                              int j, double Fx, double Fy, double& rho, double& ux, double& uy) {
    double f[9];
    gather<S>(P, L, i, j, f);
    if (L.site_force) force_xy_site(L, t, L.rho_prev[(size_t)j * L.pitch + i], Fx, Fy);
    macroscopic(f, Fx, Fy, rho, ux, uy);
}

// GridClass::regularisedBC (src/Grid.cpp:387-465) on a local copy of the
// site's populations; rn/uxn/uyn are the site's rho_n/u_n values as applyBCs
// left them.
template <bool CM>
__device__ __forceinline__ void regularised(double f[9], int type, int nx, int ny, int nd, double& rn, double un[2],
                                            double cs, double rho_x1, double rho_x2) {
    const bool corner = (nx != 0 && ny != 0);
    const int nn = nd == 0 ? nx : ny;
    if (corner) {
        if (type == LIFE_VELOCITY || type == LIFE_WALL || type == LIFE_FREESLIP) rn = 2.0 * rho_x1 - rho_x2;
    } else {
        double fplus = 0.0, fzero = 0.0;
#pragma unroll
        for (int v = 0; v < 9; v++) {
            int cn = nd == 0 ? cx_of(v) : cy_of(v);
            if (cn == -nn) fplus += f[v];
            else if (cn == 0) fzero += f[v];
        }
        if (type == LIFE_VELOCITY || type == LIFE_WALL || type == LIFE_FREESLIP)
            rn = (2.0 * fplus + fzero) / (1.0 - nn * un[nd]);
        else if (type == LIFE_PRESSURE)
            un[nd] = nn * (1.0 - (2.0 * fplus + fzero) / rn);
    }
    double Sxx = 0.0, Syy = 0.0, Sxy = 0.0;
#pragma unroll
    for (int v = 0; v < 9; v++) {
        const int cx = cx_of(v), cy = cy_of(v);
        double feq = equilibrium<CM>(v, rn, un[0], un[1]);
        if (corner) {
            if (cx == nx || cy == ny) {
                if (nx * cx + ny * cy == 0) f[v] = feq;
                else f[v] = feq + (f[opp_of(v)] - equilibrium<CM>(opp_of(v), rn, un[0], un[1]));
            }
        } else {
            int cn = nd == 0 ? cx : cy;
            if (cn == nn) f[v] = feq + (f[opp_of(v)] - equilibrium<CM>(opp_of(v), rn, un[0], un[1]));
        }
        double fneq = f[v] - feq;
        Sxx += (double)(cx * cx) * fneq;
        Syy += (double)(cy * cy) * fneq;
        Sxy += (double)(cx * cy) * fneq;
    }
    const double cs2 = LSQ(cs);
#pragma unroll
    for (int v = 0; v < 9; v++) {
        const int cx = cx_of(v), cy = cy_of(v);
        f[v] = equilibrium<CM>(v, rn, un[0], un[1]) +
               (wgt(v) / (2.0 * LQU(cs))) *
                   ((((double)(cx * cx) - cs2) * Sxx) + (((double)(cy * cy) - cs2) * Syy) + (2.0 * cx * cy * Sxy));
    }
}

// The reference state of step t at site (i,j): post-stream populations after
// the boundary condition (GridClass::applyBCs, src/Grid.cpp:302-384;
// convectiveBC :468-474) and the macroscopic moments (without the IBM
// correction, which support sites receive afterwards).
template <bool CM, class S>
__device__ __forceinline__ void site_state(const typename S::T* __restrict__ P, const LatDev& L, int t, int i, int j,
                                           double f[9], double& rho, double& ux, double& uy) {
    gather<S>(P, L, i, j, f);
    double Fx, Fy;
    force_xy_of(L, t, i, j, Fx, Fy);
    const int type = site_type(L, i, j);
    if (type != LIFE_FLUID) {
        if (type == LIFE_CONVECTIVE) {
            const double* fp = L.outlet_f_prev + (size_t)j * 3;
            const double dU0 = L.delU[j * 2 + 0], dU1 = L.delU[j * 2 + 1];
            f[2] = fp[0] + 3.0 * wgt(2) * (dU0 * cx_of(2) + dU1 * cy_of(2));
            f[6] = fp[1] + 3.0 * wgt(6) * (dU0 * cx_of(6) + dU1 * cy_of(6));
            f[8] = fp[2] + 3.0 * wgt(8) * (dU0 * cx_of(8) + dU1 * cy_of(8));
        } else {
            int nx, ny, nd;
            site_normal(L, i, j, nx, ny, nd);
            double rn = 0.0, un[2] = {0.0, 0.0};
            double r1 = 0.0, r2 = 0.0;
            const bool corner = (nx != 0 && ny != 0);
            if (type == LIFE_VELOCITY) {
                const double ramp = L.steps[t % L.steps_cap].ramp;
                un[0] = L.u_in[j * 2 + 0] * ramp;
                un[1] = L.u_in[j * 2 + 1] * ramp;
            } else if (type == LIFE_FREESLIP || type == LIFE_PRESSURE) {
                // zeroGradient order 2 along the normal on the new velocity field
                double q1, a1x, a1y, q2, a2x, a2y;
                fluid_moments<S>(P, L, t, i + nx, j + ny, Fx, Fy, q1, a1x, a1y);
                fluid_moments<S>(P, L, t, i + 2 * nx, j + 2 * ny, Fx, Fy, q2, a2x, a2y);
                if (type == LIFE_FREESLIP) un[nd] = 0.0;
                else rn = L.rho_in[j];
                const int d = 1 - nd;
                const double a1 = d == 0 ? a1x : a1y, a2 = d == 0 ? a2x : a2y;
                un[d] = (4.0 / 3.0) * a1 - (1.0 / 3.0) * a2;
                r1 = q1;
                r2 = q2;
                // a pressure corner sets only the tangential velocity; the
                // normal one is the site's velocity after the previous step
                const int k = pressure_corner(type, nx, ny, i, j);
                if (k >= 0) un[nd] = L.corner_prev[k * 2 + nd];
            }
            if (corner && (type == LIFE_VELOCITY || type == LIFE_WALL)) {
                double a, b;
                fluid_moments<S>(P, L, t, i + nx, j + ny, Fx, Fy, r1, a, b);
                fluid_moments<S>(P, L, t, i + 2 * nx, j + 2 * ny, Fx, Fy, r2, a, b);
            }
            regularised<CM>(f, type, nx, ny, nd, rn, un, L.cs, r1, r2);
        }
    }
    macroscopic(f, Fx, Fy, rho, ux, uy);
}

template <bool CM, bool UNF = false>
__device__ __forceinline__ void collide(const double f[9], double rho, double ux, double uy, double Fx, double Fy,
                                        double omega, double cs, double fs[9]) {
    if (CM) collide_cm<UNF>(f, rho, ux, uy, Fx, Fy, omega, cs, fs);
    else collide_bgk<UNF>(f, rho, ux, uy, Fx, Fy, omega, fs);
}

// Outlet side outputs of step t: final u of the last three columns and the
// post-BC f[2,6,8] of the outlet column.
__device__ __forceinline__ void outlet_outputs(const LatDev& L, int i, int j, const double f[9], double ux, double uy) {
    if (!L.convective) return;
    int c = i - (L.Nx - 3);
    if (c >= 0) {
        L.outlet_u[((size_t)c * L.Ny + j) * 2 + 0] = ux;
        L.outlet_u[((size_t)c * L.Ny + j) * 2 + 1] = uy;
    }
    if (i == L.Nx - 1) {
        double* o = L.outlet_f_next + (size_t)j * 3;
        o[0] = f[2];
        o[1] = f[6];
        o[2] = f[8];
    }
}

template <bool CM, class S>
__device__ __forceinline__ void store_collided(typename S::T* __restrict__ B, const LatDev& L, int t_next, int i,
                                               int j, const double f[9], double rho, double ux, double uy, double Ix,
                                               double Iy) {
    double Fx, Fy, fs[9];
    force_xy_next(L, t_next, rho, Fx, Fy);
    collide<CM>(f, rho, ux, uy, Fx + Ix, Fy + Iy, L.omega, L.cs, fs);
    const size_t s = (size_t)j * L.pitch + i;
#pragma unroll
    for (int v = 0; v < 9; v++) B[(size_t)v * L.S + s] = S::save(fs[v], v);
}


// What the next step reads of this step's result at a boundary site: the
// density (per-site force) and, at a pressure corner, the velocity.
__device__ __forceinline__ void store_history(const LatDev& L, int type, int i, int j, double rho, double ux,
                                              double uy) {
    if (L.site_force) L.rho_next[(size_t)j * L.pitch + i] = rho;
    if (type == LIFE_PRESSURE) {
        int nx, ny, nd;
        site_normal(L, i, j, nx, ny, nd);
        const int k = pressure_corner(type, nx, ny, i, j);
        if (k >= 0) {
            L.corner_next[k * 2 + 0] = ux;
            L.corner_next[k * 2 + 1] = uy;
        }
    }
}

// Boundary-condition site q of the perimeter, enumerated bottom row, top row,
// left column, right column: its step-t state by site_state() (regularised /
// convective conditions applied), the outlet side outputs, and the collision
// of the next step into B. FP64 arithmetic for every storage form.
template <bool CM, class S>
__device__ __forceinline__ void perimeter_site(const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                               const LatDev& L, int t, int q) {
    const int Nx = L.Nx, Ny = L.Ny;
    int i, j;
    if (q < Nx) { i = q; j = 0; }
    else if (q < 2 * Nx) { i = q - Nx; j = Ny - 1; }
    else if (q < 2 * Nx + (Ny - 2)) { i = 0; j = q - 2 * Nx + 1; }
    else if (q < 2 * Nx + 2 * (Ny - 2)) { i = Nx - 1; j = q - 2 * Nx - (Ny - 2) + 1; }
    else return;
    const int type = site_type(L, i, j);
    if (type == LIFE_FLUID) return;
    double f[9], rho, ux, uy;
    site_state<CM, S>(A, L, t, i, j, f, rho, ux, uy);
    outlet_outputs(L, i, j, f, ux, uy);
    store_history(L, type, i, j, rho, ux, uy);
    store_collided<CM, S>(B, L, t + 1, i, j, f, rho, ux, uy, 0.0, 0.0);
}

}  // namespace life
