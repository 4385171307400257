// Reduced-precision lattice kernels: FP32 shifted populations and FP16
// storage, both collided in FP32. The unit is compiled without FMA
// contraction (so the FP64 boundary code it shares with lbm_f64.cu rounds
// exactly as there); the FP32 arithmetic spells its fused multiply-adds out
// with fmaf().
//
// Interior (fluid) sites take this fast path. It holds only the deviations
// g_v = f_v - w_v in registers:
//   drho = sum g_v,  rho = 1 + drho,  rho*u = sum c_v g_v + F/2,
// and writes post-collision deviations, so no term of size w_v ever enters an
// FP32 sum. Boundary-condition sites go to the perimeter kernel and IBM
// support sites to the IBM fix-up kernel; both convert to FP64 and reuse the
// reference-order code (lbm_device.cuh).
//
// BGK (GridClass::streamCollide BGK branch, reference src/Grid.cpp:236-244):
//   g*_v = g_v + omega (geq_v - g_v) + (1 - omega/2) F_v
//   geq_v = w_v [drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u.u)]
//   F_v   = 3 w_v [(c - u).F + 3 (c.u)(c.F)]
// Central moments (src/Grid.cpp:106-233, De Rosis 2019): the inverse transform
// is linear in the moments k; its rest-state part factorises per axis,
//   E_v(u) = e(cx,ux) e(cy,uy),  e(0,u) = 2/3 - u^2,  e(+-1,u) = 1/6 +- u/2 + u^2/2,
// so g*_v = drho E_v + (E_v - w_v) + sum_m T_vm(u) k_m over the force and
// stress moments, with E_v - w_v = w_x d_y + d_x w_y + d_x d_y free of
// cancellation (d = e - e|_{u=0}).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include <cudaTypedefs.h>

#include "collide_cm.cuh"
#include "lbm_device.cuh"
#include <type_traits>

#include "lbm_kernels.h"
#include "tma.cuh"

namespace life {

// Two sites' FP32 arithmetic in one instruction: the packed f32x2 add / mul /
// fma of sm_100+, written as inline PTX with the explicit .rn rounding mode.
// Each lane is an IEEE round-to-nearest FP32 operation, so each lane of a V2
// computation gives, bit for bit, the float computation written with the
// same expressions (a - b is a + (-b) in IEEE arithmetic, signed zeros
// included; negation flips the sign bits), provided no product is fused
// into a following addition: in this kernel the compiler did fuse one
// lane's multiply and add into an fma (with the __fmul2_rn / __fadd2_rn
// intrinsics and with this inline PTX alike; measured as one unit in the
// last place on ~1 site in 10^6 per step), which the one-site path, compiled
// without contraction, does not do. The BGK collision below is therefore
// written so that no product feeds an addition, and the packed form is used
// for BGK only.
struct V2 {
    unsigned long long b;  // lane x in the low 32 bits, lane y in the high 32 bits
    __device__ __forceinline__ float x() const {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(b));
        return lo;
    }
    __device__ __forceinline__ float y() const {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(b));
        return hi;
    }
};
__device__ __forceinline__ V2 v2(float a, float b) {
    V2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.b) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ V2 v2(float a) { return v2(a, a); }
__device__ __forceinline__ V2 operator+(V2 a, V2 b) {
    V2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.b) : "l"(a.b), "l"(b.b));
    return r;
}
// negation flips the sign bits (two integer operations; the collision below
// puts its signs into constants instead)
__device__ __forceinline__ V2 operator-(V2 a) { return V2{a.b ^ 0x8000000080000000ull}; }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) {
    V2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.b) : "l"(a.b), "l"(b.b));
    return r;
}
__device__ __forceinline__ V2 operator*(V2 a, V2 b) {
    V2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.b) : "l"(a.b), "l"(b.b));
    return r;
}
__device__ __forceinline__ V2 operator+(float a, V2 b) { return v2(a) + b; }
__device__ __forceinline__ V2 operator+(V2 a, float b) { return a + v2(b); }
__device__ __forceinline__ V2 operator-(float a, V2 b) { return v2(a) - b; }
__device__ __forceinline__ V2 operator-(V2 a, float b) { return a - v2(b); }
__device__ __forceinline__ V2 operator*(float a, V2 b) { return v2(a) * b; }
__device__ __forceinline__ V2 operator*(V2 a, float b) { return a * v2(b); }
__device__ __forceinline__ V2 fmaf(V2 a, V2 b, V2 c) {
    V2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.b) : "l"(a.b), "l"(b.b), "l"(c.b));
    return r;
}
__device__ __forceinline__ V2 fmaf(float a, V2 b, V2 c) { return fmaf(v2(a), b, c); }
__device__ __forceinline__ V2 fmaf(V2 a, float b, V2 c) { return fmaf(a, v2(b), c); }
__device__ __forceinline__ V2 fmaf(V2 a, V2 b, float c) { return fmaf(a, b, v2(c)); }
__device__ __forceinline__ V2 fmaf(float a, float b, V2 c) { return fmaf(v2(a), v2(b), c); }
__device__ __forceinline__ V2 fmaf(float a, V2 b, float c) { return fmaf(v2(a), b, v2(c)); }
__device__ __forceinline__ V2 fmaf(V2 a, float b, float c) { return fmaf(a, v2(b), v2(c)); }
using ::fmaf;

template <class T> __device__ __forceinline__ T zero_of();
template <> __device__ __forceinline__ float zero_of<float>() { return 0.0f; }
template <> __device__ __forceinline__ V2 zero_of<V2>() { return v2(0.0f); }

template <class T>
__device__ __forceinline__ void e1d(T u, T e[3], float w[3], T d[3]) {
    // index 0: c = 0, 1: c = +1, 2: c = -1
    const T u2 = u * u;
    w[0] = 2.0f / 3.0f;
    w[1] = w[2] = 1.0f / 6.0f;
    d[0] = -u2;
    d[1] = fmaf(0.5f, u, 0.5f * u2);
    d[2] = fmaf(-0.5f, u, 0.5f * u2);
    e[0] = w[0] + d[0];
    e[1] = w[1] + d[1];
    e[2] = w[2] + d[2];
}

__device__ __forceinline__ int ax(int c) { return c == 0 ? 0 : (c > 0 ? 1 : 2); }

// c_v . (a, b) for the D2Q9 velocity v (components 0 or +-1, known at
// compile time after unrolling): only the additions and signs it needs.
template <class T>
__device__ __forceinline__ T cdot(int v, T a, T b) {
    const int cx = cx_of(v), cy = cy_of(v);
    const T xa = cx == 0 ? zero_of<T>() : (cx > 0 ? a : -a);
    if (cy == 0) return xa;
    const T yb = cy > 0 ? b : -b;
    return cx == 0 ? yb : xa + yb;
}

// FORCED = false: the force of this step is zero everywhere (no gravity, no
// Womersley term), so every forcing term is an exact zero and is not formed.
// px, py: the momentum with the half force term, inv = 1/rho (ux = px inv,
// uy = py inv). In BGK no product feeds an addition: c.u of a diagonal
// direction is (px +- py) inv, and w (rho inner + dr) - g is one fused
// multiply-add. A compiler that fuses a product into a following addition
// (as one did for the packed two-site form) then has nothing to fuse, so the
// one-site and two-site forms round identically.
// RAW (BGK with FP16 storage): r holds the stored values (g_v = r_v s_v with
// the direction's power-of-two scale s_v), and gs receives the stored values
// of the result, g*_v / s_v. Multiplying by a power of two commutes with
// round-to-nearest (no result comes near the FP32 subnormal range), so
// w / s_v (w (...) - g_v) rounds to the same value divided by s_v, and the
// relaxation with r_v in place of g_v gives g*_v / s_v with no multiply per
// direction on the way out.
template <bool CM, bool FORCED, bool RAW = false, class T>
__device__ __forceinline__ void collide_dev32(const T g[9], const T r[9], T dr, T rho, T mx, T my, T ux, T uy, T px,
                                              T py, T inv, float Gx, float Gy, float omega, T gs[9]) {
    if (!CM) {
        // Signs sit in constants, not in negations of values (free for one
        // float, but two integer operations for a packed pair); each rewrite
        // below is exact (negation commutes with round-to-nearest), so every
        // value is the one of the plain form
        //   inner = fma(4.5 cu, cu, fma(3, cu, -1.5 u.u)),
        //   g* = fma(omega, fma(w, fma(rho, inner, dr), -g), g).
        // A direction's c.u is s c0 with s = +-1 and c0 one of ux, uy,
        // cs = c.u of (1,1), cd = c.u of (1,-1): (4.5 c.u) c.u = (4.5 c0) c0,
        // fma(3, c.u, x) = fma(3 s, c0, x), and fma(w, z, -g) = -fma(-w, z, g),
        // so g* = fma(-omega, fma(-w, z, g), g).
        const T nusq = (-1.5f) * fmaf(ux, ux, uy * uy);
        const T uF = FORCED ? fmaf(ux, Gx, uy * Gy) : zero_of<T>();
        const float fo = fmaf(-0.5f, omega, 1.0f);
        const T cs = (px + py) * inv, cd = (px - py) * inv;
        const T c0[4] = {ux, uy, cs, cd};
        T q4[4], q3[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            q4[k] = 4.5f * c0[k];
            if (FORCED) q3[k] = 3.0f * c0[k];
        }
#pragma unroll
        for (int v = 0; v < 9; v++) {
            const float w = wgt_f(v);
            const int cx = cx_of(v), cy = cy_of(v);
            const int k = cy == 0 ? 0 : (cx == 0 ? 1 : (cx == cy ? 2 : 3));
            const float sg = (cx != 0 ? cx : cy) > 0 ? 1.0f : -1.0f;
            const bool rest = cx == 0 && cy == 0;
            const T inner = rest ? fmaf(zero_of<T>(), zero_of<T>(), fmaf(3.0f, zero_of<T>(), nusq))
                                 : fmaf(q4[k], c0[k], fmaf(3.0f * sg, c0[k], nusq));
            const float sv = RAW ? h16_inv(v) : 1.0f;
            const T gv = RAW ? r[v] : g[v];
            const T a = fmaf(-omega, fmaf(-(w * sv), fmaf(rho, inner, dr), gv), gv);
            if (FORCED) {
                // fma(3 c.u, cF, cF - u.F) = fma(3 c0, s cF, cF - u.F)
                const float cF = cdot(v, Gx, Gy);
                const T t = rest ? fmaf(zero_of<T>(), cF, cF - uF) : fmaf(q3[k], sg * cF, cF - uF);
                const T Fv = ((3.0f * w) * sv) * t;
                gs[v] = fmaf(fo, Fv, a);
            } else {
                gs[v] = a;
            }
        }
    } else {
        // raw second moments of the deviations
        const T dxxyy = (g[1] + g[2]) - (g[3] + g[4]);
        const T gxy = (g[5] + g[6]) - (g[7] + g[8]);
        const float om1 = 1.0f - omega;
        const T k4 = om1 * fmaf(ux * ux - uy * uy, rho, fmaf(2.0f * uy, my, fmaf(-2.0f * ux, mx, dxxyy)));
        const T k5 = om1 * fmaf(ux * uy, rho, fmaf(-ux, my, fmaf(-uy, mx, gxy)));
        // force moments (exact zeros, and unused, when not FORCED)
        const float k1 = FORCED ? 0.5f * Gx : 0.0f, k2 = FORCED ? 0.5f * Gy : 0.0f;
        const float k7 = FORCED ? Gx * (1.0f / 6.0f) : 0.0f, k6 = FORCED ? Gy * (1.0f / 6.0f) : 0.0f;
        T ex[3], dx[3], ey[3], dy[3];
        float wx[3], wy[3];
        e1d(ux, ex, wx, dx);
        e1d(uy, ey, wy, dy);
        const T X2 = ux * ux, Y2 = uy * uy, XY = ux * uy;
        // T_v1..T_v7 (force/stress columns of the inverse transform)
        T T1[9], T2[9], T4[9], T5[9], T6[9], T7[9];
        T1[0] = 2.0f * ux * (Y2 - 1.0f);          T2[0] = 2.0f * uy * (X2 - 1.0f);
        T4[0] = -0.5f * (X2 - Y2);                T5[0] = 4.0f * XY;
        T6[0] = 2.0f * uy;                        T7[0] = 2.0f * ux;
        T1[1] = -0.5f * (2.0f * ux + 1.0f) * (Y2 - 1.0f);  T2[1] = -XY * (ux + 1.0f);
        T4[1] = 0.25f * (X2 + ux - Y2 + 1.0f);    T5[1] = -uy * (2.0f * ux + 1.0f);
        T6[1] = -uy;                              T7[1] = -0.5f * (2.0f * ux + 1.0f);
        T1[2] = -0.5f * (2.0f * ux - 1.0f) * (Y2 - 1.0f);  T2[2] = -XY * (ux - 1.0f);
        T4[2] = 0.25f * (X2 - ux - Y2 + 1.0f);    T5[2] = -uy * (2.0f * ux - 1.0f);
        T6[2] = -uy;                              T7[2] = -0.5f * (2.0f * ux - 1.0f);
        T1[3] = -XY * (uy + 1.0f);                T2[3] = -0.5f * (X2 - 1.0f) * (2.0f * uy + 1.0f);
        T4[3] = 0.25f * (X2 - Y2 - uy - 1.0f);    T5[3] = -ux * (2.0f * uy + 1.0f);
        T6[3] = -0.5f * (2.0f * uy + 1.0f);       T7[3] = -ux;
        T1[4] = -XY * (uy - 1.0f);                T2[4] = -0.5f * (X2 - 1.0f) * (2.0f * uy - 1.0f);
        T4[4] = 0.25f * (X2 - Y2 + uy - 1.0f);    T5[4] = -ux * (2.0f * uy - 1.0f);
        T6[4] = -0.5f * (2.0f * uy - 1.0f);       T7[4] = -ux;
        T1[5] = 0.25f * uy * (2.0f * ux + 1.0f) * (uy + 1.0f);  T2[5] = 0.25f * ux * (ux + 1.0f) * (2.0f * uy + 1.0f);
        T4[5] = -0.125f * (ux - uy) * (ux + uy + 1.0f);          T5[5] = 0.25f * (2.0f * ux + 1.0f) * (2.0f * uy + 1.0f);
        T6[5] = 0.25f * (2.0f * uy + 1.0f);                      T7[5] = 0.25f * (2.0f * ux + 1.0f);
        T1[6] = 0.25f * uy * (2.0f * ux - 1.0f) * (uy - 1.0f);  T2[6] = 0.25f * ux * (ux - 1.0f) * (2.0f * uy - 1.0f);
        T4[6] = -0.125f * (ux - uy) * (ux + uy - 1.0f);          T5[6] = 0.25f * (2.0f * ux - 1.0f) * (2.0f * uy - 1.0f);
        T6[6] = 0.25f * (2.0f * uy - 1.0f);                      T7[6] = 0.25f * (2.0f * ux - 1.0f);
        T1[7] = 0.25f * uy * (2.0f * ux + 1.0f) * (uy - 1.0f);  T2[7] = 0.25f * ux * (ux + 1.0f) * (2.0f * uy - 1.0f);
        T4[7] = -0.125f * (ux + uy) * (ux - uy + 1.0f);          T5[7] = 0.25f * (2.0f * ux + 1.0f) * (2.0f * uy - 1.0f);
        T6[7] = 0.25f * (2.0f * uy - 1.0f);                      T7[7] = 0.25f * (2.0f * ux + 1.0f);
        T1[8] = 0.25f * uy * (2.0f * ux - 1.0f) * (uy + 1.0f);  T2[8] = 0.25f * ux * (ux - 1.0f) * (2.0f * uy + 1.0f);
        T4[8] = -0.125f * (ux + uy) * (ux - uy - 1.0f);          T5[8] = 0.25f * (2.0f * ux - 1.0f) * (2.0f * uy + 1.0f);
        T6[8] = 0.25f * (2.0f * uy + 1.0f);                      T7[8] = 0.25f * (2.0f * ux - 1.0f);
#pragma unroll
        for (int v = 0; v < 9; v++) {
            const int a = ax(cx_of(v)), b = ax(cy_of(v));
            const T E = ex[a] * ey[b];
            const T D = fmaf(dx[a], dy[b], fmaf(wx[a], dy[b], dx[a] * wy[b]));
            T acc = fmaf(dr, E, D);
            if (FORCED) {
                acc = fmaf(T1[v], k1, acc);
                acc = fmaf(T2[v], k2, acc);
            }
            acc = fmaf(T4[v], k4, acc);
            acc = fmaf(T5[v], k5, acc);
            if (FORCED) {
                acc = fmaf(T6[v], k6, acc);
                acc = fmaf(T7[v], k7, acc);
            }
            gs[v] = acc;
        }
    }
}

template <bool CM, bool FORCED, class S, bool SITE = false>
__device__ __forceinline__ void finish_site_lowp(const float r[9], typename S::T* __restrict__ B, const LatDev& L,
                                                 int t, int i, int j);

// One interior site, reduced-precision storage. Sites on a boundary-condition
// wall are left to the perimeter kernel.
template <bool CM, bool FORCED, class S, bool SITE = false>
__device__ __forceinline__ void interior_site_lowp_f(const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                                     const LatDev& L, int t, int i, int j) {
    if (site_type(L, i, j) != LIFE_FLUID) return;
    const bool edge = (i == 0) | (i == L.Nx - 1) | (j == 0) | (j == L.Ny - 1);
    float r[9];
    const size_t base = (size_t)j * L.pitch + i;
    if (!edge) {
#pragma unroll
        for (int v = 0; v < 9; v++)
            r[v] = S::raw(A[(size_t)v * L.S + base - cx_of(v) - (long long)cy_of(v) * L.pitch]);
    } else {
#pragma unroll
        for (int v = 0; v < 9; v++) {
            int si = i - cx_of(v), sj = j - cy_of(v);
            si = si < 0 ? si + L.Nx : (si >= L.Nx ? si - L.Nx : si);
            sj = sj < 0 ? sj + L.Ny : (sj >= L.Ny ? sj - L.Ny : sj);
            r[v] = S::raw(A[(size_t)v * L.S + (size_t)sj * L.pitch + si]);
        }
    }
    finish_site_lowp<CM, FORCED, S, SITE>(r, B, L, t, i, j);
}

// The rest of an interior site once its nine pulled stored values r (as
// floats) are in registers: deviations, moments, outlet columns, collision,
// store. SITE: the case has a per-site force (WOMERSLEY with gravity; a
// separate instantiation, used only by the kernels that take such cases).
template <bool CM, bool FORCED, class S, bool SITE>
__device__ __forceinline__ void finish_site_lowp(const float r[9], typename S::T* __restrict__ B, const LatDev& L,
                                                 int t, int i, int j) {
    constexpr bool RAW = S::SCALED && !CM;
    float g[9];
#pragma unroll
    for (int v = 0; v < 9; v++) g[v] = S::scaled(r[v], v);
    const size_t base = (size_t)j * L.pitch + i;
    float Fxd = 0.0f, Fyd = 0.0f, Gxd = 0.0f, Gyd = 0.0f;
    if (FORCED) {
        if (SITE) {
            force_xy_site_f(L, t, (float)L.rho_prev[base], Fxd, Fyd);
        } else {
            force_xy_at_f(L, t, Fxd, Fyd);
            force_xy_at_f(L, t + 1, Gxd, Gyd);
        }
    }
    const float dr = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) + g[8];
    const float rho = 1.0f + dr;
    if (FORCED && SITE) {
        force_xy_site_f(L, t + 1, rho, Gxd, Gyd);
        L.rho_next[base] = (double)rho;
    }
    const float mx = (g[1] - g[2]) + (g[5] - g[6]) + (g[7] - g[8]);
    const float my = (g[3] - g[4]) + (g[5] - g[6]) + (g[8] - g[7]);
    const float inv = rcp_lowp(rho);
    const float px = FORCED ? fmaf(0.5f, Fxd, mx) : mx, py = FORCED ? fmaf(0.5f, Fyd, my) : my;
    const float ux = px * inv, uy = py * inv;
    if (L.convective && i >= L.Nx - 3) {
        const int c = i - (L.Nx - 3);
        L.outlet_u[((size_t)c * L.Ny + j) * 2 + 0] = ux;
        L.outlet_u[((size_t)c * L.Ny + j) * 2 + 1] = uy;
    }
    float gs[9];
    collide_dev32<CM, FORCED, RAW>(g, r, dr, rho, mx, my, ux, uy, px, py, inv, Gxd, Gyd, L.omega_f, gs);
#pragma unroll
    for (int v = 0; v < 9; v++) B[(size_t)v * L.S + base] = RAW ? S::put_raw(gs[v]) : S::put(gs[v], v);
}

// Whether step forces exist at all for this case (a value every thread of a
// launch shares): a Womersley pressure gradient or a non-zero gravity.
__device__ __forceinline__ bool lattice_forced(const LatDev& L) {
    return L.womersley || L.Fx0_f != 0.0f || L.Fy0_f != 0.0f;
}

// SITE_OK: the kernel also takes cases with a per-site force (the one-step
// kernels k_step_lowp / k_step_tma do not; such cases use k_interior_lowp).
template <bool CM, class S, bool SITE_OK = true>
__device__ __forceinline__ void interior_site_lowp(const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                                   const LatDev& L, int t, int i, int j) {
    if (SITE_OK && L.site_force) interior_site_lowp_f<CM, true, S, true>(A, B, L, t, i, j);
    else if (lattice_forced(L)) interior_site_lowp_f<CM, true, S>(A, B, L, t, i, j);
    else interior_site_lowp_f<CM, false, S>(A, B, L, t, i, j);
}

template <bool CM, class S>
__global__ void __launch_bounds__(256) k_interior_lowp(const typename S::T* __restrict__ A,
                                                       typename S::T* __restrict__ B, LatDev L, int t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    interior_site_lowp<CM, S>(A, B, L, step_t(L, t), i, j);
}

// All cases of a batch in one persistent launch. Tile q of the batch belongs
// to case tile_case[q]; inside the case it covers tile_w sites of tile_h rows
// (tile_w = blockDim.x). Each CTA walks tiles q = blockIdx.x, +gridDim.x, ...
// The collision model is a per-case value, uniform over a CTA.
template <class S>
__global__ void __launch_bounds__(256) k_interior_batch_lowp(const BatchLatCase* __restrict__ cases,
                                                             const int* __restrict__ tile_case, int ntiles,
                                                             int tile_h, int phase) {
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
        const BatchLatCase& C = cases[tile_case[q]];
        const LatDev& L = C.L[phase];
        const int lt = q - C.tile0;
        const int tx = lt % C.tiles_x, ty = lt / C.tiles_x;
        const int i = tx * blockDim.x + threadIdx.x;
        if (i >= L.Nx) continue;
        const int t = step_t(L, 0);
        const typename S::T* A = (const typename S::T*)C.A[phase];
        typename S::T* B = (typename S::T*)C.B[phase];
        const int j1 = (ty + 1) * tile_h < L.Ny ? (ty + 1) * tile_h : L.Ny;
        for (int j = ty * tile_h; j < j1; j++) {
            if (L.cm) interior_site_lowp<true, S>(A, B, L, t, i, j);
            else interior_site_lowp<false, S>(A, B, L, t, i, j);
        }
    }
}

cudaError_t launch_interior_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    const dim3 grid((L.Nx + 255) / 256, L.Ny);
    if (L.prec == LIFE_PREC_F32) {
        if (L.cm) k_interior_lowp<true, StoreF32><<<grid, 256, 0, s>>>((const float*)A, (float*)B, L, t);
        else k_interior_lowp<false, StoreF32><<<grid, 256, 0, s>>>((const float*)A, (float*)B, L, t);
    } else {
        if (L.cm) k_interior_lowp<true, StoreF16><<<grid, 256, 0, s>>>((const __half*)A, (__half*)B, L, t);
        else k_interior_lowp<false, StoreF16><<<grid, 256, 0, s>>>((const __half*)A, (__half*)B, L, t);
    }
    return cudaGetLastError();
}

// Boundary-condition sites, reduced-precision storage (perimeter_site,
// lbm_device.cuh; FP64 arithmetic, rounded as in lbm_f64.cu).
template <bool CM, class S>
__global__ void k_perimeter_lowp(const typename S::T* __restrict__ A, typename S::T* __restrict__ B, LatDev L, int t) {
    perimeter_site<CM, S>(A, B, L, step_t(L, t), blockIdx.x * blockDim.x + threadIdx.x);
}

// One warp per block: a boundary site is a long FP64 chain, and an SM's FP64
// unit is narrow, so the sites are spread over as many SMs as possible
// rather than packed four warps to an SM.
cudaError_t launch_perimeter_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    const int n = 2 * L.Nx + 2 * (L.Ny - 2);
    const int g = (n + 31) / 32;
    if (L.prec == LIFE_PREC_F32) {
        if (L.cm) k_perimeter_lowp<true, StoreF32><<<g, 32, 0, s>>>((const float*)A, (float*)B, L, t);
        else k_perimeter_lowp<false, StoreF32><<<g, 32, 0, s>>>((const float*)A, (float*)B, L, t);
    } else {
        if (L.cm) k_perimeter_lowp<true, StoreF16><<<g, 32, 0, s>>>((const __half*)A, (__half*)B, L, t);
        else k_perimeter_lowp<false, StoreF16><<<g, 32, 0, s>>>((const __half*)A, (__half*)B, L, t);
    }
    return cudaGetLastError();
}

// The perimeter path of k_step_lowp as a separate (not inlined) function: it
// needs more registers than the interior path, and the spills the launch
// bound forces stay inside it.
template <bool CM, class S>
__device__ __noinline__ void perimeter_site_call(const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                                 const LatDev& L, int t, int q) {
    perimeter_site<CM, S>(A, B, L, t, q);
}

// One whole step of one case in one launch: the first `pb` blocks take the
// boundary perimeter (long FP64 chains on few sites), the rest the interior
// rows (256 sites per block). Blocks are dispatched in index order, so the
// perimeter starts at once and finishes under the interior's time. The
// launch bound keeps the interior's register budget (and occupancy); the
// perimeter path spills to local memory instead.
// The interior block index b splits into row j = b / bx and column block
// b - j bx; with bx_m != 0 the quotient is __umulhi(b, bx_m), which the host
// has checked to be exact for every b of the launch.
template <bool CM, class S>
__global__ void __launch_bounds__(256, 6) k_step_lowp(const typename S::T* __restrict__ A,
                                                      typename S::T* __restrict__ B, LatDev L, int t, int pb, int bx,
                                                      unsigned bx_m) {
    t = step_t(L, t);
    if ((int)blockIdx.x < pb) {
        perimeter_site_call<CM, S>(A, B, L, t, blockIdx.x * blockDim.x + threadIdx.x);
        return;
    }
    const unsigned b = blockIdx.x - pb;
    const int j = bx_m ? (int)__umulhi(b, bx_m) : (int)(b / (unsigned)bx);
    const int i = (int)(b - (unsigned)j * (unsigned)bx) * blockDim.x + threadIdx.x;
    if (i >= L.Nx) return;
    interior_site_lowp<CM, S, false>(A, B, L, t, i, j);
}

// ---- TMA-staged tiles ---------------------------------------------------
//
// Persistent CTAs take the interior tiles (W x H sites of rows 1..Ny-2 and
// columns 1..Nx-2) from a counter. For each tile one thread issues one bulk
// tensor copy of the tile plus a halo of one row above and below and HALO
// sites left and right (HALO keeps the box start on a 16-byte boundary), for
// all nine population planes, into one of the shared-memory stages, while the
// CTA computes an earlier tile; the copy's completion is counted on the
// stage's mbarrier. The sites then read their nine pulled populations from
// shared memory and finish exactly as in the one-site path
// (finish_site_lowp), so the results are the same bits. The first blocks of
// the grid take the boundary-condition sites and the periodic edge sites, as
// in k_step_lowp.
template <class S>
struct TmaTile;
#ifndef LIFE_TMA_F16_H
#define LIFE_TMA_F16_H 12
#endif
#ifndef LIFE_TMA_F16_STAGES
#define LIFE_TMA_F16_STAGES 2
#endif
#ifndef LIFE_TMA_F16_CTAS
#define LIFE_TMA_F16_CTAS 3
#endif
template <>
struct TmaTile<StoreF16> {
    static constexpr int W = 128, H = LIFE_TMA_F16_H, HALO = 8, ELEM = 2, STAGES = LIFE_TMA_F16_STAGES;
    static constexpr int CTAS = LIFE_TMA_F16_CTAS;  // resident CTAs per SM the register budget is set for
    static constexpr CUtensorMapDataType DTYPE = CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
};
#ifndef LIFE_TMA_F32_H
#define LIFE_TMA_F32_H 8
#endif
#ifndef LIFE_TMA_F32_CTAS
#define LIFE_TMA_F32_CTAS 2
#endif
template <>
struct TmaTile<StoreF32> {
    static constexpr int W = 128, H = LIFE_TMA_F32_H, HALO = 4, ELEM = 4, STAGES = 2, CTAS = LIFE_TMA_F32_CTAS;
    static constexpr CUtensorMapDataType DTYPE = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
};
template <class S>
struct TmaShape {
    static constexpr int Wb = TmaTile<S>::W + 2 * TmaTile<S>::HALO, Hb = TmaTile<S>::H + 2;
    static constexpr int BOX = Wb * Hb * TmaTile<S>::ELEM;  // bytes of one plane's box
    // the nine planes of a tile arrive as one (Wb, Hb, 9) box, densely packed
    static constexpr int PLANE = BOX;
    static constexpr int STAGE = (9 * PLANE + 127) / 128 * 128;
    static constexpr int NST = TmaTile<S>::STAGES;
    // the stages, one mbarrier per stage and a flag, and slack to align the
    // stages to 128 bytes (the bulk tensor copies' shared-memory alignment)
    static constexpr int SMEM = NST * STAGE + 128 + 128;
    static_assert(16 * NST + 4 * (NST + 1) <= 128, "mbarriers and tile slots fit the 128-byte tail");
};

// Waits that gave up (never expected; the host turns a non-zero count into
// LIFE_ERR_TIMEOUT).
__device__ int g_tma_timeouts;

__device__ __forceinline__ bool perimeter_ij(const LatDev& L, int q, int& i, int& j) {
    const int Nx = L.Nx, Ny = L.Ny;
    if (q < Nx) { i = q; j = 0; }
    else if (q < 2 * Nx) { i = q - Nx; j = Ny - 1; }
    else if (q < 2 * Nx + (Ny - 2)) { i = 0; j = q - 2 * Nx + 1; }
    else if (q < 2 * Nx + 2 * (Ny - 2)) { i = Nx - 1; j = q - 2 * Nx - (Ny - 2) + 1; }
    else return false;
    return true;
}

template <bool CM, bool FORCED, class S>
__device__ __forceinline__ void tma_tile_sites(const unsigned char* stage, typename S::T* __restrict__ B,
                                               const LatDev& L, int t, int i0, int j0) {
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    const int ii = (int)threadIdx.x % TT::W;
    const int i = i0 + ii;
    if (i < 1 || i > L.Nx - 2) return;
    for (int jj = (int)threadIdx.x / TT::W; jj < TT::H; jj += (int)blockDim.x / TT::W) {
        const int j = j0 + jj;
        if (j > L.Ny - 2) break;
        float r[9];
#pragma unroll
        for (int v = 0; v < 9; v++) {
            const typename S::T* plane = reinterpret_cast<const typename S::T*>(stage + v * SH::PLANE);
            r[v] = S::raw(plane[(jj + 1 - cy_of(v)) * SH::Wb + (ii + TT::HALO - cx_of(v))]);
        }
        finish_site_lowp<CM, FORCED, S>(r, B, L, t, i, j);
    }
}

// Two adjacent stored values as floats (S::raw of each), and back (S::put_raw).
template <class S>
struct PairIO;
template <>
struct PairIO<StoreF16> {
    __device__ static __forceinline__ V2 load2(const __half* p) {  // p 4-byte aligned
        const __half2 h = *reinterpret_cast<const __half2*>(p);
        return v2(__half2float(__low2half(h)), __half2float(__high2half(h)));
    }
    __device__ static __forceinline__ V2 load11(const __half* p) {
        return v2(__half2float(p[0]), __half2float(p[1]));
    }
    __device__ static __forceinline__ void store2(__half* p, V2 o) {  // p 4-byte aligned
        *reinterpret_cast<__half2*>(p) = __halves2half2(__float2half_rn(o.x()), __float2half_rn(o.y()));
    }
};
template <>
struct PairIO<StoreF32> {
    __device__ static __forceinline__ V2 load2(const float* p) {  // p 8-byte aligned
        const float2 f = *reinterpret_cast<const float2*>(p);
        return v2(f.x, f.y);
    }
    __device__ static __forceinline__ V2 load11(const float* p) { return v2(p[0], p[1]); }
    __device__ static __forceinline__ void store2(float* p, V2 o) {  // p 8-byte aligned
        *reinterpret_cast<float2*>(p) = make_float2(o.x(), o.y());
    }
};

// BGK tiles with two x-adjacent sites per thread (an even column and the
// next): paired loads where the pulled pair is aligned (directions with no x
// component), the collision in packed FP32x2 (V2), and one paired store per
// direction. Each lane computes exactly what finish_site_lowp computes for
// its site (the same operations in the same order), so the results are the
// same bits. Pairs with a site outside columns 1..Nx-2, or reaching the
// convective outlet's last three columns (which also write side outputs),
// take the one-site path.
// The pair of columns (ii, ii+1) of tile row jj.
template <bool FORCED, class S>
__device__ __forceinline__ void tma_pair(const unsigned char* stage, typename S::T* __restrict__ B, const LatDev& L,
                                         int t, int i0, int j0, int jj, int ii) {
    using T = typename S::T;
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    const int i = i0 + ii;
    const bool full = i >= 1 && i + 1 <= L.Nx - 2 && !(L.convective && i + 1 >= L.Nx - 3);
    const int j = j0 + jj;
    if (j > L.Ny - 2) return;
    if (!full) {
        for (int q = 0; q < 2; q++) {
            const int iq = i + q;
            if (iq < 1 || iq > L.Nx - 2) continue;
            float r[9];
#pragma unroll
            for (int v = 0; v < 9; v++) {
                const T* plane = reinterpret_cast<const T*>(stage + v * SH::PLANE);
                r[v] = S::raw(plane[(jj + 1 - cy_of(v)) * SH::Wb + (ii + q + TT::HALO - cx_of(v))]);
            }
            finish_site_lowp<false, FORCED, S>(r, B, L, t, iq, j);
        }
        return;
    }
    V2 r[9], g[9];
#pragma unroll
    for (int v = 0; v < 9; v++) {
        const T* plane = reinterpret_cast<const T*>(stage + v * SH::PLANE);
        const int at = (jj + 1 - cy_of(v)) * SH::Wb + (ii + TT::HALO - cx_of(v));
        // (ii + HALO) is even: the pair of a direction with no x component is aligned
        r[v] = cx_of(v) == 0 ? PairIO<S>::load2(plane + at) : PairIO<S>::load11(plane + at);
        g[v] = S::SCALED ? r[v] * h16_scale(v) : r[v];
    }
    float Fxd = 0.0f, Fyd = 0.0f, Gxd = 0.0f, Gyd = 0.0f;
    if (FORCED) {
        force_xy_at_f(L, t, Fxd, Fyd);
        force_xy_at_f(L, t + 1, Gxd, Gyd);
    }
    const V2 dr = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) + g[8];
    const V2 rho = 1.0f + dr;
    const V2 mx = (g[1] - g[2]) + (g[5] - g[6]) + (g[7] - g[8]);
    const V2 my = (g[3] - g[4]) + (g[5] - g[6]) + (g[8] - g[7]);
    // rcp_lowp per lane (-rho is -1 - dr exactly)
    const V2 y0 = v2(rcp_approx(rho.x()), rcp_approx(rho.y()));
    const V2 inv = fmaf(y0, fmaf((-1.0f) - dr, y0, 1.0f), y0);
    const V2 px = FORCED ? fmaf(0.5f, Fxd, mx) : mx, py = FORCED ? fmaf(0.5f, Fyd, my) : my;
    const V2 ux = px * inv, uy = py * inv;
    V2 gs[9];
    collide_dev32<false, FORCED, S::SCALED>(g, r, dr, rho, mx, my, ux, uy, px, py, inv, Gxd, Gyd, L.omega_f, gs);
    T* out = B + (size_t)j * L.pitch + i;
#pragma unroll
    for (int v = 0; v < 9; v++) PairIO<S>::store2(out + (size_t)v * L.S, gs[v]);
}

// The last CTA of a launch to finish clears the tile counters for the next
// launch (called once by every persistent CTA, after its last tile).
__device__ __forceinline__ void step_tma_done(int* ctr, int ncta) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctr[1], 1) == ncta - 1) {
            ctr[0] = 0;
            ctr[1] = 0;
            __threadfence();
        }
    }
}

// BGK tiles with a pipeline per warp instead of CTA barriers: the warps
// share each tile's site pairs (two sites per lane per pass). Stage s has a
// "full" mbarrier (the producer's arrival with the copies' byte count, or a
// plain arrival with tile -1 when the counter is exhausted) and an "empty"
// mbarrier that every warp arrives on when it has read the stage. Thread 0 is
// also the producer: before computing tile k it refills the stage of tile
// k-1 with tile k+NST-1 once all warps have released it. A warp therefore
// waits only for its own data and, through the producer, for the slowest
// warp two tiles back, not for every warp at every tile.
template <class S>
__device__ __forceinline__ void tma_tiles_by_warp(const CUtensorMap& tm, typename S::T* __restrict__ B,
                                                  const LatDev& L, int t, int tiles_x, int ntiles,
                                                  unsigned char* smem) {
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    constexpr int NST = SH::NST, NW = 8;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * SH::STAGE);
    uint64_t* empty = full + NST;
    int* s_tile = reinterpret_cast<int*>(empty + NST);  // tile held by each stage, or -1
    int& s_err = s_tile[NST];
    int* ctr = L.tile_ctr;
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int q = 0; q < NST; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], NW);
        }
        s_err = 0;
        mbar_fence_init();
    }
    __syncthreads();
    // producer state (thread 0): stage fills so far, whether tiles ran out
    int fills[NST] = {0};
    bool out = false;
    auto fill = [&](int st) {
        const int tile = atomicAdd(&ctr[0], 1);
        s_tile[st] = tile < ntiles ? tile : -1;
        fills[st]++;
        if (tile < ntiles) {
            const int i0 = (tile % tiles_x) * TT::W, j0 = 1 + (tile / tiles_x) * TT::H;
            mbar_arrive_expect_tx(&full[st], 9u * SH::BOX);
            tma_load_3d(smem + st * SH::STAGE, &tm, i0 - TT::HALO, j0 - 1, 0, &full[st]);
        } else {
            out = true;
            mbar_arrive(&full[st]);
        }
    };
    if (threadIdx.x == 0)
        for (int q = 0; q < NST - 1 && !out; q++) fill(q);
    const bool forced = lattice_forced(L);
    for (int k = 0;; k++) {
        const int st = k % NST;
        if (threadIdx.x == 0 && !out) {
            const int kp = k + NST - 1, sp = kp % NST;
            // the stage's previous tile (kp - NST) must be released by all warps
            if (kp < NST || mbar_wait_bounded(&empty[sp], (unsigned)(kp / NST - 1) & 1u, 1u << 22)) {
                fence_proxy_async_smem();
                fill(sp);
            } else {
                atomicAdd(&g_tma_timeouts, 1);
                s_err = 1;
                out = true;
            }
        }
        if (!mbar_wait_bounded(&full[st], (unsigned)(k / NST) & 1u, 1u << 22)) {
            if (lane == 0) atomicAdd(&g_tma_timeouts, 1);
            break;
        }
        const int tile = s_tile[st];
        if (tile < 0 || *(volatile int*)&s_err) break;
        const int i0 = (tile % tiles_x) * TT::W, j0 = 1 + (tile / tiles_x) * TT::H;
        // pair p of the tile: row p / 64, columns 2 (p % 64) and the next
        for (int p = warp * 32 + lane; p < TT::H * (TT::W / 2); p += NW * 32) {
            if (forced) tma_pair<true, S>(smem + st * SH::STAGE, B, L, t, i0, j0, p / (TT::W / 2), 2 * (p % (TT::W / 2)));
            else tma_pair<false, S>(smem + st * SH::STAGE, B, L, t, i0, j0, p / (TT::W / 2), 2 * (p % (TT::W / 2)));
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
    }
    __syncthreads();
    // copies still in flight (after a timeout) land before the CTA leaves
    if (threadIdx.x == 0)
        for (int q = 0; q < NST; q++)
            if (fills[q] > 0) mbar_wait_bounded(&full[q], (unsigned)(fills[q] - 1) & 1u, 1u << 22);
}

template <bool CM, class S>
__global__ void __launch_bounds__(256, TmaTile<S>::CTAS) k_step_tma(const __grid_constant__ CUtensorMap tm,
                                                  const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                                  LatDev L, int t, int pb, int tiles_x, int ntiles) {
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    constexpr int NST = SH::NST;
    t = step_t(L, t);
    if ((int)blockIdx.x < pb) {
        // boundary-condition sites; an edge site of a periodic wall is an
        // interior site with wrapped neighbours (each call skips the other kind)
        const int q = blockIdx.x * blockDim.x + threadIdx.x;
        perimeter_site_call<CM, S>(A, B, L, t, q);
        int i, j;
        if (perimeter_ij(L, q, i, j)) interior_site_lowp<CM, S, false>(A, B, L, t, i, j);
        return;
    }
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                           ~static_cast<uintptr_t>(127));
    const int ncta = (int)gridDim.x - pb;
    int* ctr = L.tile_ctr;  // [0]: tiles handed out, [1]: CTAs finished
    if constexpr (!CM) {
        tma_tiles_by_warp<S>(tm, B, L, t, tiles_x, ntiles, smem);
        step_tma_done(ctr, ncta);
        return;
    }
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + NST * SH::STAGE);
    int* s_tile = reinterpret_cast<int*>(smem + NST * SH::STAGE + 8 * NST);  // tile held by each stage, or -1
    int& s_ok = s_tile[NST];
    if (threadIdx.x == 0) {
        for (int q = 0; q < NST; q++) mbar_init(&bar[q], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int tile, int st) {
        const int i0 = (tile % tiles_x) * TT::W, j0 = 1 + (tile / tiles_x) * TT::H;
        mbar_arrive_expect_tx(&bar[st], 9u * SH::BOX);
        tma_load_3d(smem + st * SH::STAGE, &tm, i0 - TT::HALO, j0 - 1, 0, &bar[st]);
    };
    // Tiles are handed out by a counter, so CTAs that start late (behind the
    // boundary blocks) take fewer tiles and the step ends evenly. The stage of
    // tile k+NST-1 is filled while tile k is computed; it is the stage tile
    // k-1 used. The results do not depend on which CTA takes which tile.
    auto grab = [&](int st) {
        const int tile = atomicAdd(&ctr[0], 1);
        s_tile[st] = tile < ntiles ? tile : -1;
        if (tile < ntiles) issue(tile, st);
    };
    if (threadIdx.x == 0)
        for (int q = 0; q < NST - 1; q++) grab(q);
    const bool forced = lattice_forced(L);
    for (int k = 0;; k++) {
        const int st = k % NST;
        if (threadIdx.x == 0) {
            fence_proxy_async_smem();
            grab((k + NST - 1) % NST);
            s_ok = 1;
            if (s_tile[st] >= 0 && !mbar_wait_bounded(&bar[st], (unsigned)(k / NST) & 1u, 1u << 22)) {
                // give the copies in flight into the other stages time to land
                // before the CTA (and its shared memory) goes away
                for (int q = 1; q < NST; q++)
                    if (s_tile[(k + q) % NST] >= 0)
                        mbar_wait_bounded(&bar[(k + q) % NST], (unsigned)((k + q) / NST) & 1u, 1u << 22);
                atomicAdd(&g_tma_timeouts, 1);
                s_ok = 0;
            }
        }
        __syncthreads();
        const int tile = s_tile[st];
        if (tile < 0 || !s_ok) break;
        const int i0 = (tile % tiles_x) * TT::W, j0 = 1 + (tile / tiles_x) * TT::H;
        if (forced) tma_tile_sites<CM, true, S>(smem + st * SH::STAGE, B, L, t, i0, j0);
        else tma_tile_sites<CM, false, S>(smem + st * SH::STAGE, B, L, t, i0, j0);
        __syncthreads();
    }
    step_tma_done(ctr, ncta);
}

// The tensor map of one population buffer: dims (pitch, Ny, 9 planes), box
// (Wb, Hb, 1), no swizzle, zero fill outside the buffer.
template <class S>
static cudaError_t plane_tensor_map(CUtensorMap* tm, const void* base, const LatDev& L) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    const cuuint64_t dims[3] = {(cuuint64_t)L.pitch, (cuuint64_t)L.Ny, 9};
    const cuuint64_t strides[2] = {(cuuint64_t)L.pitch * TT::ELEM, (cuuint64_t)L.S * TT::ELEM};
    const cuuint32_t box[3] = {(cuuint32_t)SH::Wb, (cuuint32_t)SH::Hb, 9};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(tm, TT::DTYPE, 3, const_cast<void*>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <bool CM, class S>
static cudaError_t launch_step_tma_t(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    using TT = TmaTile<S>;
    using SH = TmaShape<S>;
    static int per_sm[64] = {0}, sms[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!per_sm[dev]) {
        e = cudaFuncSetAttribute(k_step_tma<CM, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, SH::SMEM);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[dev], k_step_tma<CM, S>, 256, SH::SMEM);
        if (e != cudaSuccess) return e;
        if (per_sm[dev] < 1) per_sm[dev] = 1;
    }
    CUtensorMap tm;
    if ((e = plane_tensor_map<S>(&tm, A, L)) != cudaSuccess) return e;
    const int n = 2 * L.Nx + 2 * (L.Ny - 2);
    const int pb = (n + 255) / 256;
    const int tiles_x = (L.Nx - 1 + TT::W - 1) / TT::W, tiles_y = (L.Ny - 2 + TT::H - 1) / TT::H;
    const int ntiles = tiles_x * tiles_y;
    const int persistent = std::min(ntiles, sms[dev] * per_sm[dev]);
    k_step_tma<CM, S><<<pb + std::max(persistent, 1), 256, SH::SMEM, s>>>(
        tm, (const typename S::T*)A, (typename S::T*)B, L, t, pb, tiles_x, ntiles);
    return cudaGetLastError();
}

int tma_timeouts() {
    int h = 0;
    if (cudaMemcpyFromSymbol(&h, g_tma_timeouts, sizeof h) != cudaSuccess) return -1;
    return h;
}

// Which step kernel a reduced-precision case uses: the TMA-staged tiles
// (k_step_tma) for both storage forms; the one-site kernel (k_step_lowp) is
// kept for comparison. Measured at 4096^2: FP16 95.6-99.6k (one-site) against
// 159k MLUPS (staged), FP32 85.8-86.3k against 90.2-90.9k.
// LIFE_STEP_KERNEL=site|tma overrides, for measurements and for the tests
// that compare the two bit for bit.
enum { STEP_SITE = 1, STEP_TMA = 3 };
static int step_kernel(int prec) {
    static int forced = -1;
    if (forced < 0) {
        const char* e = getenv("LIFE_STEP_KERNEL");
        forced = 0;
        if (e && !strcmp(e, "site")) forced = STEP_SITE;
        else if (e && !strcmp(e, "tma")) forced = STEP_TMA;
    }
    if (forced) return forced;
    (void)prec;
    return STEP_TMA;
}

cudaError_t launch_step_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    const int kind = step_kernel(L.prec);
    if (kind == STEP_TMA) {
        if (L.prec == LIFE_PREC_F32)
            return L.cm ? launch_step_tma_t<true, StoreF32>(A, B, L, t, s) : launch_step_tma_t<false, StoreF32>(A, B, L, t, s);
        return L.cm ? launch_step_tma_t<true, StoreF16>(A, B, L, t, s) : launch_step_tma_t<false, StoreF16>(A, B, L, t, s);
    }

    const int n = 2 * L.Nx + 2 * (L.Ny - 2);
    const int pb = (n + 255) / 256, bx = (L.Nx + 255) / 256;
    const unsigned grid = (unsigned)(pb + bx * L.Ny);
    // m = floor(2^32 / bx) + 1 gives floor(b / bx) = umulhi(b, m) exactly
    // when b (m bx - 2^32) < 2^32 for the largest b; else divide
    const unsigned long long m = (1ull << 32) / (unsigned long long)bx + 1ull;
    const unsigned long long bmax = (unsigned long long)bx * (unsigned long long)L.Ny;
    const unsigned bx_m = (m < (1ull << 32) && bmax * (m * (unsigned long long)bx - (1ull << 32)) < (1ull << 32))
                              ? (unsigned)m : 0u;
    if (L.prec == LIFE_PREC_F32) {
        if (L.cm) k_step_lowp<true, StoreF32><<<grid, 256, 0, s>>>((const float*)A, (float*)B, L, t, pb, bx, bx_m);
        else k_step_lowp<false, StoreF32><<<grid, 256, 0, s>>>((const float*)A, (float*)B, L, t, pb, bx, bx_m);
    } else {
        if (L.cm) k_step_lowp<true, StoreF16><<<grid, 256, 0, s>>>((const __half*)A, (__half*)B, L, t, pb, bx, bx_m);
        else k_step_lowp<false, StoreF16><<<grid, 256, 0, s>>>((const __half*)A, (__half*)B, L, t, pb, bx, bx_m);
    }
    return cudaGetLastError();
}

cudaError_t launch_interior_batch_lowp(int prec, const BatchLatCase* cases, const int* tile_case, int ntiles,
                                       int tile_w, int tile_h, int grid, int phase, cudaStream_t s) {
    if (prec == LIFE_PREC_F32)
        k_interior_batch_lowp<StoreF32><<<grid, tile_w, 0, s>>>(cases, tile_case, ntiles, tile_h, phase);
    else
        k_interior_batch_lowp<StoreF16><<<grid, tile_w, 0, s>>>(cases, tile_case, ntiles, tile_h, phase);
    return cudaGetLastError();
}

int batch_blocks_per_sm_lowp(int prec, int tile_w) {
    int n = 0;
    if (prec == LIFE_PREC_F32)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_interior_batch_lowp<StoreF32>, tile_w, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_interior_batch_lowp<StoreF16>, tile_w, 0);
    return n;
}

}  // namespace life
