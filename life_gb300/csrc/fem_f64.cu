// Flexible-body kernels (FP64, --fmad=false, reference operation order).
//
// One CTA per flexible body runs the FEM work of that body:
//   k_fsi_predict   predictor (first subiteration) or Aitken relaxation,
//                   then updateFEMValues / finishNewmark / updateIBMValues
//                   (FEMBodyClass::predictor, src/FEMBody.cpp:259-289;
//                   ObjectsClass::recomputeObjectVals, src/Objects.cpp:152-232)
//   k_fem_dynamic   FEMBodyClass::dynamicFEM (src/FEMBody.cpp:26-68): load
//                   vector, Newton-Raphson with Newmark and the dense LU solve,
//                   marker update, subiteration residual
// and
//   k_fsi_support   findSupport + computeDs of flexible markers
//   k_fsi_epsilon   epsilon systems (per flexible body or all markers)
//   k_fsi_residual  femKernel's ordered residual sums, the loop condition and
//                   the next Aitken factor (src/Objects.cpp:63-99, 179-190)
//
// Element matrices are computed in parallel and assembled entry by entry in
// element order, the order of the reference's sequential assembly. Products
// with the element rotation T skip its structural zeros; a skipped term is an
// exact zero, so results are unchanged.
#include <cuda_runtime.h>

#include <atomic>

#include "band_lu.h"
#include "crtrig.h"
#include "div_rn.cuh"
#include "fem_kernels.h"

namespace life {

#define DSQ(x) ((x) * (x))
#define DTH(x) ((x) * (x) * (x))
__device__ constexpr double kPI = 3.14159265358979323846;

__device__ __forceinline__ double* vec(FemBodyDev& B, int name) { return B.pool + (size_t)B.slots[name] * B.n; }

__device__ __forceinline__ double shift_angle_d(double a) {
    a = fmod(a + kPI, 2.0 * kPI);
    if (a < 0.0) a += 2.0 * kPI;
    return a - kPI;
}

__device__ __forceinline__ double dirac_d(double dist) {
    double a = fabs(dist);
    if (a > 1.5) return 0.0;
    if (a > 0.5) return (5.0 - 3.0 * a - sqrt(-3.0 * DSQ(1.0 - a) + 1.0)) / 6.0;
    return (1.0 + sqrt(1.0 - 3.0 * DSQ(a))) / 3.0;
}

// Element rotation T = diag(R, R), R = [[c, s, 0], [-s, c, 0], [0, 0, 1]]
// (FEMElementClass::setElementTransform, src/FEMElement.cpp:255-262).
__host__ __device__ constexpr bool tnz(int i, int j) {
    return (i < 2 && j < 2) || (i == 2 && j == 2) || (i >= 3 && i < 5 && j >= 3 && j < 5) || (i == 5 && j == 5);
}
__device__ __forceinline__ double tval(int i, int j, double c, double s) {
    const int a = i % 3, b = j % 3;
    if (a == 2) return 1.0;
    if (a == 0) return b == 0 ? c : s;
    return b == 0 ? -s : c;
}

// out = T^T A T with the reference's summation order over non-zero terms.
__device__ __forceinline__ void tt_a_t(const double* A, double c, double s, double* out) {
    double R1[36];
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (tnz(k, i)) acc += tval(k, i, c, s) * A[k * 6 + j];
            R1[i * 6 + j] = acc;
        }
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (tnz(k, j)) acc += R1[i * 6 + k] * tval(k, j, c, s);
            out[i * 6 + j] = acc;
        }
}

// FEMBodyClass::updateFEMValues (src/FEMBody.cpp:198-223)
__device__ void update_fem_values(FemBodyDev& B) {
    const double* U = vec(B, V_U);
    for (int n = threadIdx.x; n < B.nNodes; n += blockDim.x) {
        double* nd = B.node + n * 6;
        nd[2] = nd[0] + U[n * 3 + 0];
        nd[3] = nd[1] + U[n * 3 + 1];
        nd[5] = nd[4] + U[n * 3 + 2];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < B.nEl; e += blockDim.x) {
        const double* n0 = B.node + e * 6;
        const double* n1 = B.node + (e + 1) * 6;
        const double ev0 = n1[2] - n0[2], ev1 = n1[3] - n0[3];
        double* el = B.el + (size_t)e * EL_STRIDE;
        // correctly rounded trigonometry (crtrig.h): the same bits on every
        // device and on a host checker
        const double ang = life_cr_atan2(ev1, ev0);
        double dd = 0.0;
        dd += ev0 * ev0;
        dd += ev1 * ev1;
        el[EL_ANG] = ang;
        el[EL_L] = sqrt(dd);
        double sa, ca;
        life_cr_sincos(ang, &sa, &ca);
        el[EL_COS] = ca;
        el[EL_SIN] = sa;
    }
    __syncthreads();
}

// FEMBodyClass::finishNewmark (src/FEMBody.cpp:129-144)
__device__ void finish_newmark(FemBodyDev& B, const FsiDev& F) {
    const double Dt = F.Dt, al = F.alpha, de = F.delta;
    const double a6 = 1.0 / (al * DSQ(Dt)), a7 = -1.0 / (al * Dt), a8 = -(1.0 / (2.0 * al) - 1.0);
    const double a9 = Dt * (1.0 - de), a10 = de * Dt;
    double* U = vec(B, V_U);
    double* Un = vec(B, V_Un);
    double* Ud = vec(B, V_Udot);
    double* Udd = vec(B, V_Udotdot);
    double* Udn = vec(B, V_Udotn);
    double* Uddn = vec(B, V_Udotdotn);
    for (int i = threadIdx.x; i < B.n; i += blockDim.x) {
        const double udd = a6 * (U[i] - Un[i]) + a7 * Udn[i] + a8 * Uddn[i];
        Udd[i] = udd;
        Ud[i] = Udn[i] + a9 * Uddn[i] + a10 * udd;
    }
    __syncthreads();
}

// FEMElementClass::shapeFuns (src/FEMElement.cpp:141-160)
__device__ __forceinline__ void shape_funs_d(double res[2], const double v[6], double zeta, double L) {
    const double N0 = 1.0 - (zeta + 1.0) / 2.0;
    const double N1 = 1.0 - 3.0 * DSQ((zeta + 1.0) / 2.0) + 2.0 * DTH((zeta + 1.0) / 2.0);
    const double N2 = ((zeta + 1.0) / 2.0 - 2.0 * DSQ((zeta + 1.0) / 2.0) + DTH((zeta + 1.0) / 2.0)) * L;
    const double N3 = (zeta + 1.0) / 2.0;
    const double N4 = 3.0 * DSQ((zeta + 1.0) / 2.0) - 2.0 * DTH((zeta + 1.0) / 2.0);
    const double N5 = (-DSQ((zeta + 1.0) / 2.0) + DTH((zeta + 1.0) / 2.0)) * L;
    res[0] = v[0] * N0 + v[3] * N3;
    res[1] = v[1] * N1 + v[2] * N2 + v[4] * N4 + v[5] * N5;
}

// T * v over non-zero entries of T.
__device__ __forceinline__ void t_vec(const double v[6], double c, double s, double out[6]) {
#pragma unroll
    for (int i = 0; i < 6; i++) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j++)
            if (tnz(i, j)) acc += tval(i, j, c, s) * v[j];
        out[i] = acc;
    }
}
// T^T * v over non-zero entries of T.
__device__ __forceinline__ void tt_vec(const double v[6], double c, double s, double out[6]) {
#pragma unroll
    for (int i = 0; i < 6; i++) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j++)
            if (tnz(j, i)) acc += tval(j, i, c, s) * v[j];
        out[i] = acc;
    }
}

// FEMBodyClass::updateIBMValues (src/FEMBody.cpp:147-195)
__device__ void update_ibm(FemBodyDev& B, const MarkerDev& M) {
    const double* U = vec(B, V_U);
    const double* Ud = vec(B, V_Udot);
    for (int i = threadIdx.x; i < B.nMark; i += blockDim.x) {
        const int e = B.mapEl[i];
        const double zeta = B.mapZeta[i];
        const double* el = B.el + (size_t)e * EL_STRIDE;
        const double c = el[EL_COS], s = el[EL_SIN], ang = el[EL_ANG], L = el[EL_L];
        double dU[6], dUd[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            dU[k] = U[3 * e + k];
            dUd[k] = Ud[3 * e + k];
        }
        const double* nd0 = B.node + e * 6;
#pragma unroll
        for (int n = 0; n < 2; n++) {
            const double* nd = B.node + (e + n) * 6;
            dU[n * 3 + 0] += nd[0] - nd0[2];
            dU[n * 3 + 1] += nd[1] - nd0[3];
            dU[n * 3 + 2] += nd[4] - ang;
            dU[n * 3 + 2] = shift_angle_d(dU[n * 3 + 2]);
        }
        double lU[6], lUd[6], sU[2], sUd[2];
        t_vec(dU, c, s, lU);
        t_vec(dUd, c, s, lUd);
        shape_funs_d(sU, lU, zeta, L);
        shape_funs_d(sUd, lUd, zeta, L);
        const double gU0 = (0.0 + c * sU[0]) + (-s) * sU[1];
        const double gU1 = (0.0 + s * sU[0]) + c * sU[1];
        const double gV0 = (0.0 + c * sUd[0]) + (-s) * sUd[1];
        const double gV1 = (0.0 + s * sUd[0]) + c * sUd[1];
        const int k = B.mbase + i;
        M.pos[k * 2 + 0] = nd0[2] + gU0;
        M.pos[k * 2 + 1] = nd0[3] + gU1;
        M.vel[k * 2 + 0] = gV0;
        M.vel[k * 2 + 1] = gV1;
    }
    __syncthreads();
}

__device__ __forceinline__ void swap_slots(FemBodyDev& B, int a, int b) {
    const int t = B.slots[a];
    B.slots[a] = B.slots[b];
    B.slots[b] = t;
}

// Predictor (subiteration 0) or relaxation (later subiterations).
__global__ void __launch_bounds__(256) k_fsi_predict(FsiDev F, MarkerDev M) {
    FemBodyDev& B = F.bodies[blockIdx.x];
    const int subIt = F.s->subIt;
    const int t = F.s->t;
    if (subIt == 0) {
        if (threadIdx.x == 0) {
            // FEMBodyClass::resetValues (src/FEMBody.cpp:341-349)
            swap_slots(B, V_Unm2, V_Unm1);
            swap_slots(B, V_Unm1, V_Un);
            swap_slots(B, V_Un, V_U);
            swap_slots(B, V_Udotn, V_Udot);
            swap_slots(B, V_Udotdotn, V_Udotdot);
        }
        __syncthreads();
        double* U = vec(B, V_U);
        const double* Un = vec(B, V_Un);
        const double* Unm1 = vec(B, V_Unm1);
        const double* Unm2 = vec(B, V_Unm2);
        for (int i = threadIdx.x; i < B.n; i += blockDim.x) {
            if (t > 2) U[i] = 2.5 * Un[i] - 2.0 * Unm1[i] + 0.5 * Unm2[i];
            else if (t == 2) U[i] = 2.0 * Un[i] - Unm1[i];
            else if (t == 1) U[i] = Un[i];
        }
    } else {
        const double relax = F.s->relax;
        double* U = vec(B, V_U);
        const double* Uk = vec(B, V_Ukm1);
        for (int i = threadIdx.x; i < B.n; i += blockDim.x) U[i] = Uk[i] + relax * (U[i] - Uk[i]);
    }
    __syncthreads();
    update_fem_values(B);
    finish_newmark(B, F);
    update_ibm(B, M);
    if (threadIdx.x == 0) swap_slots(B, V_Ukm1, V_U);
}

// IBMNodeClass::findSupport + computeDs (src/IBMNode.cpp:139-204) for the
// markers of flexible bodies, one warp per marker. Lanes 0..24 test the 5 x 5
// lattice nodes around the nearest node, lane = 5*(i - inear + 2) + (j -
// jnear + 2), so the ballot packs the supporting nodes in the reference's
// loop order (i outer, j inner). The spacing ds is the minimum of sqrt(dd)/Dx
// over the body's other markers; correctly rounded sqrt and division are
// monotone, so it equals sqrt(min dd)/Dx, and the lanes only reduce dd.
__global__ void __launch_bounds__(128) k_fsi_support(FsiDev F, MarkerDev M) {
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= F.nFlexMarkers) return;  // uniform per warp
    const int k = F.flexMarkers[q];
    const double Dx = F.Dx;
    const double px = M.pos[k * 2], py = M.pos[k * 2 + 1];
    const double sx = px / Dx, sy = py / Dx;
    const int inear = (int)round(sx), jnear = (int)round(sy);
    const int i = inear - 2 + lane / 5, j = jnear - 2 + lane % 5;
    double dX = 0.0, dY = 0.0;
    bool in = false;
    if (lane < 25) {
        dX = fabs(sx - i);
        dY = fabs(sy - j);
        in = dX < 1.5 && dY < 1.5 && i >= 0 && i <= F.Nx - 1 && j >= 0 && j <= F.Ny - 1;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    const int slot = __popc(bal & ((1u << lane) - 1u));
    const int total = __popc(bal);
    if (lane < 9) {
        M.si[k * 9 + lane] = 0;
        M.sj[k * 9 + lane] = 0;
        M.sd[k * 9 + lane] = 0.0;
    }
    __syncwarp();
    if (in && slot < 9) {
        M.si[k * 9 + slot] = i;
        M.sj[k * 9 + slot] = j;
        M.sd[k * 9 + slot] = dirac_d(dX) * dirac_d(dY);
    }
    if (lane == 0) {
        M.nsupp[k] = total < 9 ? total : 9;
        if (total > 9) atomicCAS(&F.status[0], 0, LIFE_ERR_SUPPORT);
    }
    const int b = F.markerBody[k];
    const int b0 = F.bodyStart[b], bn = F.bodyCount[b];
    // non-negative doubles order like their bit patterns; NaN never passes dd < best
    unsigned long long best = 0x7ff0000000000000ull;  // +inf
    for (int n = lane; n < bn; n += 32) {
        const int o = b0 + n;
        if (o != k) {
            const double d0 = px - M.pos[o * 2], d1 = py - M.pos[o * 2 + 1];
            double dd = 0.0;
            dd += d0 * d0;
            dd += d1 * d1;
            if (dd < __longlong_as_double((long long)best)) best = (unsigned long long)__double_as_longlong(dd);
        }
    }
    const unsigned bh = __reduce_min_sync(0xffffffffu, (unsigned)(best >> 32));
    const unsigned bl = __reduce_min_sync(0xffffffffu, (unsigned)(best >> 32) == bh ? (unsigned)best : 0xffffffffu);
    if (lane == 0) {
        const double mag = sqrt(__longlong_as_double((long long)(((unsigned long long)bh << 32) | bl))) / Dx;
        M.ds[k] = mag < 10.0 ? mag : 10.0;
    }
}

// Dense LU with band-limited loops (band_lu.h semantics) by one warp.
// M(i,j) = A[(bc+j)*dim + bc+i]. lmax[c] tracks the last row that can hold a
// multiplier of column c after row interchanges.
__device__ void warp_lu_factor(double* A, int dim, int bc, int kl, int ku, int* piv, int* lmax) {
    const int lane = threadIdx.x & 31;
    const int n = dim - bc;
    for (int c = lane; c < n; c += 32) lmax[c] = c;
    __syncwarp();
    for (int j = 0; j < n; j++) {
        const int imax = j + kl < n - 1 ? j + kl : n - 1;
        // first maximal |M(i,j)|, i in [j, imax] (LAPACK idamax semantics)
        int best = j;
        double bval = -1.0;
        for (int i0 = j; i0 <= imax; i0 += 32) {
            const int i = i0 + lane;
            double va = -1.0;
            int vi = i;
            if (i <= imax) va = fabs(lu_m(A, dim, bc, i, j));
            for (int o = 16; o > 0; o >>= 1) {
                const double oa = __shfl_down_sync(0xffffffffu, va, o);
                const int oi = __shfl_down_sync(0xffffffffu, vi, o);
                if (oa > va || (oa == va && oi < vi)) { va = oa; vi = oi; }
            }
            va = __shfl_sync(0xffffffffu, va, 0);
            vi = __shfl_sync(0xffffffffu, vi, 0);
            if (va > bval) { bval = va; best = vi; }
        }
        const int jp = best;
        if (lane == 0) piv[j] = jp;
        const double pv = lu_m(A, dim, bc, jp, j);
        if (pv != 0.0) {
            if (jp != j) {
                for (int k = lane; k < n; k += 32) {
                    const double tj = lu_m(A, dim, bc, j, k), tp = lu_m(A, dim, bc, jp, k);
                    if (k < j && tj != 0.0 && lmax[k] < jp) lmax[k] = jp;
                    lu_m(A, dim, bc, j, k) = tp;
                    lu_m(A, dim, bc, jp, k) = tj;
                }
                __syncwarp();
            }
            const double r = 1.0 / lu_m(A, dim, bc, j, j);
            for (int i = j + 1 + lane; i <= imax; i += 32) lu_m(A, dim, bc, i, j) *= r;
        }
        if (lane == 0 && lmax[j] < imax) lmax[j] = imax;
        __syncwarp();
        const int kmax = j + kl + ku < n - 1 ? j + kl + ku : n - 1;
        const int rows = imax - j, cols = kmax - j;
        for (int q = lane; q < rows * cols; q += 32) {
            const int i = j + 1 + q % rows, k = j + 1 + q / rows;
            const double t = -lu_m(A, dim, bc, j, k);
            lu_m(A, dim, bc, i, k) += lu_m(A, dim, bc, i, j) * t;
        }
        __syncwarp();
    }
}

// Transposed solve (lane 0); x has dim entries, the first bc zeroed.
__device__ void warp_lu_solve(const double* A_, int dim, int bc, int kl, int ku, const int* piv, const int* lmax,
                              const double* b, double* x) {
    const int lane = threadIdx.x & 31;
    double* A = const_cast<double*>(A_);
    const int n = dim - bc;
    for (int i = lane; i < bc; i += 32) x[i] = 0.0;
    for (int i = lane; i < n; i += 32) x[bc + i] = b[bc + i];
    __syncwarp();
    if (lane == 0) {
        double* y = x + bc;
        const int w = kl + ku;
        for (int i = 0; i < n; i++) {
            double t = y[i];
            for (int k = (i - w > 0 ? i - w : 0); k < i; k++) t -= lu_m(A, dim, bc, k, i) * y[k];
            y[i] = t / lu_m(A, dim, bc, i, i);
        }
        for (int i = n - 1; i >= 0; i--) {
            double t = y[i];
            const int kend = lmax[i];
            for (int k = i + 1; k <= kend; k++) t -= lu_m(A, dim, bc, k, i) * y[k];
            y[i] = t;
        }
        for (int i = n - 1; i >= 0; i--)
            if (piv[i] != i) {
                const double t = y[i];
                y[i] = y[piv[i]];
                y[piv[i]] = t;
            }
    }
    __syncwarp();
}


// ---------------------------------------------------------------------------
// Band LU in shared memory with the dense textbook arithmetic.
//
// M is nn x nn with kl sub- and ku super-diagonals; row i of Bd holds M(i, c)
// for c in [i-kl, i+kl+ku] at Bd[i*W + c - i + kl], W = 2*kl + ku + 1. The
// factorisation performs exactly the operations of the dense unblocked LU
// (first maximal pivot, reciprocal scaling, rank-1 update; band_lu.h), but
// like LAPACK's banded routine it does not move the multipliers of earlier
// columns when it swaps rows. The dense transposed solve reads each
// multiplier from the row where the later swaps would have carried it; the
// solve below follows each multiplier to that final row (Fp, updated swap by
// swap from the last step back), so it forms the same products and sums
// them in the same order as the dense solve. Results are bit-identical.
__device__ __forceinline__ double& bd(double* Bd, int W, int kl, int i, int c) { return Bd[i * W + c - i + kl]; }

// One warp; kl <= 31. Lane l holds the candidate M(j+l, j) of column j. The
// pivot is the first maximal magnitude (LAPACK idamax: a NaN in the first
// place wins, later NaNs never do); magnitudes are compared as bit patterns,
// which order like the values for non-negative doubles. Each candidate's
// reciprocal is formed while the pivot is being chosen and the pivot's is
// kept: the same correctly rounded 1/pivot as a division after the choice.
__device__ void band_factor_smem(double* Bd, int nn, int kl, int ku, int W, int* piv) {
    const int lane = threadIdx.x & 31;
    for (int j = 0; j < nn; j++) {
        const int imax = j + kl < nn - 1 ? j + kl : nn - 1;
        const int kmax = j + kl + ku < nn - 1 ? j + kl + ku : nn - 1;
        const bool valid = j + lane <= imax;
        const double v = valid ? bd(Bd, W, kl, j + lane, j) : 0.0;
        const double rc = 1.0 / v;
        unsigned long long key = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
        if (key > 0x7ff0000000000000ull) key = lane == 0 ? ~0ull : 0ull;
        const unsigned kh = (unsigned)(key >> 32), klo = (unsigned)key;
        const unsigned mh = __reduce_max_sync(0xffffffffu, valid ? kh : 0u);
        const bool c1 = valid && kh == mh;
        const unsigned ml = __reduce_max_sync(0xffffffffu, c1 ? klo : 0u);
        const int src = __ffs(__ballot_sync(0xffffffffu, c1 && klo == ml)) - 1;
        const int jp = j + src;
        const double pv = __shfl_sync(0xffffffffu, v, src);
        const double r = __shfl_sync(0xffffffffu, rc, src);
        if (lane == 0) piv[j] = jp;
        if (pv != 0.0) {
            if (jp != j) {
                for (int c = j + lane; c <= kmax; c += 32) {
                    const double t = bd(Bd, W, kl, j, c);
                    bd(Bd, W, kl, j, c) = bd(Bd, W, kl, jp, c);
                    bd(Bd, W, kl, jp, c) = t;
                }
                __syncwarp();
            }
            for (int i = j + 1 + lane; i <= imax; i += 32) bd(Bd, W, kl, i, j) *= r;
        }
        __syncwarp();
        const int rows = imax - j, cols = kmax - j;
        for (int q = lane; q < rows * cols; q += 32) {
            const int i = j + 1 + q % rows, k = j + 1 + q / rows;
            const double t = -bd(Bd, W, kl, j, k);
            bd(Bd, W, kl, i, k) += bd(Bd, W, kl, i, j) * t;
        }
        __syncwarp();
    }
}

__global__ void k_selftest_division(long long n, unsigned long long seed, unsigned long long* bad) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        // splitmix64 streams for the two operands; exponents over a wide range
        unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(2 * q + 1);
        auto mix = [](unsigned long long x) {
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
            return x ^ (x >> 31);
        };
        const unsigned long long u = mix(z), v = mix(z + 0x9e3779b97f4a7c15ull);
        const unsigned long long w = mix(z ^ 0x5851f42d4c957f2dull);
        // exponent spread: mostly near 1, sometimes anywhere in the normal range
        const int span = (w & 7) == 0 ? 2000 : 80;
        const long long xa = (long long)(1023 + (long long)((w >> 8) % span) - span / 2);
        const long long xb = (long long)(1023 + (long long)((w >> 24) % span) - span / 2);
        const unsigned long long ba = (u & 0x800fffffffffffffull) | ((unsigned long long)(xa < 1 ? 1 : (xa > 2046 ? 2046 : xa)) << 52);
        const unsigned long long bb = (v & 0x800fffffffffffffull) | ((unsigned long long)(xb < 1 ? 1 : (xb > 2046 ? 2046 : xb)) << 52);
        // one numerator in 64 is a signed zero (the velocity of a site at rest)
        const double a = ((w >> 40) & 63) == 0 ? __longlong_as_double((long long)(u & 0x8000000000000000ull))
                                                : __longlong_as_double((long long)ba);
        const double b = __longlong_as_double((long long)bb);
        const double ref = a / b;
        const double got = div_rn_recip(a, b, __drcp_rn(b));
        if (__double_as_longlong(ref) != __double_as_longlong(got) && !(ref != ref && got != got)) atomicAdd(bad, 1ull);
    }
}

__device__ __forceinline__ void named_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// First maximal |v| over the lanes with `valid` (LAPACK idamax: a NaN in
// lane 0 wins, later NaNs never do), as the lane index. Magnitudes are
// compared as bit patterns, which order like the values for non-negative
// doubles. Whole warp.
__device__ __forceinline__ int pick_pivot(double v, bool valid, int lane) {
    unsigned long long key = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    if (key > 0x7ff0000000000000ull) key = lane == 0 ? ~0ull : 0ull;
    const unsigned kh = (unsigned)(key >> 32), klo = (unsigned)key;
    const unsigned mh = __reduce_max_sync(0xffffffffu, valid ? kh : 0u);
    const bool c1 = valid && kh == mh;
    const unsigned ml = __reduce_max_sync(0xffffffffu, c1 ? klo : 0u);
    return __ffs(__ballot_sync(0xffffffffu, c1 && klo == ml)) - 1;
}

// Band LU of M and the forward half of the transposed solve (U^T y = b, y in
// place), pipelined over warps 0-3 of the CTA; kl <= 31 and kl + ku <= 31.
// The operations are those of band_factor_smem followed by the row-ordered
// forward substitution; only who does them, and when, differs. The critical
// path is warp 0's chain per column: reciprocal of the pivot, multipliers,
// update of the next column's candidates. Everything else runs beside it:
//   warp 0: step j's row swap, the scaling and the step-j update of column
//           j+1, barrier 1, then the reciprocals of column j+1's candidates
//           (each lane its own; the pivot's is kept, the same correctly
//           rounded 1/pivot as a division after the choice). Column j+1's
//           candidates are already in its registers (the rows it just
//           updated, plus one row no earlier step touched);
//   warp 3: after barrier 1, the choice of column j+1's pivot from the same
//           candidates, which are final in shared memory by then, handed to
//           warp 0 in s_src through barrier 2;
//   warps 1, 3: after barrier 1, the step-j update of columns j+2..kmax,
//           split between them, then barrier 2 (which warp 0 waits on before
//           the swap of step j+1, the first thing to touch those rows again);
//   warp 2: after barrier 1, forward row j (row j of U is final once the swap
//           of step j is done): y_j = t_j / U(j,j) and every row r in
//           (j, j+kl+ku] subtracts U(j,r) y_j. Each row still subtracts its
//           terms in ascending order, so every sum is formed as before.
// Barrier counts: warp 0 calls barrier 1 nn times and barrier 2 nn-1 times
// (before each swap after the first); warps 1 and 3 call barrier 1 nn times
// and barrier 2 after every step but the last; warp 2 calls barrier 1 nn
// times. The k-th calls pair up, so every barrier completes. Needs at least
// 128 threads; with fewer, warp 0 does everything.
__device__ void band_lu_forward(double* Bd, int nn, int kl, int ku, int W, int* piv, double* y, double* rcp) {
    __shared__ int s_src;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (blockDim.x < 128) {
        if (warp == 0) {
            band_factor_smem(Bd, nn, kl, ku, W, piv);
            if (lane == 0)
                for (int i = 0; i < nn; i++) {
                    double t = y[i];
                    for (int k = (i - kl - ku > 0 ? i - kl - ku : 0); k < i; k++) t -= bd(Bd, W, kl, k, i) * y[k];
                    y[i] = t / bd(Bd, W, kl, i, i);
                }
            __syncwarp();
        }
        return;
    }
    if (warp == 0) {
        // lane l holds the pivot candidate M(j+l, j) and its reciprocal
        const int imax0 = kl < nn - 1 ? kl : nn - 1;
        double v = lane <= imax0 ? bd(Bd, W, kl, lane, 0) : 0.0;
        double rc = __drcp_rn(v);
        int src = pick_pivot(v, lane <= imax0, lane);
        for (int j = 0; j < nn; j++) {
            const int imax = j + kl < nn - 1 ? j + kl : nn - 1;
            const int kmax = j + kl + ku < nn - 1 ? j + kl + ku : nn - 1;
            if (j > 0) {
                named_bar(2, 96);
                src = s_src;
            }
            const int jp = j + src;
            const double pv = __shfl_sync(0xffffffffu, v, src);
            const double v0 = __shfl_sync(0xffffffffu, v, 0);
            if (lane == 0) piv[j] = jp;
            // pivot != 0 (NaN counts as non-zero), tested on the bits
            const bool nz = ((unsigned long long)__double_as_longlong(pv) << 1) != 0ull;
            const bool swapped = nz && jp != j;
            const int c = j + lane;
            double rj = 0.0, rp = 0.0;
            if (c <= kmax) {
                rj = bd(Bd, W, kl, j, c);
                rp = bd(Bd, W, kl, jp, c);
            }
            const bool mrow = lane >= 1 && j + lane <= imax;  // multiplier row i = j + lane
            const bool early = j + 1 <= kmax;
            double x = 0.0;
            if (mrow && early) x = bd(Bd, W, kl, j + lane, j + 1);
            const double oj1 = __shfl_sync(0xffffffffu, rj, 1);  // old M(j, j+1)
            const double op1 = __shfl_sync(0xffffffffu, rp, 1);  // old M(jp, j+1)
            const double r = __shfl_sync(0xffffffffu, rc, src);
            if (lane == 0) rcp[j] = r;  // RN(1 / U(j,j)) for the forward solve
            // post-swap values
            const double a = (swapped && j + lane == jp) ? v0 : v;
            const double u1 = swapped ? op1 : oj1;
            if (swapped && j + lane == jp) x = oj1;
            const double L = nz ? a * r : a;
            double nx = 0.0;
            // x + L * (-u1), written as the identical x - L * u1
            if (mrow && early) nx = x - L * u1;
            if (swapped && c <= kmax) {
                bd(Bd, W, kl, j, c) = rp;
                if (c >= j + 2) bd(Bd, W, kl, jp, c) = rj;
            }
            if (mrow) {
                bd(Bd, W, kl, j + lane, j) = L;
                if (early) bd(Bd, W, kl, j + lane, j + 1) = nx;
            }
            named_bar(1, 128);
            // column j+1's candidates: rows j+1..imax were just updated (lane
            // l+1 holds row j+1+l); row j+1+kl, if it exists, is untouched
            if (j + 1 < nn) {
                const int imax1 = j + 1 + kl < nn - 1 ? j + 1 + kl : nn - 1;
                const int row = j + 1 + lane;
                double nv = __shfl_down_sync(0xffffffffu, nx, 1);
                if (row > imax1) nv = 0.0;
                else if (row > imax) nv = bd(Bd, W, kl, row, j + 1);
                v = nv;
                rc = __drcp_rn(v);
            }
        }
    } else if (warp == 1 || warp == 3) {
        // entry q of the kl x (kl+ku-1) block of a full step, kept in registers
        const int q0 = lane + (warp == 3 ? 32 : 0);
        const int fr = kl > 0 ? kl : 1, fc = kl + ku - 1;
        const int qi0 = q0 % fr, qk0 = q0 / fr, qi1 = (q0 + 64) % fr, qk1 = (q0 + 64) / fr;
        for (int j = 0; j < nn; j++) {
            named_bar(1, 128);
            const int imax = j + kl < nn - 1 ? j + kl : nn - 1;
            const int kmax = j + kl + ku < nn - 1 ? j + kl + ku : nn - 1;
            const int rows = imax - j, cols = kmax - j - 1;
            if (warp == 3 && j + 1 < nn) {
                // column j+1's pivot: rows j+1..imax hold warp 0's updated
                // values, row j+1+kl its untouched one
                const int imax1 = j + 1 + kl < nn - 1 ? j + 1 + kl : nn - 1;
                const int row = j + 1 + lane;
                const double cv = row <= imax1 ? bd(Bd, W, kl, row, j + 1) : 0.0;
                const int sp = pick_pivot(cv, row <= imax1, lane);
                if (lane == 0) s_src = sp;
            }
            if (rows == kl && cols == fc && rows * cols <= 128) {
                // bd(i,k) + bd(i,j) * (-bd(j,k)), written as the identical
                // bd(i,k) - bd(i,j) * bd(j,k)
                if (q0 < rows * cols) {
                    const int i = j + 1 + qi0, k = j + 2 + qk0;
                    bd(Bd, W, kl, i, k) = bd(Bd, W, kl, i, k) - bd(Bd, W, kl, i, j) * bd(Bd, W, kl, j, k);
                }
                if (q0 + 64 < rows * cols) {
                    const int i = j + 1 + qi1, k = j + 2 + qk1;
                    bd(Bd, W, kl, i, k) = bd(Bd, W, kl, i, k) - bd(Bd, W, kl, i, j) * bd(Bd, W, kl, j, k);
                }
            } else {
                for (int q = q0; q < rows * cols; q += 64) {
                    const int i = j + 1 + q % rows, k = j + 2 + q / rows;
                    bd(Bd, W, kl, i, k) = bd(Bd, W, kl, i, k) - bd(Bd, W, kl, i, j) * bd(Bd, W, kl, j, k);
                }
            }
            if (j < nn - 1) named_bar(2, 96);
        }
    } else if (warp == 2) {
        const int w = kl + ku;
        double t = lane < nn ? y[lane] : 0.0;
        for (int k = 0; k < nn; k++) {
            named_bar(1, 128);
            const int owner = k & 31;
            const double tk = __shfl_sync(0xffffffffu, t, owner);
            const double yk = div_rn_recip(tk, bd(Bd, W, kl, k, k), rcp[k]);
            if (lane == owner) {
                y[k] = yk;
                t = k + 32 < nn ? y[k + 32] : 0.0;
            }
            const int rr = k + 1 + ((lane - k - 1) & 31);
            if (rr <= k + w && rr < nn) t = t - bd(Bd, W, kl, k, rr) * yk;
        }
        __syncwarp();
    }
}

// The forward half of the transposed solve alone (U^T y = b, y in place) on
// factors band_lu_forward produced earlier: warp 2's part of that routine
// without the pipeline, the same operations in the same order. One warp.
__device__ void band_forward_only(const double* Bd_, int nn, int kl, int ku, int W, double* y, const double* rcp) {
    double* Bd = const_cast<double*>(Bd_);
    const int lane = threadIdx.x & 31, w = kl + ku;
    double t = lane < nn ? y[lane] : 0.0;
    for (int k = 0; k < nn; k++) {
        const int owner = k & 31;
        const double tk = __shfl_sync(0xffffffffu, t, owner);
        const double yk = div_rn_recip(tk, bd(Bd, W, kl, k, k), rcp[k]);
        if (lane == owner) {
            y[k] = yk;
            t = k + 32 < nn ? y[k + 32] : 0.0;
        }
        const int rr = k + 1 + ((lane - k - 1) & 31);
        if (rr <= k + w && rr < nn) t = t - bd(Bd, W, kl, k, rr) * yk;
    }
    __syncwarp();
}

// Backward half of the transposed solve (L^T), one warp, after
// band_lu_forward: lane l forms the product of the multiplier stored in band
// row i+1+l with y at its final row Fp[i+1+l] (Fp: nn ints of scratch) and
// puts it at its rank among those rows; lane 0 subtracts them in ascending
// final row, the order of the dense solve. Then the row interchanges.
__device__ void band_solve_back(const double* Bd_, int nn, int kl, int W, const int* piv, int* Fp, double* y) {
    double* Bd = const_cast<double*>(Bd_);
    __shared__ double s_prod[32];
    const int lane = threadIdx.x & 31;
    bool any = false;
    for (int i0 = 0; i0 < nn; i0 += 32) {
        const int i = i0 + lane;
        any |= __any_sync(0xffffffffu, i < nn && piv[i] != i);
    }
    if (!any) {
        // No interchange: every multiplier stays in its row, the final rows
        // are i+1..i+kl in ascending order, and lane l's product is the l-th
        // term. The newest value y[i+1] is lane 0's running sum of the
        // previous row.
        double ti = 0.0;
        for (int i = nn - 1; i >= 0; i--) {
            const int m = (i + kl < nn - 1 ? i + kl : nn - 1) - i;
            const bool act = lane < m;
            double yv = 0.0, bv = 0.0;
            if (act) {
                bv = bd(Bd, W, kl, i + 1 + lane, i);
                yv = lane == 0 ? ti : y[i + 1 + lane];
            }
            const double pr = bv * yv;
            double acc = y[i];
            for (int q = 0; q < m; q++) acc = acc - __shfl_sync(0xffffffffu, pr, q);
            ti = acc;
            if (lane == 0) y[i] = ti;
            __syncwarp();
        }
        return;
    }
    for (int r = lane; r < nn; r += 32) Fp[r] = r;
    __syncwarp();
    for (int i = nn - 1; i >= 0; i--) {
        const int rmax = i + kl < nn - 1 ? i + kl : nn - 1;
        const int m = rmax - i;
        const bool act = lane < m;
        const int fk = act ? Fp[i + 1 + lane] : 0x7fffffff;
        int rank = 0;
        for (int q = 0; q < m; q++) rank += __shfl_sync(0xffffffffu, fk, q) < fk ? 1 : 0;
        if (act) s_prod[rank] = bd(Bd, W, kl, i + 1 + lane, i) * y[fk];
        __syncwarp();
        if (lane == 0) {
            double ti = y[i];
            for (int q = 0; q < m; q++) ti = ti - s_prod[q];
            y[i] = ti;
            const int p = piv[i];
            const int tmp = Fp[i];
            Fp[i] = Fp[p];
            Fp[p] = tmp;
        }
        __syncwarp();
    }
    if (lane == 0)
        for (int i = nn - 1; i >= 0; i--)
            if (piv[i] != i) {
                const double tt = y[i];
                y[i] = y[piv[i]];
                y[piv[i]] = tt;
            }
    __syncwarp();
}

// Transposed solve M^T x = y in place (one lane, any band); Fp is nn ints of
// scratch.
__device__ void band_solve_smem(double* Bd, int nn, int kl, int ku, int W, const int* piv, int* Fp, double* y) {
    const int w = kl + ku;
    for (int i = 0; i < nn; i++) {
        double t = y[i];
        for (int k = (i - w > 0 ? i - w : 0); k < i; k++) t -= bd(Bd, W, kl, k, i) * y[k];
        y[i] = t / bd(Bd, W, kl, i, i);
    }
    for (int r = 0; r < nn; r++) Fp[r] = r;
    int fk[32];
    double fv[32];
    for (int i = nn - 1; i >= 0; i--) {
        const int rmax = i + kl < nn - 1 ? i + kl : nn - 1;
        int m = 0;
        for (int r = i + 1; r <= rmax; r++) {
            const int k = Fp[r];
            const double v = bd(Bd, W, kl, r, i);
            int q = m++;
            while (q > 0 && fk[q - 1] > k) {
                fk[q] = fk[q - 1];
                fv[q] = fv[q - 1];
                q--;
            }
            fk[q] = k;
            fv[q] = v;
        }
        double t = y[i];
        for (int q = 0; q < m; q++) t -= fv[q] * y[fk[q]];
        y[i] = t;
        const int p = piv[i];
        const int tmp = Fp[i];
        Fp[i] = Fp[p];
        Fp[p] = tmp;
    }
    for (int i = nn - 1; i >= 0; i--)
        if (piv[i] != i) {
            const double t = y[i];
            y[i] = y[piv[i]];
            y[piv[i]] = t;
        }
}

// Epsilon system of a contiguous marker range [m0, m0+dim) (ObjectsClass::
// computeEpsilon, src/Objects.cpp:264-311). Markers interact only when both
// coordinates are within 3 lattice units (the support is +-1.5); those pairs
// set the band of the system.
__device__ __forceinline__ bool eps_near(const MarkerDev& M, int ki, int kj, double Dx) {
    return fabs(M.pos[ki * 2] - M.pos[kj * 2]) / Dx < 3.0 && fabs(M.pos[ki * 2 + 1] - M.pos[kj * 2 + 1]) / Dx < 3.0;
}

__device__ __forceinline__ double eps_entry(const MarkerDev& M, int ki, int kj, double Dx) {
    const double xj = M.pos[kj * 2], yj = M.pos[kj * 2 + 1];
    double acc = 0.0;
    const int ns = M.nsupp[ki];
    for (int s = 0; s < ns; s++) {
        const double dvi = M.sd[ki * 9 + s];
        const double dX = fabs(xj / Dx - M.si[ki * 9 + s]);
        const double dY = fabs(yj / Dx - M.sj[ki * 9 + s]);
        acc += dvi * (dirac_d(dX) * dirac_d(dY));
    }
    return acc * (1.0 * 1.0 * M.ds[kj]);
}

// Fast path of the epsilon system, all in shared memory (`sm`, `sm_doubles`):
//   xy[2*dim]    marker positions
//   ph[10*dim]   kernel tables: for marker k and axis a, s = pos/Dx and
//                ph[k*10 + 5a + o] = dirac(|s - c|) at lattice line
//                c = c0[2k+a] + o, c0 = floor(s) - 2, o = 0..4. The kernel is
//                zero beyond 1.5, so every line outside the table gives the
//                exact 0.0 the direct evaluation gives.
//   c0[2*dim]    (ints)
//   cand[cap]    pairs that pass a conservative prefilter (|dx| and |dy|
//                below 3*Dx*(1 + 2^-40)), then their matrix entries
//   band / y / pivots / final rows of the banded LU
// Entries use the same operations and operands as eps_entry, so they are
// identical. Returns false (uniformly) when the marker set does not fit; the
// caller then runs the direct path.
__device__ __forceinline__ double eps_entry_tab(const MarkerDev& M, int ki, int jl, const double* ph, const int* c0,
                                                double dsj) {
    double acc = 0.0;
    const int ns = M.nsupp[ki];
    for (int s = 0; s < ns; s++) {
        const double dvi = M.sd[ki * 9 + s];
        const int ox = M.si[ki * 9 + s] - c0[jl * 2], oy = M.sj[ki * 9 + s] - c0[jl * 2 + 1];
        const double px = (ox >= 0 && ox < 5) ? ph[jl * 10 + ox] : 0.0;
        const double py = (oy >= 0 && oy < 5) ? ph[jl * 10 + 5 + oy] : 0.0;
        acc += dvi * (px * py);
    }
    return acc * (1.0 * 1.0 * dsj);
}

__device__ bool epsilon_fast(const FsiDev& F, const MarkerDev& M, int m0, int dim, double* A, double* bx, int* piv,
                             int* lmax, double* sm, int sm_doubles) {
    __shared__ int s_kl, s_ku, s_nc;
    const long long fixed = 13LL * dim + 64;
    if (!sm || dim > 4096 || fixed >= sm_doubles) return false;
    const int cap = (int)((sm_doubles - fixed) / 3);
    double* xy = sm;
    double* ph = xy + 2 * dim;
    int* c0 = reinterpret_cast<int*>(ph + 10 * dim);
    double* cval = ph + 11 * dim + 1;
    int* ckey = reinterpret_cast<int*>(cval + cap);
    double* band = cval + cap + (cap + 1) / 2 + 1;
    const long long band_doubles = sm_doubles - (band - sm);
    const double Dx = F.Dx;
    if (threadIdx.x == 0) { s_kl = 0; s_ku = 0; s_nc = 0; }
    for (int q = threadIdx.x; q < 2 * dim; q += blockDim.x) xy[q] = M.pos[m0 * 2 + q];
    __syncthreads();
    for (int q = threadIdx.x; q < 10 * dim; q += blockDim.x) {
        const int k = q / 10, a = (q % 10) / 5, o = q % 5;
        const double sc = xy[2 * k + a] / Dx;
        const int base = (int)floor(sc) - 2;
        if (o == 0) c0[2 * k + a] = base;
        ph[q] = dirac_d(fabs(sc - (base + o)));
    }
    // prefilter + compaction, whole warps per iteration
    const double lim = 3.0 * Dx * (1.0 + 0x1p-40);
    const int lane = threadIdx.x & 31;
    const int total = dim * dim;
    for (int p0 = threadIdx.x & ~31; p0 < total; p0 += blockDim.x) {
        const int pp = p0 + lane;
        bool c = false;
        if (pp < total) {
            const int i = pp / dim, j = pp % dim;
            c = fabs(xy[2 * i] - xy[2 * j]) < lim && fabs(xy[2 * i + 1] - xy[2 * j + 1]) < lim;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, c);
        int base = 0;
        if (lane == 0 && bal) base = atomicAdd(&s_nc, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int slot = base + __popc(bal & ((1u << lane) - 1u));
        if (c && slot < cap) ckey[slot] = pp;
    }
    __syncthreads();
    const int nc = s_nc;
    if (nc > cap) return false;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int pp = ckey[c];
        const int i = pp / dim, j = pp % dim;
        if (fabs(xy[2 * i] - xy[2 * j]) / Dx < 3.0 && fabs(xy[2 * i + 1] - xy[2 * j + 1]) / Dx < 3.0) {
            cval[c] = eps_entry_tab(M, m0 + i, j, ph, c0, M.ds[m0 + j]);
            if (j > i) atomicMax(&s_kl, j - i);
            else if (i > j) atomicMax(&s_ku, i - j);
        } else {
            ckey[c] = -1;
        }
    }
    __syncthreads();
    const int kl = s_kl, ku = s_ku, W = 2 * kl + ku + 1;
    if (kl < 32 && kl + ku < 32 && (long long)dim * W + 3 * dim + 1 <= band_doubles) {
        double* Bd = band;
        double* y = Bd + (size_t)dim * W;
        int* sp = reinterpret_cast<int*>(y + dim);
        int* fp = sp + dim;
        for (int q = threadIdx.x; q < dim * W; q += blockDim.x) Bd[q] = 0.0;
        for (int i = threadIdx.x; i < dim; i += blockDim.x) y[i] = 1.0;
        __syncthreads();
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
            const int pp = ckey[c];
            if (pp >= 0) bd(Bd, W, kl, pp % dim, pp / dim) = cval[c];
        }
        __syncthreads();
        if (threadIdx.x < 128) band_lu_forward(Bd, dim, kl, ku, W, sp, y, reinterpret_cast<double*>(fp + dim));
        __syncthreads();
        if (threadIdx.x < 32) band_solve_back(Bd, dim, kl, W, sp, fp, y);
        __syncthreads();
        for (int i = threadIdx.x; i < dim; i += blockDim.x) M.eps[m0 + i] = y[i];
        __syncthreads();
        return true;
    }
    // wide band: dense system in global scratch, same entries
    for (long long q = threadIdx.x; q < (long long)dim * dim; q += blockDim.x) A[q] = 0.0;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) bx[i] = 1.0;
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int pp = ckey[c];
        if (pp >= 0) A[pp] = cval[c];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        warp_lu_factor(A, dim, 0, kl, ku, piv, lmax);
        warp_lu_solve(A, dim, 0, kl, ku, piv, lmax, bx, bx);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < dim; i += blockDim.x) M.eps[m0 + i] = bx[i];
    __syncthreads();
    return true;
}

// Direct path (marker sets beyond the shared-memory plan): entries evaluated
// pair by pair, band LU in `smem` when it fits, else the dense LU in A.
__device__ void epsilon_range(const FsiDev& F, const MarkerDev& M, int m0, int dim, double* A, double* bx, int* piv,
                              int* lmax, double* smem = nullptr, int smem_doubles = 0) {
    if (epsilon_fast(F, M, m0, dim, A, bx, piv, lmax, smem, smem_doubles)) return;
    __shared__ int s_kl, s_ku;
    if (threadIdx.x == 0) { s_kl = 0; s_ku = 0; }
    __syncthreads();
    const double Dx = F.Dx;
    // bandwidths of the LU's view M = A^T: A[i][j] sits at M(j, i)
    for (long long p = threadIdx.x; p < (long long)dim * dim; p += blockDim.x) {
        const int i = (int)(p / dim), j = (int)(p % dim);
        if (i != j && eps_near(M, m0 + i, m0 + j, Dx)) {
            if (j > i) atomicMax(&s_kl, j - i);
            else atomicMax(&s_ku, i - j);
        }
    }
    __syncthreads();
    const int kl = s_kl, ku = s_ku, W = 2 * kl + ku + 1;
    const long long need = (long long)dim * W + 3 * dim + 1;  // band, y, two int arrays, reciprocals
    if (smem && kl < 32 && need <= smem_doubles) {
        double* Bd = smem;
        double* y = Bd + (size_t)dim * W;
        int* sp = reinterpret_cast<int*>(y + dim);
        int* fp = sp + dim;
        for (long long q = threadIdx.x; q < (long long)dim * W; q += blockDim.x) Bd[q] = 0.0;
        for (int i = threadIdx.x; i < dim; i += blockDim.x) y[i] = 1.0;
        __syncthreads();
        const int bw = kl > ku ? kl : ku;
        for (long long p = threadIdx.x; p < (long long)dim * dim; p += blockDim.x) {
            const int i = (int)(p / dim), j = (int)(p % dim);
            if (j - i > bw || i - j > bw) continue;
            if (eps_near(M, m0 + i, m0 + j, Dx)) bd(Bd, W, kl, j, i) = eps_entry(M, m0 + i, m0 + j, Dx);
        }
        __syncthreads();
        if (kl + ku < 32) {
            if (threadIdx.x < 128) band_lu_forward(Bd, dim, kl, ku, W, sp, y, reinterpret_cast<double*>(fp + dim));
            __syncthreads();
            if (threadIdx.x < 32) band_solve_back(Bd, dim, kl, W, sp, fp, y);
        } else if (threadIdx.x < 32) {
            band_factor_smem(Bd, dim, kl, ku, W, sp);
            if (threadIdx.x == 0) band_solve_smem(Bd, dim, kl, ku, W, sp, fp, y);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < dim; i += blockDim.x) M.eps[m0 + i] = y[i];
        __syncthreads();
        return;
    }
    for (long long p = threadIdx.x; p < (long long)dim * dim; p += blockDim.x) A[p] = 0.0;
    __syncthreads();
    for (long long p = threadIdx.x; p < (long long)dim * dim; p += blockDim.x) {
        const int i = (int)(p / dim), j = (int)(p % dim);
        if (eps_near(M, m0 + i, m0 + j, Dx)) A[p] = eps_entry(M, m0 + i, m0 + j, Dx);
    }
    for (int i = threadIdx.x; i < dim; i += blockDim.x) bx[i] = 1.0;
    __syncthreads();
    if (threadIdx.x < 32) {
        warp_lu_factor(A, dim, 0, kl, ku, piv, lmax);
        warp_lu_solve(A, dim, 0, kl, ku, piv, lmax, bx, bx);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < dim; i += blockDim.x) M.eps[m0 + i] = bx[i];
    __syncthreads();
}

constexpr int kEpsSmemDoubles = 25000;  // 200000 bytes of dynamic shared memory (opt-in)

__global__ void __launch_bounds__(256) k_fsi_epsilon_body(FsiDev F, MarkerDev M) {
    extern __shared__ double eps_smem[];
    FemBodyDev& B = F.bodies[blockIdx.x];
    epsilon_range(F, M, B.mbase, B.nMark, B.epsA, B.epsB, B.piv, B.lmax, eps_smem, kEpsSmemDoubles);
}

__global__ void __launch_bounds__(256) k_fsi_epsilon_uni(FsiDev F, MarkerDev M) {
    extern __shared__ double eps_smem[];
    epsilon_range(F, M, 0, M.n, F.uniA, F.uniB, F.uniPiv, F.uniLmax, eps_smem, kEpsSmemDoubles);
}

// FEMBodyClass::dynamicFEM (src/FEMBody.cpp:26-68) for one body per CTA.
__global__ void __launch_bounds__(256) k_fem_dynamic(FsiDev F, MarkerDev M) {
    FemBodyDev& B = F.bodies[blockIdx.x];
    __shared__ double s_res;
    __shared__ int s_it;
    const int n = B.n;
    const int nn = n - B.bc;
    constexpr int KW = 2 * 5 + 5 + 1;  // band width of the LU (kl = ku = 5)
    extern __shared__ double fem_smem[];
    double* sBd = fem_smem;            // [nn][KW] LU band
    double* sMb = sBd + nn * KW;       // [n][11] mass band
    double* sKe = sMb + n * 11;        // [n][11] stiffness band
    double* sV = sKe + n * 11;         // [n] Newmark vector
    double* sY = sV + n;               // [nn] right-hand side / solution
    int* sPiv = reinterpret_cast<int*>(sY + nn);
    int* sFp = sPiv + nn;
    double* sRcp = reinterpret_cast<double*>(sFp + nn);  // [nn] pivot reciprocals
    // Every subiteration restarts from U_n (U = U_n, Udot = Udot_n, ...), so
    // the first Newton iteration of every subiteration of a step builds the
    // same element matrices, internal force F, K_eff = K + a0 M and M v with
    // v = a0 (U_n - U) + a2 Udot + a3 Udotdot; only the load R differs.
    // Subiteration 0 keeps that iteration's LU factors, F and M v; the later
    // subiterations form F_eff = (R - F) + M v from them and solve with the
    // kept factors (the same factorisation of the same matrix).
    const bool reuse = F.s->subIt > 0;
    double* cBd = B.lu_cache;
    double* cRcp = cBd + (size_t)nn * KW;
    double* cF = cRcp + nn;
    double* cMv = cF + n;
    int* cPiv = reinterpret_cast<int*>(cMv + n);
    {
        double* U = vec(B, V_U);
        double* Ud = vec(B, V_Udot);
        double* Udd = vec(B, V_Udotdot);
        const double* Un = vec(B, V_Un);
        const double* Udn = vec(B, V_Udotn);
        const double* Uddn = vec(B, V_Udotdotn);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            U[i] = Un[i];
            Ud[i] = Udn[i];
            Udd[i] = Uddn[i];
        }
    }
    __syncthreads();
    // updateFEMValues at U = U_n: subiteration 0 evaluates it and keeps the
    // node positions and element values (length, angle, cos, sin); the later
    // subiterations restart from the same U_n and copy them back
    {
        double* cNode = reinterpret_cast<double*>(cMv + n) + (nn + 1) / 2;
        double* cEl = cNode + 3 * (size_t)B.nNodes;
        if (!reuse) {
            update_fem_values(B);
            for (int q = threadIdx.x; q < B.nNodes; q += blockDim.x) {
                const double* nd = B.node + q * 6;
                cNode[q * 3 + 0] = nd[2];
                cNode[q * 3 + 1] = nd[3];
                cNode[q * 3 + 2] = nd[5];
            }
            for (int e = threadIdx.x; e < B.nEl; e += blockDim.x) {
                const double* el = B.el + (size_t)e * EL_STRIDE;
                cEl[e * 4 + 0] = el[EL_ANG];
                cEl[e * 4 + 1] = el[EL_L];
                cEl[e * 4 + 2] = el[EL_COS];
                cEl[e * 4 + 3] = el[EL_SIN];
            }
        } else {
            for (int q = threadIdx.x; q < B.nNodes; q += blockDim.x) {
                double* nd = B.node + q * 6;
                nd[2] = cNode[q * 3 + 0];
                nd[3] = cNode[q * 3 + 1];
                nd[5] = cNode[q * 3 + 2];
            }
            for (int e = threadIdx.x; e < B.nEl; e += blockDim.x) {
                double* el = B.el + (size_t)e * EL_STRIDE;
                el[EL_ANG] = cEl[e * 4 + 0];
                el[EL_L] = cEl[e * 4 + 1];
                el[EL_COS] = cEl[e * 4 + 2];
                el[EL_SIN] = cEl[e * 4 + 3];
            }
            __syncthreads();
        }
    }
    // constructRVector (src/FEMBody.cpp:226-234; FEMElementClass::loadVector,
    // src/FEMElement.cpp:27-69): contributions per force-map entry, then an
    // ordered assembly.
    {
        const double forceScale = F.Dm / DSQ(F.Dt);
        for (int q = threadIdx.x; q < B.nfmap; q += blockDim.x) {
            const int e = B.fmapEl[q];
            const double* el = B.el + (size_t)e * EL_STRIDE;
            const double c = el[EL_COS], s = el[EL_SIN], L = el[EL_L];
            const double wgt0 = el[EL_RHO] * el[EL_A] * F.gravityX, wgt1 = el[EL_RHO] * el[EL_A] * F.gravityY;
            const int k = B.mbase + B.fmapNode[q];
            const double a = B.fmapZ[q * 2], b = B.fmapZ[q * 2 + 1];
            const double sc = -M.eps[k] * 1.0 * forceScale;
            const double g0 = sc * M.force[k * 2] + wgt0, g1 = sc * M.force[k * 2 + 1] + wgt1;
            const double F0 = (0.0 + c * g0) + s * g1;
            const double F1 = (0.0 + (-s) * g0) + c * g1;
            double R[6], RG[6];
            R[0] = F0 * 0.5 * L * (0.5 * b - 0.5 * a + 0.25 * DSQ(a) - 0.25 * DSQ(b));
            R[1] = F1 * 0.5 * L * (0.5 * b - 0.5 * a - DSQ(a) * DSQ(a) / 16.0 + DSQ(b) * DSQ(b) / 16.0 + 3.0 * DSQ(a) / 8.0 - 3.0 * DSQ(b) / 8.0);
            R[2] = F1 * 0.5 * L * (L * (-DSQ(a) * DSQ(a) + DSQ(b) * DSQ(b)) / 32.0 - L * (-DTH(a) + DTH(b)) / 24.0 - L * (-DSQ(a) + DSQ(b)) / 16.0 + L * (b - a) / 8.0);
            R[3] = F0 * 0.5 * L * (-0.25 * DSQ(a) + 0.25 * DSQ(b) + 0.5 * b - 0.5 * a);
            R[4] = F1 * 0.5 * L * (0.5 * b - 0.5 * a + DSQ(a) * DSQ(a) / 16.0 - DSQ(b) * DSQ(b) / 16.0 - 3.0 * DSQ(a) / 8.0 + 3.0 * DSQ(b) / 8.0);
            R[5] = F1 * 0.5 * L * (L * (-DSQ(a) * DSQ(a) + DSQ(b) * DSQ(b)) / 32.0 + L * (-DTH(a) + DTH(b)) / 24.0 - L * (-DSQ(a) + DSQ(b)) / 16.0 - L * (b - a) / 8.0);
            tt_vec(R, c, s, RG);
            for (int r = 0; r < 6; r++) B.rgscr[q * 6 + r] = RG[r];
        }
        __syncthreads();
        double* Rv = vec(B, V_R);
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            double acc = 0.0;
            const int e1 = r / 3 - 1, e2 = r / 3;
            for (int e = (e1 < 0 ? 0 : e1); e <= e2 && e < B.nEl; e++)
                for (int q = B.fmapStart[e]; q < B.fmapStart[e + 1]; q++) acc += B.rgscr[q * 6 + (r - 3 * e)];
            Rv[r] = acc;
        }
        __syncthreads();
    }
    const double Dt = F.Dt, al = F.alpha;
    const double a0 = 1.0 / (al * DSQ(Dt)), a2 = 1.0 / (al * Dt), a3 = 1.0 / (2.0 * al) - 1.0;
    if (threadIdx.x == 0) s_it = 0;
    __syncthreads();
    do {
        const bool first = s_it == 0;
        if (first && reuse) {
            // the kept factors and vectors of this step's first iteration
            double* Fv = vec(B, V_F);
            const double* Rv = vec(B, V_R);
            for (int q = threadIdx.x; q < nn * KW; q += blockDim.x) sBd[q] = cBd[q];
            for (int i = threadIdx.x; i < nn; i += blockDim.x) {
                sPiv[i] = cPiv[i];
                sRcp[i] = cRcp[i];
            }
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const double fe = Rv[i] - cF[i] + cMv[i];
                Fv[i] = fe;
                if (i >= B.bc) sY[i - B.bc] = fe;
            }
            __syncthreads();
            if (threadIdx.x < 32) band_forward_only(sBd, nn, 5, 5, KW, sY, sRcp);
            __syncthreads();
            if (threadIdx.x < 32) band_solve_back(sBd, nn, 5, KW, sPiv, sFp, sY);
            __syncthreads();
        } else {
            // buildGlobalMatrices (src/FEMBody.cpp:90-109)
            for (int e = threadIdx.x; e < B.nEl; e += blockDim.x) {
                const double* el = B.el + (size_t)e * EL_STRIDE;
                const double L = el[EL_L], L0 = el[EL_L0], E = el[EL_E], A = el[EL_A], I = el[EL_I];
                const double c = el[EL_COS], s = el[EL_SIN], ang = el[EL_ANG];
                const double u = (DSQ(L) - DSQ(L0)) / (L + L0);
                const double th1 = shift_angle_d(B.node[e * 6 + 5] - ang);
                const double th2 = shift_angle_d(B.node[(e + 1) * 6 + 5] - ang);
                const double F0 = (E * A / L0) * u;
                const double M1 = (2 * E * I / L0) * (2.0 * th1 + th2);
                const double M2 = (2 * E * I / L0) * (th1 + 2.0 * th2);
                double Fl[6];
                Fl[0] = -F0;
                Fl[1] = (1.0 / L0) * (M1 + M2);
                Fl[2] = M1;
                Fl[3] = F0;
                Fl[4] = -(1.0 / L0) * (M1 + M2);
                Fl[5] = M2;
                double* sc = B.elscr + (size_t)e * ES_STRIDE;
                tt_vec(Fl, c, s, sc + ES_F);
                tt_a_t(el + EL_M, c, s, sc + ES_M);
                double G[36], G2[36], KNL[36];
                tt_a_t(el + EL_KL, c, s, G);
                const double Fa = -Fl[0], V0 = Fl[4];
    #pragma unroll
                for (int q = 0; q < 36; q++) KNL[q] = 0.0;
                KNL[0 * 6 + 1] = -V0 / L0;
                KNL[0 * 6 + 4] = V0 / L0;
                KNL[1 * 6 + 0] = -V0 / L0;
                KNL[1 * 6 + 1] = Fa / L0;
                KNL[1 * 6 + 3] = V0 / L0;
                KNL[1 * 6 + 4] = -Fa / L0;
                KNL[3 * 6 + 1] = V0 / L0;
                KNL[3 * 6 + 4] = -V0 / L0;
                KNL[4 * 6 + 0] = V0 / L0;
                KNL[4 * 6 + 1] = -Fa / L0;
                KNL[4 * 6 + 3] = -V0 / L0;
                KNL[4 * 6 + 4] = Fa / L0;
                tt_a_t(KNL, c, s, G2);
    #pragma unroll
                for (int q = 0; q < 36; q++) sc[ES_K + q] = G[q] + G2[q];
            }
            __syncthreads();
            // Ordered assembly of M, K (band |r-c| <= 5) and F, then setNewmark
            // (src/FEMBody.cpp:112-126): K_eff = K + a0*M goes straight into the
            // shared-memory band of the LU's view M(i,j) = K_eff[bc+j][bc+i].
            {
                double* Fv = vec(B, V_F);
                for (int q = threadIdx.x; q < nn * KW; q += blockDim.x) sBd[q] = 0.0;
                for (int p = threadIdx.x; p < n * 11; p += blockDim.x) {
                    const int r = p / 11, cc = r - 5 + p % 11;
                    if (cc < 0 || cc >= n) continue;
                    double am = 0.0, ak = 0.0;
                    const int lo = (r > cc ? r : cc), hi = (r < cc ? r : cc);
                    for (int e = (lo / 3 - 1 < 0 ? 0 : lo / 3 - 1); e <= hi / 3 && e < B.nEl; e++) {
                        const int li = r - 3 * e, lj = cc - 3 * e;
                        if (li < 0 || li > 5 || lj < 0 || lj > 5) continue;
                        const double* sc = B.elscr + (size_t)e * ES_STRIDE;
                        am += sc[ES_M + li * 6 + lj];
                        ak += sc[ES_K + li * 6 + lj];
                    }
                    sMb[p] = am;
                    sKe[p] = ak;
                }
                for (int r = threadIdx.x; r < n; r += blockDim.x) {
                    double af = 0.0;
                    for (int e = (r / 3 - 1 < 0 ? 0 : r / 3 - 1); e <= r / 3 && e < B.nEl; e++)
                        af += B.elscr[(size_t)e * ES_STRIDE + ES_F + (r - 3 * e)];
                    Fv[r] = af;
                }
                const double* U = vec(B, V_U);
                const double* Un = vec(B, V_Un);
                const double* Ud = vec(B, V_Udot);
                const double* Udd = vec(B, V_Udotdot);
                for (int i = threadIdx.x; i < n; i += blockDim.x) sV[i] = a0 * (Un[i] - U[i]) + a2 * Ud[i] + a3 * Udd[i];
                __syncthreads();
                const double* Rv = vec(B, V_R);
                for (int i = threadIdx.x; i < n; i += blockDim.x) {
                    double mv = 0.0;
                    for (int j = (i - 5 < 0 ? 0 : i - 5); j <= i + 5 && j < n; j++) mv += sMb[i * 11 + (j - i + 5)] * sV[j];
                    if (first) {
                        cF[i] = Fv[i];
                        cMv[i] = mv;
                    }
                    const double fe = Rv[i] - Fv[i] + mv;
                    Fv[i] = fe;
                    if (i >= B.bc) sY[i - B.bc] = fe;
                }
                for (int p = threadIdx.x; p < n * 11; p += blockDim.x) {
                    const int r = p / 11, cc = r - 5 + p % 11;
                    if (cc < B.bc || cc >= n || r < B.bc) continue;
                    const double keff = sKe[p] + a0 * sMb[p];
                    bd(sBd, KW, 5, cc - B.bc, r - B.bc) = keff;
                }
            }
            __syncthreads();
            // delU = solveLAPACK(K, F, bcDOFs) (src/Utils.cpp:288-311)
            if (threadIdx.x < 128) band_lu_forward(sBd, nn, 5, 5, KW, sPiv, sY, sRcp);
            __syncthreads();
            if (first) {
                for (int q = threadIdx.x; q < nn * KW; q += blockDim.x) cBd[q] = sBd[q];
                for (int i = threadIdx.x; i < nn; i += blockDim.x) {
                    cPiv[i] = sPiv[i];
                    cRcp[i] = sRcp[i];
                }
            }
            if (threadIdx.x < 32) band_solve_back(sBd, nn, 5, KW, sPiv, sFp, sY);
            __syncthreads();
        }
        {
            double* dU = vec(B, V_delU);
            for (int i = threadIdx.x; i < n; i += blockDim.x) dU[i] = i < B.bc ? 0.0 : sY[i - B.bc];
        }
        __syncthreads();
        {
            double* U = vec(B, V_U);
            const double* dU = vec(B, V_delU);
            for (int i = threadIdx.x; i < n; i += blockDim.x) U[i] = U[i] + dU[i];
        }
        __syncthreads();
        // squares in parallel, then the sum in index order (one thread)
        {
            const double* dU = vec(B, V_delU);
            for (int i = threadIdx.x; i < n; i += blockDim.x) sV[i] = dU[i] * dU[i];
        }
        update_fem_values(B);
        if (threadIdx.x == 0) {
            double dd = 0.0;
            for (int i = 0; i < n; i++) dd += sV[i];
            s_res = sqrt(dd) / (F.ref_L * sqrt((double)n));
            s_it++;
        }
        __syncthreads();
    } while (s_res > 1e-10 && s_it < 20);
    finish_newmark(B, F);
    update_ibm(B, M);
    if (threadIdx.x == 0) {
        B.itNR = s_it;
        B.resNR = s_res;
        swap_slots(B, V_Rkm1, V_Rk);
    }
    __syncthreads();
    // FEMBodyClass::subResidual (src/FEMBody.cpp:244-256): the terms in
    // parallel, each of the three sums in index order by one thread of its
    // own warp.
    {
        double* Rk = vec(B, V_Rk);
        const double* Rkm1 = vec(B, V_Rkm1);
        const double* U = vec(B, V_U);
        const double* Uk = vec(B, V_Ukm1);
        double* tr = sMb;
        double* tn = sMb + n;
        double* td = sMb + 2 * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double r = U[i] - Uk[i];
            const double d = r - Rkm1[i];
            Rk[i] = r;
            tr[i] = r * r;
            tn[i] = Rkm1[i] * d;
            td[i] = d * d;
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0 && threadIdx.x < 96) {
            const double* t = sMb + (threadIdx.x >> 5) * n;
            double acc = 0.0;
            for (int i = 0; i < n; i++) acc += t[i];
            if (threadIdx.x == 0) B.subRes = acc;
            else if (threadIdx.x == 32) B.subNum = acc;
            else B.subDen = acc;
        }
    }
}

// Standalone epsilon solve over n markers with caller-provided scratch
// (A: n*n, b: n, piv, lmax: n).
__global__ void __launch_bounds__(256) k_epsilon_markers(FsiDev F, MarkerDev M, int n, double* A, double* b, int* piv,
                                                         int* lmax) {
    extern __shared__ double eps_smem[];
    epsilon_range(F, M, 0, n, A, b, piv, lmax, eps_smem, kEpsSmemDoubles);
}

// Element transform after a restart load (FEMElementClass::setElementTransform,
// src/FEMElement.cpp:255-262, called from ObjectsClass::readRestart,
// src/Objects.cpp:1195-1200): cos and sin of the loaded angles, with the
// same functions update_fem_values uses during a step.
__global__ void k_fem_element_trig(double* el, int nEl) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nEl) return;
    const double ang = el[(size_t)e * EL_STRIDE + EL_ANG];
    double sa, ca;
    life_cr_sincos(ang, &sa, &ca);
    el[(size_t)e * EL_STRIDE + EL_COS] = ca;
    el[(size_t)e * EL_STRIDE + EL_SIN] = sa;
}

cudaError_t launch_fem_element_trig(double* el, int nEl, cudaStream_t s) {
    if (nEl <= 0) return cudaSuccess;
    k_fem_element_trig<<<(nEl + 127) / 128, 128, 0, s>>>(el, nEl);
    return cudaGetLastError();
}

// The epsilon kernels take 200000 bytes of dynamic shared memory (opt-in);
// the attribute is set once per device.
cudaError_t epsilon_configure() {
    static std::atomic<int> done[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64 && done[dev].load()) return cudaSuccess;
    const int bytes = kEpsSmemDoubles * (int)sizeof(double);
    e = cudaFuncSetAttribute(k_fsi_epsilon_body, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fsi_epsilon_uni, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_epsilon_markers, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev].store(1);
    return e;
}

cudaError_t launch_epsilon_markers(const MarkerDev& M, int n, double Dx, double* A, double* b, int* piv, int* lmax,
                                   cudaStream_t s) {
    FsiDev F{};
    F.Dx = Dx;
    cudaError_t e = epsilon_configure();
    if (e != cudaSuccess) return e;
    k_epsilon_markers<<<1, 256, kEpsSmemDoubles * sizeof(double), s>>>(F, M, n, A, b, piv, lmax);
    return cudaGetLastError();
}

// ObjectsClass::femKernel sums + loop condition + next relaxation factor.
// Inside the captured loop graph the condition also drives the WHILE node.
__global__ void k_fsi_residual(FsiDev F, cudaGraphConditionalHandle cond, int use_cond) {
    if (threadIdx.x != 0) return;
    FsiScalars& S = *F.s;
    double res = 0.0, num = 0.0, den = 0.0;
    for (int b = 0; b < F.nFlex; b++) {
        res += F.bodies[b].subRes;
        num += F.bodies[b].subNum;
        den += F.bodies[b].subDen;
    }
    S.subRes = sqrt(res) / (F.ref_L * sqrt((double)F.simDOFs));
    S.subNum = num;
    S.subDen = den;
    S.subIt += 1;
    S.lastNR = F.nFlex > 0 ? F.bodies[0].itNR : 0;
    const int cont = (S.subIt < 20 && S.subRes > F.subTol) ? 1 : 0;
    if (cont) {
        if (S.subIt == 1) {
            const double a = fabs(S.relax);
            const int sg = (0.0 < S.relax) - (S.relax < 0.0);
            S.relax = (double)(sg * (a < F.relaxMax ? a : F.relaxMax));
        } else {
            S.relax = -S.relax * S.subNum / S.subDen;
        }
    } else if (S.subIt == 20) {
        if (atomicCAS(&F.status[0], 0, LIFE_ERR_SUBITER) == 0) F.status[1] = S.t;
    }
    *F.cont = cont;
    if (use_cond) cudaGraphSetConditional(cond, cont ? 1u : 0u);
}

__global__ void k_fsi_begin(FsiDev F, int t, const int* t_dev, int t_off) {
    F.s->t = t_dev ? *t_dev + t_off : t;
    F.s->subIt = 0;
    *F.cont = 1;
}

size_t fem_dynamic_smem(int n, int bc) {
    const int nn = n - bc;
    return sizeof(double) * ((size_t)nn * 17 + (size_t)n * 22 + n + nn) + sizeof(int) * 2 * (size_t)nn;
}

// The opt-in shared-memory size is an attribute of the kernel, shared by every
// case on the device, so it only ever grows: a case created later with
// smaller bodies must not lower it below what a live case launches with.
cudaError_t fem_dynamic_configure(size_t smem) {
    static std::atomic<size_t> set[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    size_t cur = set[dev].load();
    if (smem > cur) {
        e = cudaFuncSetAttribute(k_fem_dynamic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        while (cur < smem && !set[dev].compare_exchange_weak(cur, smem)) {
        }
    }
    return epsilon_configure();
}

cudaError_t launch_fsi_begin(const FsiDev& F, int t, cudaStream_t s, const int* t_dev, int t_off) {
    k_fsi_begin<<<1, 1, 0, s>>>(F, t, t_dev, t_off);
    return cudaGetLastError();
}

cudaError_t launch_fsi_subiteration(const FsiDev& F, const MarkerDev& M, const void* P, const LatDev& L, int t,
                                    double velScale, cudaStream_t s, int* launches,
                                    const cudaGraphConditionalHandle* cond) {
    k_fsi_predict<<<F.nFlex, 256, 0, s>>>(F, M);
    k_fsi_support<<<(F.nFlexMarkers + 3) / 4, 128, 0, s>>>(F, M);
    if (F.uni) k_fsi_epsilon_uni<<<1, 256, kEpsSmemDoubles * sizeof(double), s>>>(F, M);
    else k_fsi_epsilon_body<<<F.nFlex, 256, kEpsSmemDoubles * sizeof(double), s>>>(F, M);
    cudaError_t e = launch_ibm_interp(P, L, t, M, velScale, s, cond ? &F.s->t : nullptr);
    if (e != cudaSuccess) return e;
    k_fem_dynamic<<<F.nFlex, 256, F.fem_smem, s>>>(F, M);
    k_fsi_residual<<<1, 32, 0, s>>>(F, cond ? *cond : cudaGraphConditionalHandle{}, cond ? 1 : 0);
    if (launches) *launches += 6;
    return cudaGetLastError();
}

}  // namespace life

namespace {
__global__ void k_selftest_trig(int op, long long n, const double* x, const double* y, double* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double s, c;
        if (op == 2) {
            out[i] = life_cr_atan2(y[i], x[i]);
        } else {
            life_cr_sincos(x[i], &s, &c);
            out[i] = op == 0 ? s : c;
        }
    }
}
}  // namespace

extern "C" int life_selftest_trig(int32_t op, int64_t n, const double* x, const double* y, double* out) {
    if (op < 0 || op > 2 || n <= 0 || !x || !out || (op == 2 && !y))
        return life::set_error(LIFE_ERR_INVALID, "bad arguments");
    double *dx = nullptr, *dy = nullptr, *dout = nullptr;
    const size_t bytes = sizeof(double) * (size_t)n;
    cudaError_t e = cudaMalloc(&dx, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dout, bytes);
    if (e == cudaSuccess && op == 2) e = cudaMalloc(&dy, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && op == 2) e = cudaMemcpy(dy, y, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_selftest_trig<<<152 * 4, 256>>>(op, (long long)n, dx, dy, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dout);
    if (e != cudaSuccess) return life::cuda_fail(e, "life_selftest_trig");
    return LIFE_OK;
}

extern "C" int life_selftest_division(int64_t n, uint64_t seed, int64_t* mismatches) {
    if (n <= 0 || !mismatches) return life::set_error(LIFE_ERR_INVALID, "bad arguments");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        life::k_selftest_division<<<152 * 8, 256>>>((long long)n, (unsigned long long)seed, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return life::cuda_fail(e, "life_selftest_division");
    *mismatches = (int64_t)h;
    return LIFE_OK;
}
