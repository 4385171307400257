// Lattice kernels with FP64 arithmetic: the plain form that reproduces the
// reference's CPU FP64 results, plus the FP64-arithmetic parts every storage
// form shares (boundary sites, start-up, restart, export). Compiled with
// --fmad=false (see the header of lbm_device.cuh).
//
//   k_init_rows/fill initial equilibrium state and the first collision
//   k_interior_f64  fused pull-stream + macroscopic + collision of the next
//                   step for fluid sites (one read and one write of the nine
//                   populations per site)
//   k_perimeter     the same for boundary-condition sites, with the
//                   regularised / convective conditions applied
//   k_outlet_f64    convective outlet speed (sequential mean, as the reference;
//                   a fixed-order tree sum for the reduced-precision forms)
//   k_state         collision from an explicit state (restart read)
//   k_export        reference-layout fields of the current step
//   k_maxvel        max |u| and NaN scan
#include <cuda_runtime.h>

#include <type_traits>

#include "collide_cm.cuh"
#include "lbm_device.cuh"
#include "lbm_kernels.h"

namespace life {

// GridClass::initialiseGrid (reference src/Grid.cpp:998-1061): rho = 1,
// initial velocity, f = feq; then the collision of step t0+1. Every site of
// row j starts from the equilibrium at rho = 1 of one of two velocities: the
// row's (uniform, or the inlet profile at j) or zero at a wall site. The two
// variants of every row are formed once (k_init_rows: a thread per row and
// variant, the FP64 chain of store_collided's arithmetic), then every site
// stores its variant (k_init_fill, a write of the lattice).
template <class S>
struct InitRow {
    typename S::T out[9];  // the stored populations after the first collision
    double f[9], u[2];     // the state before it (outlet side outputs, corner history)
};

template <bool CM, class S>
__global__ void k_init_rows(InitRow<S>* __restrict__ rows, LatDev L, int t0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = k >> 1, w = k & 1;
    if (j >= L.Ny) return;
    double ux, uy;
    if (w == 1 || L.init_mode == 0) { ux = 0.0; uy = 0.0; }
    else if (L.init_mode == 1) { ux = L.u_in[j * 2]; uy = L.u_in[j * 2 + 1]; }
    else { ux = L.u0x; uy = L.u0y; }
    const double rho = 1.0;
    double f[9], fs[9], Fx, Fy;
#pragma unroll
    for (int v = 0; v < 9; v++) f[v] = equilibrium<CM>(v, rho, ux, uy);
    force_xy_next(L, t0 + 1, rho, Fx, Fy);
    collide<CM>(f, rho, ux, uy, Fx + 0.0, Fy + 0.0, L.omega, L.cs, fs);
    InitRow<S>& r = rows[k];
#pragma unroll
    for (int v = 0; v < 9; v++) {
        r.out[v] = S::save(fs[v], v);
        r.f[v] = f[v];
    }
    r.u[0] = ux;
    r.u[1] = uy;
}

template <class S>
__global__ void k_init_fill(typename S::T* __restrict__ B, const InitRow<S>* __restrict__ rows, LatDev L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    const int type = site_type(L, i, j);
    const InitRow<S>& r = rows[2 * j + (type == LIFE_WALL ? 1 : 0)];
    outlet_outputs(L, i, j, r.f, r.u[0], r.u[1]);
    store_history(L, type, i, j, 1.0, r.u[0], r.u[1]);
    const size_t s = (size_t)j * L.pitch + i;
#pragma unroll
    for (int v = 0; v < 9; v++) B[(size_t)v * L.S + s] = r.out[v];
}

// One time step, interior sites, FP64: S_t from P_t (A), then P_{t+1} into B.
// Sites on a boundary-condition wall are left to k_perimeter; IBM support
// sites are collided again by the IBM fix-up kernel once the spread force is
// known. Same arithmetic as site_state() for a fluid site. SITE: the case
// has a per-site force (WOMERSLEY with gravity), a separate instantiation so
// the other cases' kernels do not carry its registers.
template <bool CM, bool SITE>
__device__ __forceinline__ void interior_site_f64(const double* __restrict__ A, double* __restrict__ B,
                                                  const LatDev& L, int t, int i, int j) {
    if (site_type(L, i, j) != LIFE_FLUID) return;
    double f[9], rho, ux, uy, Fx, Fy;
    const bool edge = (i == 0) | (i == L.Nx - 1) | (j == 0) | (j == L.Ny - 1);
    if (edge) {
        gather<StoreF64>(A, L, i, j, f);
    } else {
        const size_t base = (size_t)j * L.pitch + i;
#pragma unroll
        for (int v = 0; v < 9; v++) f[v] = A[(size_t)v * L.S + base - cx_of(v) - (long long)cy_of(v) * L.pitch];
    }
    if (SITE) {
        const size_t s = (size_t)j * L.pitch + i;
        force_xy_site(L, t, L.rho_prev[s], Fx, Fy);
        macroscopic(f, Fx, Fy, rho, ux, uy);
        outlet_outputs(L, i, j, f, ux, uy);
        L.rho_next[s] = rho;
        double Gx, Gy, fs[9];
        force_xy_site(L, t + 1, rho, Gx, Gy);
        collide<CM>(f, rho, ux, uy, Gx + 0.0, Gy + 0.0, L.omega, L.cs, fs);
#pragma unroll
        for (int v = 0; v < 9; v++) B[(size_t)v * L.S + s] = fs[v];
    } else if (lattice_forced_d(L)) {
        force_xy_at(L, t, Fx, Fy);
        macroscopic(f, Fx, Fy, rho, ux, uy);
        outlet_outputs(L, i, j, f, ux, uy);
        double Gx, Gy, fs[9];
        force_xy_at(L, t + 1, Gx, Gy);
        collide<CM>(f, rho, ux, uy, Gx + 0.0, Gy + 0.0, L.omega, L.cs, fs);
#pragma unroll
        for (int v = 0; v < 9; v++) B[(size_t)v * L.S + (size_t)j * L.pitch + i] = fs[v];
    } else {
        // zero force at every step: the velocity without the force half-term
        // (the same value) and no forcing terms in the collision
        macroscopic_unforced(f, rho, ux, uy);
        outlet_outputs(L, i, j, f, ux, uy);
        double fs[9];
        collide<CM, true>(f, rho, ux, uy, 0.0, 0.0, L.omega, L.cs, fs);
        const size_t s = (size_t)j * L.pitch + i;
#pragma unroll
        for (int v = 0; v < 9; v++) B[(size_t)v * L.S + s] = fs[v];
    }
}

template <bool CM, bool SITE>
__global__ void __launch_bounds__(128) k_interior_f64(const double* __restrict__ A, double* __restrict__ B, LatDev L,
                                                      int t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    interior_site_f64<CM, SITE>(A, B, L, step_t(L, t), i, j);
}

// All cases of a batch in one persistent launch (see k_interior_batch_lowp).
__global__ void __launch_bounds__(256) k_interior_batch_f64(const BatchLatCase* __restrict__ cases,
                                                            const int* __restrict__ tile_case, int ntiles, int tile_h,
                                                            int phase) {
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
        const BatchLatCase& C = cases[tile_case[q]];
        const LatDev& L = C.L[phase];
        const int lt = q - C.tile0;
        const int tx = lt % C.tiles_x, ty = lt / C.tiles_x;
        const int i = tx * blockDim.x + threadIdx.x;
        if (i >= L.Nx) continue;
        const int t = step_t(L, 0);
        const double* A = (const double*)C.A[phase];
        double* B = (double*)C.B[phase];
        const int j1 = (ty + 1) * tile_h < L.Ny ? (ty + 1) * tile_h : L.Ny;
        for (int j = ty * tile_h; j < j1; j++) {
            if (L.site_force) {
                if (L.cm) interior_site_f64<true, true>(A, B, L, t, i, j);
                else interior_site_f64<false, true>(A, B, L, t, i, j);
            } else {
                if (L.cm) interior_site_f64<true, false>(A, B, L, t, i, j);
                else interior_site_f64<false, false>(A, B, L, t, i, j);
            }
        }
    }
}

// Boundary-condition sites of one step, FP64 storage (perimeter_site,
// lbm_device.cuh); the reduced-precision forms have theirs in lbm_lowp.cu.
template <bool CM, class S>
__global__ void k_perimeter(const typename S::T* __restrict__ A, typename S::T* __restrict__ B, LatDev L, int t) {
    perimeter_site<CM, S>(A, B, L, step_t(L, t), blockIdx.x * blockDim.x + threadIdx.x);
}

// GridClass::convectiveSpeed (src/Grid.cpp:477-495): the mean outlet speed is
// a sequential sum over j, as in the reference.
__global__ void k_outlet_f64(LatDev L, double* __restrict__ delU) {
    __shared__ double uOut_s;
    __shared__ double col[1024];
    const int Ny = L.Ny;
    const double* u1 = L.outlet_u + (size_t)2 * Ny * 2;  // column Nx-1
    const double* u2 = L.outlet_u + (size_t)1 * Ny * 2;  // column Nx-2
    const double* u3 = L.outlet_u;                       // column Nx-3
    if (L.prec != LIFE_PREC_F64) {
        // Reduced-precision forms (whose state is not the reference's bits):
        // a tree sum in a fixed order (strided per thread, then the warps,
        // then the warp sums in order), the same on every run; a chain of
        // ~15 dependent FP64 additions instead of Ny.
        __shared__ double wsum[32];
        double part = 0.0;
        for (int j = threadIdx.x; j < Ny; j += blockDim.x) part += u1[j * 2];
        for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) a += wsum[w];
            uOut_s = a / (double)Ny;
        }
    } else {
        // All threads stage the outlet column through shared memory; one
        // thread then adds it up in j order, as the reference does.
        double acc = 0.0;
        for (int j0 = 0; j0 < Ny; j0 += 1024) {
            const int m = Ny - j0 < 1024 ? Ny - j0 : 1024;
            __syncthreads();
            for (int j = threadIdx.x; j < m; j += blockDim.x) col[j] = u1[(j0 + j) * 2];
            __syncthreads();
            if (threadIdx.x == 0)
                for (int j = 0; j < m; j++) acc += col[j];
        }
        if (threadIdx.x == 0) {
            acc /= (double)Ny;
            uOut_s = acc;
        }
    }
    __syncthreads();
    const double uOut = uOut_s;
    for (int j = threadIdx.x; j < Ny; j += blockDim.x)
        for (int d = 0; d < 2; d++)
            delU[j * 2 + d] = (-uOut / 2.0) * (3.0 * u1[j * 2 + d] - 4.0 * u2[j * 2 + d] + u3[j * 2 + d]);
}

// Collision from an explicit reference-layout state (GridClass::readRestart,
// src/Grid.cpp:1072-1160, followed by the next step's collision).
template <bool CM, class S>
__global__ void k_state(typename S::T* __restrict__ B, LatDev L, int t, const double* __restrict__ rho_in,
                            const double* __restrict__ u_in, const double* __restrict__ f_in,
                            const double* __restrict__ fibm_in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    const size_t id = (size_t)i * L.Ny + j;
    double f[9];
#pragma unroll
    for (int v = 0; v < 9; v++) f[v] = f_in[id * 9 + v];
    const double rho = rho_in[id], ux = u_in[id * 2], uy = u_in[id * 2 + 1];
    outlet_outputs(L, i, j, f, ux, uy);
    store_history(L, site_type(L, i, j), i, j, rho, ux, uy);
    store_collided<CM, S>(B, L, t + 1, i, j, f, rho, ux, uy, fibm_in[id * 2], fibm_in[id * 2 + 1]);
}

// In the reduced-precision forms a fluid site without an IBM force gets its
// velocity exactly as the step kernels form it, in FP32 (finish_site_lowp:
// deviations, 1/rho by rcp_lowp, momentum with the half force), and
// its density as 1 + the FP32 deviation sum in FP64; the FP64 path
// (site_state) would spend ~50 FP64 operations per site on the narrow FP64
// pipe. Boundary and IBM-corrected sites, populations requested, and the
// per-site force take the FP64 path, as their kernels do.
template <class S>
__device__ __forceinline__ bool export_fluid_lowp(const typename S::T* __restrict__ P, const LatDev& L, int t, int i,
                                                  int j, bool allowed, double& rho, double& ux, double& uy) {
    if constexpr (std::is_same<S, StoreF64>::value) {
        return false;
    } else {
        if (!allowed || L.site_force || site_type(L, i, j) != LIFE_FLUID) return false;
        if (L.force_ibm) {
            const size_t s = (size_t)j * L.pitch + i;
            if (L.force_ibm[s] != 0.0 || L.force_ibm[L.S + s] != 0.0) return false;
        }
        float g[9];
#pragma unroll
        for (int v = 0; v < 9; v++) {
            int si = i - cx_of(v), sj = j - cy_of(v);
            si = si < 0 ? si + L.Nx : (si >= L.Nx ? si - L.Nx : si);
            sj = sj < 0 ? sj + L.Ny : (sj >= L.Ny ? sj - L.Ny : sj);
            g[v] = S::dev(P[(size_t)v * L.S + (size_t)sj * L.pitch + si], v);
        }
        float Fxd = 0.0f, Fyd = 0.0f;
        if (L.womersley || L.Fx0_f != 0.0f || L.Fy0_f != 0.0f) force_xy_at_f(L, t, Fxd, Fyd);
        const float dr = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) + g[8];
        const float rf = 1.0f + dr;
        const float mx = (g[1] - g[2]) + (g[5] - g[6]) + (g[7] - g[8]);
        const float my = (g[3] - g[4]) + (g[5] - g[6]) + (g[8] - g[7]);
        const float inv = rcp_lowp(rf);
        const bool forced = L.womersley || L.Fx0_f != 0.0f || L.Fy0_f != 0.0f;
        const float px = forced ? fmaf(0.5f, Fxd, mx) : mx, py = forced ? fmaf(0.5f, Fyd, my) : my;
        rho = 1.0 + (double)dr;
        ux = (double)(px * inv);
        uy = (double)(py * inv);
        return true;
    }
}

// Reference-layout export of the state after step t (what
// GridClass::writeRestart dumps, src/Grid.cpp:1191-1222). The reference
// layout is column-major in the device's terms (id = i*Ny + j), so a block
// computes a 32 x 32 tile of sites with i fastest (the pulls read whole rows
// of each population plane) and writes rho, u and force_ibm through shared
// memory with j fastest (whole runs of the output); f, exported for restart
// sets and parity checks, is written per site.
template <bool CM, class S>
__global__ void __launch_bounds__(256) k_export(const typename S::T* __restrict__ P, LatDev L, int t,
                                                double* __restrict__ rho_out, double* __restrict__ u_out,
                                                double* __restrict__ f_out, double* __restrict__ fibm_out, int i0,
                                                int i1) {
    // columns i0 <= i < i1 (their reference-layout rows id = i*Ny + j are
    // one contiguous range of the output)
    __shared__ double s_rho[32][33];
    __shared__ double2 s_u[32][33], s_fi[32][33];
    const int ib = i0 + blockIdx.x * 32, jb = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = ib + tx;
#pragma unroll 1
    for (int q = ty; q < 32; q += 8) {
        const int j = jb + q;
        if (i >= i1 || j >= L.Ny) continue;
        double f[9], rho, ux, uy;
        double Ix = 0.0, Iy = 0.0;
        if (export_fluid_lowp<S>(P, L, t, i, j, f_out == nullptr, rho, ux, uy)) {
            s_rho[tx][q] = rho;
            s_u[tx][q] = make_double2(ux, uy);
            s_fi[tx][q] = make_double2(0.0, 0.0);
            continue;
        }
        site_state<CM, S>(P, L, t, i, j, f, rho, ux, uy);
        if (L.force_ibm) {
            const size_t s = (size_t)j * L.pitch + i;
            Ix = L.force_ibm[s];
            Iy = L.force_ibm[L.S + s];
            if (Ix != 0.0 || Iy != 0.0) {
                double Fx, Fy;
                force_xy_of(L, t, i, j, Fx, Fy);
                macroscopic_ibm(f, Fx, Fy, Ix, Iy, rho, ux, uy);
            }
        }
        s_rho[tx][q] = rho;
        s_u[tx][q] = make_double2(ux, uy);
        s_fi[tx][q] = make_double2(Ix, Iy);
        if (f_out) {
            const size_t id = (size_t)i * L.Ny + j;
            for (int v = 0; v < 9; v++) f_out[id * 9 + v] = f[v];
        }
    }
    __syncthreads();
    // transposed: thread tx now walks j
#pragma unroll 1
    for (int r = ty; r < 32; r += 8) {
        const int io = ib + r, jo = jb + tx;
        if (io >= i1 || jo >= L.Ny) continue;
        const size_t id = (size_t)io * L.Ny + jo;
        if (rho_out) rho_out[id] = s_rho[r][tx];
        if (u_out) reinterpret_cast<double2*>(u_out)[id] = s_u[r][tx];
        if (fibm_out) reinterpret_cast<double2*>(fibm_out)[id] = s_fi[r][tx];
    }
}

// The arrays GridClass::writeVTK writes (src/Grid.cpp:860-893), in VTK point
// order (x fastest, the device's own order): density rho*Drho, pressure
// ref_P + (rho - rho_p/Drho) c_s^2 Dm / (Dx Dt^2) and velocity u Dx/Dt with a
// zero third component, each in the reference's operation order. `initial`
// selects the state before the first step (as k_export_init).
template <bool CM, class S>
__global__ void k_export_vti(const typename S::T* __restrict__ P, LatDev L, int t, int initial, VtiScale V,
                             double* __restrict__ dens, double* __restrict__ pres, double* __restrict__ vel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    double rho, ux, uy;
    if (initial) {
        rho = 1.0;
        if (L.init_mode == 0) { ux = 0.0; uy = 0.0; }
        else if (L.init_mode == 1) { ux = L.u_in[j * 2]; uy = L.u_in[j * 2 + 1]; }
        else { ux = L.u0x; uy = L.u0y; }
        if (site_type(L, i, j) == LIFE_WALL) { ux = 0.0; uy = 0.0; }
    } else {
        double f[9];
        site_state<CM, S>(P, L, t, i, j, f, rho, ux, uy);
        if (L.force_ibm) {
            const size_t s = (size_t)j * L.pitch + i;
            const double Ix = L.force_ibm[s], Iy = L.force_ibm[L.S + s];
            if (Ix != 0.0 || Iy != 0.0) {
                double Fx, Fy;
                force_xy_of(L, t, i, j, Fx, Fy);
                macroscopic_ibm(f, Fx, Fy, Ix, Iy, rho, ux, uy);
            }
        }
    }
    const size_t id = (size_t)j * L.Nx + i;
    if (dens) dens[id] = rho * V.Drho;
    if (pres) pres[id] = V.ref_P + (rho - V.rho_p / V.Drho) * (V.cs * V.cs) * V.Dm / (V.Dx * (V.Dt * V.Dt));
    if (vel) {
        vel[id * 3] = ux * (V.Dx / V.Dt);
        vel[id * 3 + 1] = uy * (V.Dx / V.Dt);
        vel[id * 3 + 2] = 0.0;
    }
}

// Initial state (before any step) in reference layout.
template <bool CM>
__global__ void k_export_init(LatDev L, double* __restrict__ rho_out, double* __restrict__ u_out,
                                  double* __restrict__ f_out, double* __restrict__ fibm_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= L.Nx) return;
    double ux, uy;
    if (L.init_mode == 0) { ux = 0.0; uy = 0.0; }
    else if (L.init_mode == 1) { ux = L.u_in[j * 2]; uy = L.u_in[j * 2 + 1]; }
    else { ux = L.u0x; uy = L.u0y; }
    if (site_type(L, i, j) == LIFE_WALL) { ux = 0.0; uy = 0.0; }
    const size_t id = (size_t)i * L.Ny + j;
    if (rho_out) rho_out[id] = 1.0;
    if (u_out) { u_out[id * 2] = ux; u_out[id * 2 + 1] = uy; }
    if (f_out)
        for (int v = 0; v < 9; v++) f_out[id * 9 + v] = equilibrium<CM>(v, 1.0, ux, uy);
    if (fibm_out) { fibm_out[id * 2] = 0.0; fibm_out[id * 2 + 1] = 0.0; }
}

// max |u| and NaN flag over the current state (GridClass::writeInfo,
// src/Grid.cpp:562-588). out[0] = max as ordered bits, out[1] = NaN count.
template <bool CM, class S>
__global__ void k_maxvel(const typename S::T* __restrict__ P, LatDev L, int t, unsigned long long* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    double vel = 0.0;
    bool nan = false;
    if (i < L.Nx) {
        double f[9], rho, ux, uy;
        site_state<CM, S>(P, L, t, i, j, f, rho, ux, uy);
        if (L.force_ibm) {
            const size_t s = (size_t)j * L.pitch + i;
            double Ix = L.force_ibm[s], Iy = L.force_ibm[L.S + s];
            if (Ix != 0.0 || Iy != 0.0) {
                double Fx, Fy;
                force_xy_of(L, t, i, j, Fx, Fy);
                macroscopic_ibm(f, Fx, Fy, Ix, Iy, rho, ux, uy);
            }
        }
        vel = sqrt(ux * ux + uy * uy);
        nan = vel != vel;
        if (nan) vel = 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        vel = fmax(vel, __shfl_xor_sync(0xffffffffu, vel, o));
        nan = __any_sync(0xffffffffu, nan);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(vel));
        if (nan) atomicAdd(&out[1], 1ull);
    }
}

// ------------------------------------------------------------ launchers
static inline dim3 grid_of(const LatDev& L) { return dim3((L.Nx + 127) / 128, L.Ny); }

// Instantiates KERNEL for the case's storage form and collision; PTR is the
// population buffer (cast to the storage type), the rest are passed through.
#define LIFE_DISPATCH(KERNEL, CONSTQ, PTR, ...)                                                         \
    do {                                                                                                \
        if (L.prec == LIFE_PREC_F64) {                                                                  \
            if (L.cm) KERNEL<true, StoreF64><<<grid_of(L), 128, 0, s>>>((CONSTQ double*)(PTR), __VA_ARGS__); \
            else KERNEL<false, StoreF64><<<grid_of(L), 128, 0, s>>>((CONSTQ double*)(PTR), __VA_ARGS__);    \
        } else if (L.prec == LIFE_PREC_F32) {                                                           \
            if (L.cm) KERNEL<true, StoreF32><<<grid_of(L), 128, 0, s>>>((CONSTQ float*)(PTR), __VA_ARGS__);  \
            else KERNEL<false, StoreF32><<<grid_of(L), 128, 0, s>>>((CONSTQ float*)(PTR), __VA_ARGS__);     \
        } else {                                                                                        \
            if (L.cm) KERNEL<true, StoreF16><<<grid_of(L), 128, 0, s>>>((CONSTQ __half*)(PTR), __VA_ARGS__); \
            else KERNEL<false, StoreF16><<<grid_of(L), 128, 0, s>>>((CONSTQ __half*)(PTR), __VA_ARGS__);    \
        }                                                                                               \
    } while (0)

template <bool CM, class S>
static cudaError_t init_t(void* B, void* scratch, const LatDev& L, int t0, cudaStream_t s) {
    InitRow<S>* rows = reinterpret_cast<InitRow<S>*>(scratch);
    k_init_rows<CM, S><<<(2 * L.Ny + 127) / 128, 128, 0, s>>>(rows, L, t0);
    k_init_fill<S><<<grid_of(L), 128, 0, s>>>((typename S::T*)B, rows, L);
    return cudaGetLastError();
}

// scratch: device memory for 2 Ny InitRow records (the second population
// buffer, unused before the first step).
cudaError_t launch_init(void* B, void* scratch, const LatDev& L, int t0, cudaStream_t s) {
    if (L.prec == LIFE_PREC_F64) return L.cm ? init_t<true, StoreF64>(B, scratch, L, t0, s) : init_t<false, StoreF64>(B, scratch, L, t0, s);
    if (L.prec == LIFE_PREC_F32) return L.cm ? init_t<true, StoreF32>(B, scratch, L, t0, s) : init_t<false, StoreF32>(B, scratch, L, t0, s);
    return L.cm ? init_t<true, StoreF16>(B, scratch, L, t0, s) : init_t<false, StoreF16>(B, scratch, L, t0, s);
}

cudaError_t launch_interior_f64(const double* A, double* B, const LatDev& L, int t, cudaStream_t s) {
    if (L.site_force) {
        if (L.cm) k_interior_f64<true, true><<<grid_of(L), 128, 0, s>>>(A, B, L, t);
        else k_interior_f64<false, true><<<grid_of(L), 128, 0, s>>>(A, B, L, t);
    } else {
        if (L.cm) k_interior_f64<true, false><<<grid_of(L), 128, 0, s>>>(A, B, L, t);
        else k_interior_f64<false, false><<<grid_of(L), 128, 0, s>>>(A, B, L, t);
    }
    return cudaGetLastError();
}

cudaError_t launch_interior_batch_f64(const BatchLatCase* cases, const int* tile_case, int ntiles, int tile_w,
                                      int tile_h, int grid, int phase, cudaStream_t s) {
    k_interior_batch_f64<<<grid, tile_w, 0, s>>>(cases, tile_case, ntiles, tile_h, phase);
    return cudaGetLastError();
}

int batch_blocks_per_sm_f64(int tile_w) {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_interior_batch_f64, tile_w, 0);
    return n;
}

cudaError_t launch_perimeter(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    if (L.prec != LIFE_PREC_F64) return launch_perimeter_lowp(A, B, L, t, s);
    // one warp per block, spread over the SMs' FP64 units (as the
    // reduced-precision perimeter)
    const int n = 2 * L.Nx + 2 * (L.Ny - 2);
    if (L.cm) k_perimeter<true, StoreF64><<<(n + 31) / 32, 32, 0, s>>>((const double*)A, (double*)B, L, t);
    else k_perimeter<false, StoreF64><<<(n + 31) / 32, 32, 0, s>>>((const double*)A, (double*)B, L, t);
    return cudaGetLastError();
}

cudaError_t launch_outlet(const LatDev& L, double* delU, cudaStream_t s) {
    k_outlet_f64<<<1, 256, 0, s>>>(L, delU);
    return cudaGetLastError();
}

cudaError_t launch_state(void* B, const LatDev& L, int t, const double* rho, const double* u, const double* f,
                         const double* fibm, cudaStream_t s) {
    LIFE_DISPATCH(k_state, , B, L, t, rho, u, f, fibm);
    return cudaGetLastError();
}

cudaError_t launch_export(const void* P, const LatDev& L, int t, bool initial, double* rho, double* u, double* f,
                          double* fibm, cudaStream_t s, int i0, int i1) {
    if (i1 < 0) i1 = L.Nx;
    if (initial) {
        if (L.cm) k_export_init<true><<<grid_of(L), 128, 0, s>>>(L, rho, u, f, fibm);
        else k_export_init<false><<<grid_of(L), 128, 0, s>>>(L, rho, u, f, fibm);
        return cudaGetLastError();
    }
    if (i1 <= i0) return cudaSuccess;
    const dim3 g((i1 - i0 + 31) / 32, (L.Ny + 31) / 32), blk(32, 8);
    if (L.prec == LIFE_PREC_F64) {
        if (L.cm) k_export<true, StoreF64><<<g, blk, 0, s>>>((const double*)P, L, t, rho, u, f, fibm, i0, i1);
        else k_export<false, StoreF64><<<g, blk, 0, s>>>((const double*)P, L, t, rho, u, f, fibm, i0, i1);
    } else if (L.prec == LIFE_PREC_F32) {
        if (L.cm) k_export<true, StoreF32><<<g, blk, 0, s>>>((const float*)P, L, t, rho, u, f, fibm, i0, i1);
        else k_export<false, StoreF32><<<g, blk, 0, s>>>((const float*)P, L, t, rho, u, f, fibm, i0, i1);
    } else {
        if (L.cm) k_export<true, StoreF16><<<g, blk, 0, s>>>((const __half*)P, L, t, rho, u, f, fibm, i0, i1);
        else k_export<false, StoreF16><<<g, blk, 0, s>>>((const __half*)P, L, t, rho, u, f, fibm, i0, i1);
    }
    return cudaGetLastError();
}

cudaError_t launch_export_vti(const void* P, const LatDev& L, int t, bool initial, const VtiScale& V, double* dens,
                              double* pres, double* vel, cudaStream_t s) {
    LIFE_DISPATCH(k_export_vti, const, P, L, t, initial ? 1 : 0, V, dens, pres, vel);
    return cudaGetLastError();
}

cudaError_t launch_maxvel(const void* P, const LatDev& L, int t, unsigned long long* out, cudaStream_t s) {
    LIFE_DISPATCH(k_maxvel, const, P, L, t, out);
    return cudaGetLastError();
}

}  // namespace life
