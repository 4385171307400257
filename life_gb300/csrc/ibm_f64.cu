// Immersed-boundary kernels (FP64), rigid and flexible markers.
//
//   k_ibm_interp    one thread per marker: rho and rho*u at the marker's
//                   support sites (reconstructed from P_t exactly as the step
//                   kernel computed them), then the direct force
//                   (IBMNodeClass::interpolate + forceCalc,
//                   reference src/IBMNode.cpp:26-58)
//   k_ibm_clear     zero last step's IBM force at its support sites
//   k_ibm_mark      list the 16x16 lattice tiles touched by any support
//   k_ibm_spread    one CTA per touched tile: every site of the tile sums the
//                   contributions of the markers that reach it in marker order
//                   (the reference's ORDERED reduction, src/IBMNode.cpp:61-94)
//                   without atomics, applies the IBM velocity correction
//                   (updateMacroscopic, src/IBMNode.cpp:97-136) and collides
//                   the site again for the next step with the IBM force.
#include <cuda_runtime.h>

#include "collide_cm.cuh"
#include "ibm_kernels.h"
#include "lbm_device.cuh"

namespace life {

constexpr int TILE = 16;

// One warp per marker: lane s reconstructs support site s, and every lane
// then adds the nsupp terms in support order (the reference's loop), so the
// sums are formed exactly as in a sequential loop while the nine site states
// are computed side by side.
template <bool CM, class S>
__global__ void __launch_bounds__(128) k_ibm_interp(const typename S::T* __restrict__ P, LatDev L, int t, MarkerDev M,
                                                    double velScale, const int* __restrict__ t_dev) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= M.n) return;  // uniform per warp
    t = t_dev ? *t_dev : step_t(L, t);  // inside a replayed graph the step comes from the device
    const int ns = M.nsupp[k];
    double tr = 0.0, tx = 0.0, ty = 0.0;
    int i = 0, j = 0;
    if (lane < ns) {
        i = M.si[k * 9 + lane];
        j = M.sj[k * 9 + lane];
        const double d = M.sd[k * 9 + lane];
        double f[9], rho, ux, uy;
        site_state<CM, S>(P, L, t, i, j, f, rho, ux, uy);
        tr = rho * d * 1.0 * 1.0;
        tx = rho * ux * d * 1.0 * 1.0;
        ty = rho * uy * d * 1.0 * 1.0;
    }
    double iRho = 0.0, iMx = 0.0, iMy = 0.0;
    for (int q = 0; q < ns; q++) {
        iRho += __shfl_sync(0xffffffffu, tr, q);
        iMx += __shfl_sync(0xffffffffu, tx, q);
        iMy += __shfl_sync(0xffffffffu, ty, q);
    }
    const bool act = lane < ns;
    const int imin = __reduce_min_sync(0xffffffffu, act ? i : (1 << 30));
    const int imax = __reduce_max_sync(0xffffffffu, act ? i : -(1 << 30));
    const int jmin = __reduce_min_sync(0xffffffffu, act ? j : (1 << 30));
    const int jmax = __reduce_max_sync(0xffffffffu, act ? j : -(1 << 30));
    if (lane == 0) {
        const double sc = velScale * iRho;
        M.force[k * 2 + 0] = 2.0 * (sc * M.vel[k * 2 + 0] - iMx);
        M.force[k * 2 + 1] = 2.0 * (sc * M.vel[k * 2 + 1] - iMy);
        M.bbox[k] = make_int4(imin, imax, jmin, jmax);
    }
}

__global__ void k_ibm_clear(IbmScratch W, LatDev L) {
    const int n = *W.nsites_prev;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const long long s = W.sites_prev[q];
        W.force_ibm[s] = 0.0;
        W.force_ibm[L.S + s] = 0.0;
    }
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < W.nbodies; b += gridDim.x * blockDim.x)
        W.body_box[b] = make_int4(0x7fffffff, -0x7fffffff, 0x7fffffff, -0x7fffffff);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *W.nsites = 0;
        *W.ntiles = 0;
    }
}

__global__ void k_ibm_mark(MarkerDev M, IbmScratch W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M.n) return;
    const int ns = M.nsupp[k];
    for (int s = 0; s < ns; s++) {
        const int tile = (M.sj[k * 9 + s] / TILE) * W.ntx + (M.si[k * 9 + s] / TILE);
        if (atomicCAS(&W.tile_flag[tile], 0u, 1u) == 0u) W.tiles[atomicAdd(W.ntiles, 1)] = tile;
    }
    if (ns > 0) {
        const int4 bb = M.bbox[k];
        int4* box = W.body_box + W.box_of[k];
        atomicMin(&box->x, bb.x);
        atomicMax(&box->y, bb.y);
        atomicMin(&box->z, bb.z);
        atomicMax(&box->w, bb.w);
    }
}

template <bool CM, class S>
__global__ void __launch_bounds__(256) k_ibm_spread(const typename S::T* __restrict__ A, typename S::T* __restrict__ B,
                                                    LatDev L, int t, MarkerDev M, IbmScratch W) {
    __shared__ int list[256];
    __shared__ int warp_cnt[8];
    // support tables and force factors of the compacted markers
    __shared__ int s_ij[256][9];
    __shared__ double s_d[256][9];
    __shared__ double s_fx[256], s_fy[256];
    __shared__ int s_ns[256];
    // touched sites of the tile, compacted onto the first warps
    __shared__ int s_tij[256];
    __shared__ double s_tax[256], s_tay[256];
    __shared__ int s_nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    t = step_t(L, t);
    const int ntiles = *W.ntiles;
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
        const int tile = W.tiles[q];
        const int ti0 = (tile % W.ntx) * TILE, tj0 = (tile / W.ntx) * TILE;
        const int i = ti0 + (tid % TILE), j = tj0 + (tid / TILE);
        double ax = 0.0, ay = 0.0;
        bool touched = false;
        // bodies in body order, markers of a body in marker order: the
        // contributions to a site are summed in global marker order
        for (int bi = 0; bi < W.nbodies; bi++) {
          const int4 box = W.body_box[bi];
          if (box.x > ti0 + TILE - 1 || box.y < ti0 || box.z > tj0 + TILE - 1 || box.w < tj0) continue;
          const int kend = W.body_start[bi + 1];
          for (int c0 = W.body_start[bi]; c0 < kend; c0 += 256) {
            const int k = c0 + tid;
            bool hit = false;
            if (k < kend) {
                const int4 bb = M.bbox[k];
                hit = bb.x <= ti0 + TILE - 1 && bb.y >= ti0 && bb.z <= tj0 + TILE - 1 && bb.w >= tj0;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) warp_cnt[warp] = __popc(bal);
            __syncthreads();
            int off = 0, cnt = 0;
            for (int w = 0; w < 8; w++) {
                if (w < warp) off += warp_cnt[w];
                cnt += warp_cnt[w];
            }
            if (hit) {
                // stage this marker's support (site packed as j*65536 + i)
                const int r = off + __popc(bal & ((1u << lane) - 1u));
                list[r] = k;
                const int ns = M.nsupp[k];
                s_ns[r] = ns;
                for (int s = 0; s < 9; s++) {
                    s_ij[r][s] = s < ns ? (M.sj[k * 9 + s] << 16) | M.si[k * 9 + s] : -1;
                    s_d[r][s] = M.sd[k * 9 + s];
                }
                s_fx[r] = M.force[k * 2 + 0];
                s_fy[r] = M.force[k * 2 + 1];
            }
            __syncthreads();
            // Marker order within the chunk is preserved by the ordered compaction.
            const int me = (j << 16) | i;
            for (int r = 0; r < cnt; r++) {
                const int ns = s_ns[r];
                for (int s = 0; s < ns; s++)
                    if (s_ij[r][s] == me) {
                        const int m = list[r];
                        const double d = s_d[r][s];
                        const double e = M.eps[m], ds = M.ds[m];
                        ax += s_fx[r] * e * ds * 1.0 * d;
                        ay += s_fy[r] * e * ds * 1.0 * d;
                        touched = true;
                        break;
                    }
            }
            __syncthreads();
          }
        }
        if (tid == 0) {
            W.tile_flag[tile] = 0u;
            s_nt = 0;
        }
        __syncthreads();
        {
            const bool mine = touched && i < L.Nx && j < L.Ny;
            const unsigned bal = __ballot_sync(0xffffffffu, mine);
            int base = 0;
            if (lane == 0 && bal) base = atomicAdd(&s_nt, __popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (mine) {
                const int r = base + __popc(bal & ((1u << lane) - 1u));
                s_tij[r] = (j << 16) | i;
                s_tax[r] = ax;
                s_tay[r] = ay;
            }
        }
        __syncthreads();
        // the long FP64 chains (state, velocity correction, collision) on as
        // few warps as there are touched sites
        for (int r = tid; r < s_nt; r += blockDim.x) {
            const int i = s_tij[r] & 0xffff, j = s_tij[r] >> 16;
            const double ax = s_tax[r], ay = s_tay[r];
            const long long s = (long long)j * L.pitch + i;
            W.force_ibm[s] = ax;
            W.force_ibm[L.S + s] = ay;
            W.sites[atomicAdd(W.nsites, 1)] = s;
            double f[9], rho, ux, uy, Fx, Fy;
            site_state<CM, S>(A, L, t, i, j, f, rho, ux, uy);
            force_xy_of(L, t, i, j, Fx, Fy);
            macroscopic_ibm(f, Fx, Fy, ax, ay, rho, ux, uy);
            store_history(L, site_type(L, i, j), i, j, rho, ux, uy);
            if (L.convective && i >= L.Nx - 3) {
                const int c = i - (L.Nx - 3);
                L.outlet_u[((size_t)c * L.Ny + j) * 2 + 0] = ux;
                L.outlet_u[((size_t)c * L.Ny + j) * 2 + 1] = uy;
            }
            double Gx, Gy, fs[9];
            force_xy_next(L, t + 1, rho, Gx, Gy);
            collide<CM>(f, rho, ux, uy, Gx + ax, Gy + ay, L.omega, L.cs, fs);
#pragma unroll
            for (int v = 0; v < 9; v++) B[(size_t)v * L.S + s] = S::save(fs[v], v);
        }
        __syncthreads();
    }
}

// ObjectsClass::removeOverlapMarkers (src/Objects.cpp:873-884): every marker
// pair n1 < n2 whose distance is below half a lattice spacing, with the
// reference's arithmetic (sum of squares from +0, square root, division).
// Block n1 (grid-stride) tests n2 > n1 on its threads; hits are appended in
// any order (the host sorts them) while the count stays within cap, and the
// count is returned in full so the host can retry with a larger list.
__global__ void k_overlap_pairs(const double* __restrict__ pos, int nm, double Dx, int* __restrict__ count,
                                int2* __restrict__ out, int cap) {
    for (int n1 = blockIdx.x; n1 < nm; n1 += gridDim.x) {
        const double x1 = pos[2 * n1], y1 = pos[2 * n1 + 1];
        for (int n2 = n1 + 1 + (int)threadIdx.x; n2 < nm; n2 += blockDim.x) {
            const double d0 = x1 - pos[2 * n2], d1 = y1 - pos[2 * n2 + 1];
            double dd = 0.0;
            dd += d0 * d0;
            dd += d1 * d1;
            if (sqrt(dd) / Dx < 0.5) {
                const int k = atomicAdd(count, 1);
                if (k < cap) out[k] = make_int2(n1, n2);
            }
        }
    }
}

cudaError_t launch_overlap_pairs(const double* pos, int nm, double Dx, int* count, int2* out, int cap,
                                 cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = nm < 8 * sms ? (nm > 0 ? nm : 1) : 8 * sms;
    k_overlap_pairs<<<grid, 256, 0, s>>>(pos, nm, Dx, count, out, cap);
    return cudaGetLastError();
}

// ------------------------------------------------------------ launchers
#define IBM_DISPATCH(KERNEL, GRID, BLOCK, ...)                                                             \
    do {                                                                                                   \
        if (L.prec == LIFE_PREC_F64) {                                                                     \
            if (L.cm) KERNEL<true, StoreF64><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                          \
            else KERNEL<false, StoreF64><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                              \
        } else if (L.prec == LIFE_PREC_F32) {                                                              \
            if (L.cm) KERNEL<true, StoreF32><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                          \
            else KERNEL<false, StoreF32><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                              \
        } else {                                                                                           \
            if (L.cm) KERNEL<true, StoreF16><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                          \
            else KERNEL<false, StoreF16><<<GRID, BLOCK, 0, s>>>(__VA_ARGS__);                              \
        }                                                                                                  \
    } while (0)

template <class T>
struct TypedPtr {
    const void* p;
    template <class U>
    operator const U*() const { return (const U*)p; }
    template <class U>
    operator U*() const { return (U*)const_cast<void*>(p); }
};

cudaError_t launch_ibm_interp(const void* P, const LatDev& L, int t, const MarkerDev& M, double velScale,
                              cudaStream_t s, const int* t_dev) {
    if (M.n == 0) return cudaSuccess;
    const int nb = (M.n + 3) / 4;  // one warp per marker
    TypedPtr<void> Pp{P};
    IBM_DISPATCH(k_ibm_interp, nb, 128, Pp, L, t, M, velScale, t_dev);
    return cudaGetLastError();
}

cudaError_t launch_ibm_spread(const void* A, void* B, const LatDev& L, int t, const MarkerDev& M,
                              const IbmScratch& W, cudaStream_t s) {
    k_ibm_clear<<<8, 256, 0, s>>>(W, L);
    if (M.n > 0) {
        k_ibm_mark<<<(M.n + 127) / 128, 128, 0, s>>>(M, W);
        // four CTAs per SM of this device, at most one per tile
        static int sms[64] = {0};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev >= 0 && dev < 64 && sms[dev] == 0) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
        const int nsm = (dev >= 0 && dev < 64 && sms[dev] > 0) ? sms[dev] : 1;
        int grid = W.max_tiles < 4 * nsm ? W.max_tiles : 4 * nsm;
        if (grid < 1) grid = 1;
        TypedPtr<void> Ap{A}, Bp{B};
        IBM_DISPATCH(k_ibm_spread, grid, 256, Ap, Bp, L, t, M, W);
    }
    return cudaGetLastError();
}

}  // namespace life
