// Host-side launchers of the lattice kernels.
#pragma once
#include <cuda_runtime.h>

#include "life_types.h"

namespace life {

// All launchers take the population buffers as untyped pointers; their
// element type follows L.prec (double / float / __half).
cudaError_t launch_init(void* B, void* scratch, const LatDev& L, int t0, cudaStream_t s);
cudaError_t launch_interior_f64(const double* A, double* B, const LatDev& L, int t, cudaStream_t s);
cudaError_t launch_interior_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s);
cudaError_t launch_perimeter(const void* A, void* B, const LatDev& L, int t, cudaStream_t s);
cudaError_t launch_perimeter_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s);
// Perimeter and interior of one reduced-precision case in one launch.
cudaError_t launch_step_lowp(const void* A, void* B, const LatDev& L, int t, cudaStream_t s);
cudaError_t launch_outlet(const LatDev& L, double* delU, cudaStream_t s);
cudaError_t launch_state(void* B, const LatDev& L, int t, const double* rho, const double* u, const double* f,
                         const double* fibm, cudaStream_t s);
// Reference-layout export of columns i0 <= i < i1 (i1 < 0: all columns;
// the initial-state export always covers the whole lattice).
cudaError_t launch_export(const void* P, const LatDev& L, int t, bool initial, double* rho, double* u, double* f,
                          double* fibm, cudaStream_t s, int i0 = 0, int i1 = -1);
// Scalars of GridClass::writeVTK's conversions (src/Grid.cpp:860-893).
struct VtiScale {
    double Drho, ref_P, rho_p, cs, Dm, Dx, Dt;
};
// VTK-order (x fastest) density, pressure and 3-component velocity of the
// state after step t (initial: the state before the first step).
cudaError_t launch_export_vti(const void* P, const LatDev& L, int t, bool initial, const VtiScale& V, double* dens,
                              double* pres, double* vel, cudaStream_t s);
// Bounded waits of the TMA-staged step kernel that gave up (0 normally).
int tma_timeouts();
cudaError_t launch_maxvel(const void* P, const LatDev& L, int t, unsigned long long* out, cudaStream_t s);

// One case of a batched interior launch: its lattice view and buffers for the
// two step parities of a batch (phase 0: P[cur] -> P[cur^1], phase 1: back),
// and its first tile and tiles per row.
struct BatchLatCase {
    LatDev L[2];
    const void* A[2];
    void* B[2];
    int tile0, tiles_x;
};

cudaError_t launch_interior_batch_f64(const BatchLatCase* cases, const int* tile_case, int ntiles, int tile_w,
                                      int tile_h, int grid, int phase, cudaStream_t s);
cudaError_t launch_interior_batch_lowp(int prec, const BatchLatCase* cases, const int* tile_case, int ntiles,
                                       int tile_w, int tile_h, int grid, int phase, cudaStream_t s);
int batch_blocks_per_sm_f64(int tile_w);
int batch_blocks_per_sm_lowp(int prec, int tile_w);

// One lattice step: interior sites, then the boundary-condition perimeter.
// Both read A and write disjoint sites of B.
inline cudaError_t launch_step(const void* A, void* B, const LatDev& L, int t, cudaStream_t s) {
    cudaError_t e = L.prec == LIFE_PREC_F64 ? launch_interior_f64((const double*)A, (double*)B, L, t, s)
                                            : launch_interior_lowp(A, B, L, t, s);
    if (e != cudaSuccess) return e;
    return launch_perimeter(A, B, L, t, s);
}

}  // namespace life
