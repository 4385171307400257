// Host-side launchers of the lattice kernels.
#pragma once
#include <cuda_runtime.h>

#include "life_types.h"

namespace life {

cudaError_t launch_init_f64(double* B, const LatDev& L, int t0, cudaStream_t s);
cudaError_t launch_step_f64(const double* A, double* B, const LatDev& L, int t, cudaStream_t s);
cudaError_t launch_outlet_f64(const LatDev& L, double* delU, cudaStream_t s);
cudaError_t launch_state_f64(double* B, const LatDev& L, int t, const double* rho, const double* u,
                             const double* f, const double* fibm, cudaStream_t s);
cudaError_t launch_export_f64(const double* P, const LatDev& L, int t, bool initial, double* rho, double* u,
                              double* f, double* fibm, cudaStream_t s);
cudaError_t launch_maxvel_f64(const double* P, const LatDev& L, int t, unsigned long long* out, cudaStream_t s);

}  // namespace life
