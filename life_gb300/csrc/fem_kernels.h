// Flexible bodies on the device: corotational FEM with Newmark integration,
// the block Gauss-Seidel FSI subiterations and Aitken relaxation.
#pragma once
#include <cuda_runtime.h>

#include "life_internal.h"

namespace life {
struct FemDev {
    int placeholder;
};
}  // namespace life

int setup_fem(LifeCase* c);
int fem_fsi_loop(LifeCase* c, int t, const void* A, const life::LatDev& L);
