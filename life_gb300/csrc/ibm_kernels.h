// Device marker state and the IBM kernel launchers.
#pragma once
#include <cuda_runtime.h>

#include "life_types.h"

namespace life {

// Markers in global order (the reference's iNode order after de-overlap).
struct MarkerDev {
    int n;
    double* pos;    // [n][2]
    double* vel;    // [n][2]
    double* force;  // [n][2]
    double* eps;    // [n]
    double* ds;     // [n]
    int* nsupp;     // [n]
    int* si;        // [n][9]
    int* sj;        // [n][9]
    double* sd;     // [n][9] delta weights
    int4* bbox;     // [n] support bounding box (imin, imax, jmin, jmax)
    int* body;      // [n] owning body
};

// Scratch of the tile-owner spread.
struct IbmScratch {
    double* force_ibm;        // [2][S] dense IBM force of the current step
    long long* sites;         // support sites written this step
    long long* sites_prev;    // support sites of the previous step
    int* nsites;
    int* nsites_prev;
    unsigned* tile_flag;      // [ntx*nty]
    int* tiles;               // touched tiles
    int* ntiles;
    int ntx, nty, max_tiles;
    // Bodies as contiguous marker ranges [body_start[b], body_start[b+1])
    // and the bounding box of their support this step (imin, imax, jmin,
    // jmax): a tile of the spread scans only the bodies whose box reaches it.
    int nbodies;
    const int* body_start;    // [nbodies + 1]
    const int* box_of;        // [n] the range of each marker
    int4* body_box;           // [nbodies]
};

// Close marker pairs of removeOverlapMarkers (appended unordered, see
// k_overlap_pairs).
cudaError_t launch_overlap_pairs(const double* pos, int nm, double Dx, int* count, int2* out, int cap,
                                 cudaStream_t s);
// Population buffers are untyped; their element type follows L.prec.
// With t_dev, the step is read from device memory when the kernel runs.
cudaError_t launch_ibm_interp(const void* P, const LatDev& L, int t, const MarkerDev& M, double velScale,
                              cudaStream_t s, const int* t_dev = nullptr);
cudaError_t launch_ibm_spread(const void* A, void* B, const LatDev& L, int t, const MarkerDev& M,
                              const IbmScratch& W, cudaStream_t s);

}  // namespace life
