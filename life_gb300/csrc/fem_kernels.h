// Flexible bodies on the device: corotational FEM with Newmark integration,
// the block Gauss-Seidel FSI subiterations and Aitken relaxation
// (reference src/FEMBody.cpp, src/FEMElement.cpp, src/Objects.cpp:26-232).
#pragma once
#include <cuda_runtime.h>

#include "ibm_kernels.h"
#include "life_internal.h"

namespace life {

// Vectors of one FEM body (FEMBodyClass members, reference inc/FEMBody.h:80-107).
// The reference swaps whole vectors (resetValues, predictor, relaxation); the
// device keeps them in a pool and swaps slot indices instead.
enum { V_U, V_Udot, V_Udotdot, V_Un, V_Unm1, V_Unm2, V_Udotn, V_Udotdotn, V_Ukm1, V_Rk, V_Rkm1, V_R, V_F, V_delU,
       NVEC };

// Element record: L0, L, angle, A, I, E, rho, cos(angle), sin(angle), local
// mass matrix (6x6), local linear stiffness (6x6).
enum { EL_L0, EL_L, EL_ANG, EL_A, EL_I, EL_E, EL_RHO, EL_COS, EL_SIN, EL_M = 9, EL_KL = 45, EL_STRIDE = 84 };
// Per-element scratch: global mass (6x6), global stiffness (6x6), global
// internal force (6).
enum { ES_M = 0, ES_K = 36, ES_F = 72, ES_STRIDE = 78 };

// Doubles of FemBodyDev::lu_cache for n DOFs of which bc are constrained.
inline size_t fem_cache_doubles(int n, int bc, int nNodes, int nEl) {
    const size_t nn = (size_t)(n - bc);
    return nn * 16 + nn + 2 * (size_t)n + (nn + 1) / 2 + 3 * (size_t)nNodes + 4 * (size_t)nEl;
}

struct FemBodyDev {
    int n, nNodes, nEl, bc;      // DOFs, nodes, elements, constrained DOFs
    int nMark, mbase, nfmap, body;
    double L0, angle0;
    double* pool;      // [NVEC][n]
    // First Newton iteration of the step, kept by subiteration 0 for the later
    // subiterations (fem_cache_doubles): LU band [nn][16], pivot reciprocals
    // [nn], internal force [n], M * Newmark vector [n], pivots [nn] (ints),
    // and the node positions [nNodes][3] and element values [nEl][4] at U_n
    double* lu_cache;
    double* node;      // [nNodes][6]: pos0x, pos0y, posx, posy, angle0, angle
    double* el;        // [nEl][EL_STRIDE]
    double* elscr;     // [nEl][ES_STRIDE]
    int* fmapStart;    // [nEl+1]
    int* fmapEl;       // [nfmap] element of each force-map entry
    int* fmapNode;     // [nfmap] IBM marker index within the body
    double* fmapZ;     // [nfmap][2]
    double* rgscr;     // [nfmap][6] element load contributions
    int* mapEl;        // [nMark]
    double* mapZeta;   // [nMark]
    int* piv;          // [n]
    int* lmax;         // [n] last row that can hold a multiplier of column c
    double* epsA;      // [nMark][nMark] epsilon system scratch
    double* epsB;      // [nMark] right-hand side / solution
    int slots[NVEC];
    int itNR;
    double resNR, subRes, subNum, subDen;
};

// Everything the FSI kernels need besides the bodies.
struct FsiDev {
    FemBodyDev* bodies;   // [nFlex] device array
    int nFlex;
    int uni;              // UNI_EPSILON: one system over all markers
    int simDOFs;
    int nFlexMarkers;
    int* flexMarkers;     // [nFlexMarkers] global indices of flexible markers
    int* markerBody;      // [nMarkers] owning body index (host body numbering)
    int* bodyStart;       // [nBodies] first marker of each body
    int* bodyCount;       // [nBodies] marker count of each body
    double* uniA;         // [N][N] UNI epsilon scratch
    double* uniB;         // [N]
    int* uniPiv;          // [N]
    int* uniLmax;         // [N]
    FsiScalars* s;        // subIt, relax, residuals
    int* status;          // [code, t]
    int* cont;            // continue flag for the host loop
    double Dx, Dt, Dm, gravityX, gravityY, ref_L, alpha, delta, relaxMax, subTol;
    int Nx, Ny;
    size_t fem_smem;      // dynamic shared memory of k_fem_dynamic (largest body)
};

// Shared memory k_fem_dynamic needs for a body of n DOFs, bc constrained.
size_t fem_dynamic_smem(int n, int bc);
cudaError_t fem_dynamic_configure(size_t smem);
cudaError_t launch_fem_element_trig(double* el, int nEl, cudaStream_t s);

// One subiteration's kernels. With `cond`, the launch is being captured into
// the body of a WHILE graph node and the residual kernel sets its condition;
// the step is then read from the device (F.s->t).
cudaError_t launch_fsi_subiteration(const FsiDev& F, const MarkerDev& M, const void* P, const LatDev& L, int t,
                                    double velScale, cudaStream_t s, int* launches,
                                    const cudaGraphConditionalHandle* cond = nullptr);
// With t_dev (inside a replayed graph) the step is *t_dev + t_off.
cudaError_t launch_fsi_begin(const FsiDev& F, int t, cudaStream_t s, const int* t_dev = nullptr, int t_off = 0);
// Epsilon system of markers [0, n) of M into M.eps, with caller-provided scratch.
cudaError_t launch_epsilon_markers(const MarkerDev& M, int n, double Dx, double* A, double* b, int* piv, int* lmax,
                                   cudaStream_t s);

}  // namespace life

int setup_fem(LifeCase* c);
int fem_fsi_loop(LifeCase* c, int t, const void* A, const life::LatDev& L, cudaStream_t stream);
