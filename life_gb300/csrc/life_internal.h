// Internal state of a LifeCase (host side of the C-ABI).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/life_gb300.h"
#include "ibm_kernels.h"
#include "life_types.h"
#include "objects.h"

namespace life {

constexpr int kStepRing = 4096;   // entries of the per-step scalar ring
constexpr int kStepChunk = 2048;  // steps per table refill (< kStepRing - 2)

// FSI loop scalars kept on the device (ObjectsClass members subIt, relax,
// subRes, subNum, subDen; reference inc/Objects.h:66-71).
struct FsiScalars {
    int subIt;
    int lastNR;
    int t;          // time step being solved
    int pad;
    double relax, subRes, subNum, subDen;
};

struct FemHost;  // fem_host.cu

// Device side of the observables recorder (observe.cu): `capacity` rows of
// `cols` doubles (Fx, Fy, then x, y, vx, vy of each flexible body's last
// marker) and their steps; count[0] rows written, count[1] rows dropped.
struct RecorderDev {
    int every = 0, capacity = 0, cols = 0, n_tips = 0;
    double force_scale = 0.0;
    double* rows = nullptr;
    int* t = nullptr;
    int* count = nullptr;
    int* tip = nullptr;  // marker index of each flexible body's last marker
};

int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);
// Device memory of a case, tracked in c->allocs and c->dev_bytes and
// released by the case's destruction (case_dev_free_all).
int case_dev_alloc(LifeCase* c, void** p, size_t bytes);
void case_dev_free_all(LifeCase* c);

}  // namespace life

struct LifeBatch;  // batch.cu

struct LifeCase {
    LifeCaseParams p{};
    int device = -1;
    int Nx = 0, Ny = 0, pitch = 0;
    long long S = 0;
    double Dx = 0, Dt = 0, Dm = 0, Drho = 0, tau = 0, nu = 0, cs = 0;
    double Fx0 = 0, Fy0 = 0, u0x = 0, u0y = 0;
    int init_mode = 0;
    int t = 0;        // time step of the current state
    int t_set = 0;    // time step at which the state was created or loaded
    bool host_state = false;  // state loaded from host arrays (kept for export)
    std::vector<double> h_rho, h_u, h_f, h_fibm;
    // device lattice state
    void* P[2] = {nullptr, nullptr};  // element type per p.precision
    int elem = 8;     // bytes per stored population
    int cur = 0;      // P[cur] holds P_{t+1}
    double* d_u_in = nullptr;
    double* d_rho_in = nullptr;
    life::StepScalars* d_steps = nullptr;
    int steps_cap = 0, steps_n = 0;
    double* d_outlet_u = nullptr;
    double* d_outlet_f[2] = {nullptr, nullptr};
    double* d_delU = nullptr;
    // densities after alternate steps (WOMERSLEY with gravity only) and the
    // corner velocities after alternate steps (see LatDev)
    bool site_force = false;
    double* d_rho_hist[2] = {nullptr, nullptr};
    double* d_corner_u[2] = {nullptr, nullptr};
    int* d_tile_ctr = nullptr;  // LatDev::tile_ctr
    unsigned long long* d_red = nullptr;
    cudaStream_t stream = nullptr;   // every kernel of the case is ordered on this stream
    cudaStream_t side = nullptr;     // perimeter kernel, forked from and joined to `stream`
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_out = nullptr, ev_done = nullptr, ev_aux = nullptr;
    cudaStream_t aux = nullptr;      // IBM forces (interpolation / FSI loop) beside the lattice step
    // Captured step graphs of this case alone (a one-case batch on the case's
    // own stream), used by life_case_step; and whether steps are launched from
    // the host instead (LIFE_CASE_HOSTLOOP=1 or LIFE_FSI_HOSTLOOP=1).
    LifeBatch* self_batch = nullptr;
    bool host_steps = false;
    size_t dev_bytes = 0;
    std::vector<void*> allocs;
    std::vector<char> alloc_pooled;  // allocs[k] came from the memory pool
    // immersed bodies
    life::Grid0 g0{};
    life::HObjects obj;
    life::MarkerDev M{};
    life::IbmScratch W{};
    life::FemHost* fem = nullptr;
    life::FsiScalars* d_fsi = nullptr;
    int* d_status = nullptr;  // [code, t, ...]
    int status_code = 0, status_t = 0;
    int ibm_launches = 0;     // kernels launched by the IBM/FEM sequence so far
    std::string status_msg;
    // Set while a batch captures this case's step into a graph: kernels then
    // take the step index from *t_dev + t_off (see LatDev).
    const int* t_dev = nullptr;
    int t_off = 0;
    int loop_body_kernels = 0;  // kernels in one pass of a captured FSI loop body
    // observables recorder (life_case_record); rec_gen changes whenever the
    // recorder is set up or removed, so captured step graphs are rebuilt
    life::RecorderDev rec{};
    int rec_gen = 0;
};

namespace life {
LatDev lattice_view(const LifeCase* c, int t);
void batch_free(LifeBatch* b);
// nsteps steps of one case through its cached step graphs (asynchronous);
// with start/stop, CUDA events recorded around them on the case's stream.
int case_graph_steps(LifeCase* c, int nsteps, cudaEvent_t start, cudaEvent_t stop);
// Whether the case's step graphs exist (captured by an earlier run).
bool case_graphs_ready(const LifeCase* c);
// Whether a step of the case is one launch of the reduced-precision step
// kernel (which also takes the boundary sites).
bool case_fused_step(const LifeCase* c);
// Mean device time of the case's interior kernel alone over reps launches.
int case_interior_ms(LifeCase* c, int reps, float* ms);
// Kernel nodes of one captured step of the case (0 before the first capture).
int case_kernels_per_step(LifeCase* c);
void free_fem(LifeCase* c);
// The recorder's kernel for the step ending at t (a no-op without a recorder);
// inside a capture the step is read from c->t_dev.
cudaError_t launch_record(const LifeCase* c, int t, cudaStream_t s);
void free_recorder(LifeCase* c);
int ensure_steps(LifeCase* c, int t0, int n);
// removeOverlapMarkers' pair test on the device (an OverlapScan, objects.h).
int device_overlap_scan(const double* pos, int nm, double Dx, std::vector<std::pair<int, int>>* pairs,
                        std::string* err);
}  // namespace life
