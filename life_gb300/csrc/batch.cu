// Batched ensemble: many independent cases of uneven size stepped together.
//
// A batch owns ordinary LifeCase objects (each with its own device state) and
// steps them as one unit:
//   * the interior stream-collide of every case runs in ONE persistent launch
//     (k_interior_batch_*): the batch is cut into tiles of tile_w x tile_h
//     sites, case k owning tiles [tile0_k, tile0_k + tiles_k), and each CTA
//     walks the tile list with a grid-stride loop;
//   * the rest of a step (convective outlet, boundary perimeter, IBM interp /
//     FSI subiteration loop / spread) runs per case on the case's own stream,
//     so the cases overlap on the device;
//   * one whole batch step is captured into a CUDA graph, once per step
//     parity (the ping-pong buffers and outlet buffers alternate), and
//     replayed. Kernels read the step index from a per-case device counter
//     that the graph's last kernel advances, so the same two graphs serve
//     every step. A case with flexible bodies contributes its subiteration
//     loop as a conditional WHILE node (its convergence test sets the
//     condition on the device).
// Tile shapes are chosen by life_batch_autotune, which times the batched
// interior kernel for each candidate shape on the batch itself.
//
// Every case computes exactly what it computes alone: the same kernels with
// the same arguments run in the same order within the case.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/life_gb300.h"
#include "lbm_kernels.h"
#include "life_internal.h"

using namespace life;

int ibm_forces(LifeCase* c, int t, const void* A, cudaStream_t s);
int ibm_apply(LifeCase* c, int t, const void* A, void* B, cudaStream_t s);

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

namespace {

__global__ void k_batch_advance(int* __restrict__ tnow, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) tnow[k] += 1;
}

}  // namespace

struct LifeBatch {
    int device = -1;
    int prec = 0;
    int num_sms = 0;
    std::vector<LifeCase*> cases;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_int = nullptr, t0 = nullptr, t1 = nullptr;
    int* d_tnow = nullptr;
    // tiles of the batched interior launch
    int tile_w = 128, tile_h = 2;
    int ntiles = 0, grid = 0;
    long long sites = 0;
    BatchLatCase* d_cases = nullptr;
    int* d_tile_case = nullptr;
    int tile_case_cap = 0;
    // step graphs: exec[p] runs a step whose case state has the parity p
    // relative to (t_base, cur_base) of each case
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int kernel_nodes[2] = {0, 0};
    std::vector<int> t_base, cur_base, rec_gen;
    std::vector<int> ring_end;  // step tables are valid for t < ring_end[k]
    std::string status_msg;
    int status_code = 0;
    bool owns_cases = true;
    bool owns_stream = true;
    std::vector<BatchLatCase> h_cases;  // host copy of the case table
};

static void drop_graphs(LifeBatch* b) {
    for (auto& g : b->exec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

static void free_batch(LifeBatch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    if (b->owns_cases)
        for (LifeCase* c : b->cases) life_case_destroy(c);
    if (b->d_tnow) cudaFree(b->d_tnow);
    if (b->d_cases) cudaFree(b->d_cases);
    if (b->d_tile_case) cudaFree(b->d_tile_case);
    for (cudaEvent_t e : {b->ev_fork, b->ev_int, b->t0, b->t1})
        if (e) cudaEventDestroy(e);
    if (b->stream && b->owns_stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Batch-case table for the state the cases are in now: phase 0 steps
// P[cur] -> P[cur^1] at t+1, phase 1 the step after.
static int upload_case_table(LifeBatch* b) {
    const int n = (int)b->cases.size();
    std::vector<BatchLatCase> h(n);
    int tile0 = 0;
    for (int k = 0; k < n; k++) {
        LifeCase* c = b->cases[k];
        BatchLatCase& C = h[k];
        for (int p = 0; p < 2; p++) {
            C.L[p] = lattice_view(c, c->t + 1 + p);
            C.L[p].t_dev = b->d_tnow + k;
            C.L[p].t_off = 1;
            C.A[p] = c->P[c->cur ^ p];
            C.B[p] = c->P[c->cur ^ p ^ 1];
        }
        C.tile0 = tile0;
        C.tiles_x = (c->Nx + b->tile_w - 1) / b->tile_w;
        tile0 += C.tiles_x * ((c->Ny + b->tile_h - 1) / b->tile_h);
    }
    if (tile0 > b->tile_case_cap) {
        if (b->d_tile_case) cudaFree(b->d_tile_case);
        b->d_tile_case = nullptr;
        b->tile_case_cap = 0;
        CK(cudaMalloc(&b->d_tile_case, sizeof(int) * (size_t)tile0));
        b->tile_case_cap = tile0;
    }
    std::vector<int> tc((size_t)tile0);
    for (int k = 0; k < n; k++) {
        const int end = k + 1 < n ? h[k + 1].tile0 : tile0;
        std::fill(tc.begin() + h[k].tile0, tc.begin() + end, k);
    }
    b->ntiles = tile0;
    const int per_sm = b->prec == LIFE_PREC_F64 ? batch_blocks_per_sm_f64(b->tile_w)
                                                : batch_blocks_per_sm_lowp(b->prec, b->tile_w);
    b->grid = std::max(1, std::min(tile0, b->num_sms * std::max(per_sm, 1)));
    b->h_cases = h;
    CK(cudaMemcpyAsync(b->d_cases, h.data(), sizeof(BatchLatCase) * n, cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_tile_case, tc.data(), sizeof(int) * tc.size(), cudaMemcpyHostToDevice, b->stream));
    std::vector<int> tn(n);
    for (int k = 0; k < n; k++) tn[k] = b->cases[k]->t;
    CK(cudaMemcpyAsync(b->d_tnow, tn.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return LIFE_OK;
}

// One reduced-precision case runs its whole lattice step in one launch when
// the lattice is large enough for the interior to cover the boundary blocks'
// FP64 chains; on smaller lattices the separate perimeter kernel (no register
// cap, so no spills) runs beside the interior instead.
static bool fused_step(const LifeBatch* b) {
    // (a per-site force is taken only by the separate interior kernel)
    return b->cases.size() == 1 && case_fused_step(b->cases[0]);
}

// The interior launch of one batch step. `h`/`d`: the host and device copies
// of the case table (the batch's own, or the scratch table of time_interior).
static cudaError_t launch_batch_interior(LifeBatch* b, int phase, cudaStream_t s, const BatchLatCase* h = nullptr,
                                         const BatchLatCase* d = nullptr) {
    if (!h) h = b->h_cases.data();
    if (!d) d = b->d_cases;
    if (b->cases.size() == 1) {
        // one case: its own interior kernel (one CTA row segment per block);
        // in the reduced-precision forms the launch also takes the perimeter
        const BatchLatCase& C = h[0];
        const LatDev& L = C.L[phase];
        const int t = b->cases[0]->t + 1 + phase;  // ignored: kernels read *L.t_dev + L.t_off
        if (b->prec == LIFE_PREC_F64) return launch_interior_f64((const double*)C.A[phase], (double*)C.B[phase], L, t, s);
        if (fused_step(b)) return launch_step_lowp(C.A[phase], C.B[phase], L, t, s);
        return launch_interior_lowp(C.A[phase], C.B[phase], L, t, s);
    }
    if (b->prec == LIFE_PREC_F64)
        return launch_interior_batch_f64(d, b->d_tile_case, b->ntiles, b->tile_w, b->tile_h, b->grid, phase, s);
    return launch_interior_batch_lowp(b->prec, d, b->d_tile_case, b->ntiles, b->tile_w, b->tile_h, b->grid, phase, s);
}

// Before a step from state t the step tables must hold t+1 and t+2; when they
// do not, they are refilled for the next `n` steps (at most kStepChunk).
static int refill_steps(LifeBatch* b, int n) {
    for (size_t k = 0; k < b->cases.size(); k++) {
        LifeCase* c = b->cases[k];
        if (c->t + 3 <= b->ring_end[k]) continue;
        const int m = std::min(std::max(n, 1), kStepChunk) + 2;
        CK(cudaStreamSynchronize(b->stream));
        if (int rc = ensure_steps(c, c->t, m)) return rc;
        b->ring_end[k] = c->t + m;
    }
    return LIFE_OK;
}

// Captures one batch step at the cases' current state and advances the host
// view of every case by that step (t, buffer parity, IBM scratch parity).
// Per case, the convective outlet and the boundary perimeter run on the
// case's side stream; the interior launch waits only for the outlets (the
// perimeter and the interior both read P[cur] and write disjoint sites of
// P[cur^1], so they overlap). The IBM forces (interpolation, or the FSI
// subiteration loop) read only P[cur] and run beside the lattice step on the
// case's aux stream after the outlet; the spread waits for all of them.
static int capture_step(LifeBatch* b, int phase, cudaGraphExec_t* out, int* kernels) {
    cudaStream_t bs = b->stream;
    const int n = (int)b->cases.size();
    CK(cudaStreamBeginCapture(bs, cudaStreamCaptureModeThreadLocal));
    int rc = LIFE_OK;
    cudaError_t e = cudaEventRecord(b->ev_fork, bs);
    for (int k = 0; k < n && e == cudaSuccess && rc == LIFE_OK; k++) {
        LifeCase* c = b->cases[k];
        c->t_dev = b->d_tnow + k;
        c->t_off = 1;
        const int tt = c->t + 1;
        const LatDev L = lattice_view(c, tt);
        e = cudaStreamWaitEvent(c->side, b->ev_fork, 0);
        // the outlet reads the outlet columns before the interior rewrites them
        if (e == cudaSuccess && L.convective) e = launch_outlet(L, c->d_delU, c->side);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_out, c->side);
        if (e == cudaSuccess && L.convective) e = cudaStreamWaitEvent(bs, c->ev_out, 0);
        const bool fused = fused_step(b);  // perimeter inside the interior launch
        if (e == cudaSuccess && !fused) e = launch_perimeter(c->P[c->cur], c->P[c->cur ^ 1], L, tt, c->side);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_join, c->side);
        if (e == cudaSuccess && c->obj.hasIBM) {
            e = cudaStreamWaitEvent(c->aux, c->ev_out, 0);
            if (e == cudaSuccess) rc = ibm_forces(c, tt, c->P[c->cur], c->aux);
            if (e == cudaSuccess && rc == LIFE_OK) e = cudaEventRecord(c->ev_aux, c->aux);
        }
    }
    if (e == cudaSuccess && rc == LIFE_OK) e = launch_batch_interior(b, phase, bs);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_int, bs);
    for (int k = 0; k < n && e == cudaSuccess && rc == LIFE_OK; k++) {
        LifeCase* c = b->cases[k];
        const int tt = c->t + 1;
        const void* A = c->P[c->cur];
        void* B = c->P[c->cur ^ 1];
        if (c->stream != bs) e = cudaStreamWaitEvent(c->stream, b->ev_int, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_join, 0);
        if (e == cudaSuccess && c->obj.hasIBM) e = cudaStreamWaitEvent(c->stream, c->ev_aux, 0);
        if (e == cudaSuccess && c->obj.hasIBM) rc = ibm_apply(c, tt, A, B, c->stream);
        if (e == cudaSuccess && rc == LIFE_OK) e = launch_record(c, tt, c->stream);
        if (c->stream != bs) {
            if (e == cudaSuccess && rc == LIFE_OK) e = cudaEventRecord(c->ev_done, c->stream);
            if (e == cudaSuccess && rc == LIFE_OK) e = cudaStreamWaitEvent(bs, c->ev_done, 0);
        }
        c->cur ^= 1;
        c->t = tt;
    }
    if (e == cudaSuccess && rc == LIFE_OK) {
        k_batch_advance<<<(n + 127) / 128, 128, 0, bs>>>(b->d_tnow, n);
        e = cudaGetLastError();
    }
    for (LifeCase* c : b->cases) {
        c->t_dev = nullptr;
        c->t_off = 0;
    }
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(bs, &g);
    if (rc != LIFE_OK) {
        // A failure inside a loop body leaves a partly captured conditional
        // node in g; destroying such a graph has crashed the driver, so it is
        // left to the process (error path only).
        return rc;
    }
    if (e == cudaSuccess) e = ee;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (e == cudaSuccess) {
        // kernel nodes at the top level, plus one pass of each loop body
        int kn = 0;
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(g, nodes.data(), &nn);
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType ty;
            cudaGraphNodeGetType(nd, &ty);
            if (ty == cudaGraphNodeTypeKernel) kn++;
        }
        for (LifeCase* c : b->cases) kn += c->loop_body_kernels;
        *kernels = kn;
    }
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "batch step graph");
    return LIFE_OK;
}

static int build_graphs(LifeBatch* b) {
    drop_graphs(b);
    for (LifeCase* c : b->cases) CK(cudaStreamSynchronize(c->stream));
    const int n = (int)b->cases.size();
    if (int rc = refill_steps(b, 4)) return rc;
    if (int rc = upload_case_table(b)) return rc;
    b->t_base.resize(n);
    b->cur_base.resize(n);
    b->rec_gen.resize(n);
    for (int k = 0; k < n; k++) {
        b->t_base[k] = b->cases[k]->t;
        b->cur_base[k] = b->cases[k]->cur;
        b->rec_gen[k] = b->cases[k]->rec_gen;
    }
    int rc = LIFE_OK;
    for (int p = 0; p < 2 && rc == LIFE_OK; p++) rc = capture_step(b, p, &b->exec[p], &b->kernel_nodes[p]);
    // the captures advanced the host view by up to two steps: undo
    for (int k = 0; k < n; k++) {
        LifeCase* c = b->cases[k];
        const int adv = c->t - b->t_base[k];
        c->t = b->t_base[k];
        c->cur = b->cur_base[k];
        if (adv & 1) {
            std::swap(c->W.sites, c->W.sites_prev);
            std::swap(c->W.nsites, c->W.nsites_prev);
        }
    }
    if (rc != LIFE_OK) drop_graphs(b);
    return rc;
}

// Which graph runs the next step, or -1 if the cases' state no longer matches
// the state the graphs were captured from.
static int graph_phase(LifeBatch* b) {
    if (!b->exec[0] || !b->exec[1]) return -1;
    int ph = -1;
    for (size_t k = 0; k < b->cases.size(); k++) {
        const LifeCase* c = b->cases[k];
        if (c->rec_gen != b->rec_gen[k]) return -1;  // recorder set up or removed since the capture
        const int d = (c->t - b->t_base[k]) & 1;
        if ((c->cur ^ b->cur_base[k]) != d) return -1;
        if (ph < 0) ph = d;
        else if (ph != d) return -1;
    }
    return ph;
}

static int check_status(LifeBatch* b) {
    CK(cudaStreamSynchronize(b->stream));
    for (size_t k = 0; k < b->cases.size(); k++) {
        LifeCase* c = b->cases[k];
        if (!c->d_status) continue;
        int h[4];
        CK(cudaMemcpy(h, c->d_status, sizeof(h), cudaMemcpyDeviceToHost));
        if (h[0] != 0 && c->status_code == 0) {
            c->status_code = h[0];
            c->status_t = h[1];
            c->status_msg = "Subiteration scheme hit 20 iterations...exiting";
        }
        if (c->status_code && !b->status_code) {
            b->status_code = c->status_code;
            b->status_msg = "case " + std::to_string(k) + ": " + c->status_msg;
        }
    }
    if (b->status_code) return set_error(b->status_code, b->status_msg);
    return LIFE_OK;
}

static int run_batch(LifeBatch* b, int nsteps, cudaEvent_t start, cudaEvent_t stop, bool check = true) {
    if (graph_phase(b) < 0)
        if (int rc = build_graphs(b)) return rc;
    // the device step counters follow the host view
    {
        const int n = (int)b->cases.size();
        std::vector<int> tn(n);
        for (int k = 0; k < n; k++) tn[k] = b->cases[k]->t;
        CK(cudaMemcpyAsync(b->d_tnow, tn.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    }
    if (start) CK(cudaEventRecord(start, b->stream));
    for (int s = 0; s < nsteps; s++) {
        if (int rc = refill_steps(b, std::min(nsteps - s, kStepChunk))) return rc;
        const int ph = graph_phase(b);
        CK(cudaGraphLaunch(b->exec[ph], b->stream));
        for (LifeCase* c : b->cases) {
            c->t += 1;
            c->cur ^= 1;
            if (c->obj.hasIBM) {
                std::swap(c->W.sites, c->W.sites_prev);
                std::swap(c->W.nsites, c->W.nsites_prev);
            }
        }
    }
    if (stop) CK(cudaEventRecord(stop, b->stream));
    return check ? check_status(b) : LIFE_OK;
}

static int init_batch(LifeBatch* b, int n_cases, cudaStream_t use_stream = nullptr) {
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device);
    cudaError_t e = cudaSuccess;
    if (use_stream) {
        b->stream = use_stream;
        b->owns_stream = false;
    } else {
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_int, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tnow, sizeof(int) * n_cases);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_cases, sizeof(BatchLatCase) * n_cases);
    if (e != cudaSuccess) return cuda_fail(e, "batch setup");
    return LIFE_OK;
}

namespace life {
// A batch over cases the caller keeps (the server's active set). The cases
// must share one storage form; each case's queued work must be complete.
int batch_wrap(const std::vector<LifeCase*>& cases, LifeBatch** out) {
    *out = nullptr;
    if (cases.empty()) return set_error(LIFE_ERR_INVALID, "empty batch");
    LifeBatch* b = new LifeBatch();
    b->owns_cases = false;
    b->prec = cases[0]->p.precision;
    for (LifeCase* c : cases) {
        if (c->p.precision != b->prec) {
            delete b;
            return set_error(LIFE_ERR_INVALID, "all cases of a batch must use the same population storage form");
        }
        b->sites += (long long)c->Nx * c->Ny;
    }
    if (int rc = init_batch(b, (int)cases.size())) {
        free_batch(b);
        return rc;
    }
    b->cases = cases;
    b->ring_end.assign(cases.size(), 0);
    *out = b;
    return LIFE_OK;
}
void batch_free(LifeBatch* b) { free_batch(b); }

static int self_batch(LifeCase* c) {
    if (c->self_batch) return LIFE_OK;
    LifeBatch* b = new LifeBatch();
    b->owns_cases = false;
    b->prec = c->p.precision;
    b->sites = (long long)c->Nx * c->Ny;
    if (int rc = init_batch(b, 1, c->stream)) {
        free_batch(b);
        return rc;
    }
    b->cases = {c};
    b->ring_end.assign(1, 0);
    c->self_batch = b;
    return LIFE_OK;
}

bool case_graphs_ready(const LifeCase* c) {
    return c->self_batch && c->self_batch->exec[0] && c->self_batch->exec[1];
}

bool case_fused_step(const LifeCase* c) {
    return c->p.precision != LIFE_PREC_F64 && !c->site_force && (long long)c->Nx * c->Ny >= (1LL << 22);
}

int case_graph_steps(LifeCase* c, int nsteps, cudaEvent_t start, cudaEvent_t stop) {
    if (int rc = self_batch(c)) return rc;
    return run_batch(c->self_batch, nsteps, start, stop, false);
}

int case_interior_ms(LifeCase* c, int reps, float* ms) {
    if (int rc = self_batch(c)) return rc;
    return life_batch_interior_ms(c->self_batch, reps, ms);
}

int case_kernels_per_step(LifeCase* c) { return c->self_batch ? c->self_batch->kernel_nodes[0] : 0; }
int batch_steps(LifeBatch* b, int nsteps) { return life_batch_step(b, nsteps); }
// Per-case device status after a failed batch run: the index of the first
// failing case (or -1) and its code.
int batch_failed_case(LifeBatch* b, int* code) {
    for (size_t k = 0; k < b->cases.size(); k++)
        if (b->cases[k]->status_code) {
            *code = b->cases[k]->status_code;
            return (int)k;
        }
    return -1;
}
}  // namespace life

extern "C" int life_batch_create(const LifeCaseParams* params, const LifeBodyDesc* bodies, const int32_t* n_bodies,
                                 int32_t n_cases, LifeBatch** out) {
    if (!out) return set_error(LIFE_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_cases <= 0 || !params || !n_bodies) return set_error(LIFE_ERR_INVALID, "bad batch arguments");
    for (int k = 0; k < n_cases; k++)
        if (params[k].precision != params[0].precision)
            return set_error(LIFE_ERR_INVALID, "all cases of a batch must use the same population storage form");
    LifeBatch* b = new LifeBatch();
    b->prec = params[0].precision;
    if (int rc = init_batch(b, n_cases)) {
        free_batch(b);
        return rc;
    }
    size_t off = 0;
    for (int k = 0; k < n_cases; k++) {
        if (n_bodies[k] < 0 || (n_bodies[k] > 0 && !bodies)) {
            free_batch(b);
            return set_error(LIFE_ERR_INVALID, "bad body count");
        }
        LifeCase* c = nullptr;
        int rc = life_case_create(&params[k], bodies ? bodies + off : nullptr, n_bodies[k], &c);
        if (rc) {
            std::string msg = "case " + std::to_string(k) + ": " + life_last_error();
            free_batch(b);
            return set_error(rc, msg);
        }
        b->cases.push_back(c);
        b->sites += (long long)c->Nx * c->Ny;
        off += n_bodies[k];
    }
    b->ring_end.assign(n_cases, 2);
    *out = b;
    return LIFE_OK;
}

extern "C" int life_batch_destroy(LifeBatch* b) {
    free_batch(b);
    return LIFE_OK;
}

extern "C" int life_batch_step(LifeBatch* b, int32_t nsteps) {
    if (!b) return set_error(LIFE_ERR_INVALID, "batch is NULL");
    if (nsteps < 0) return set_error(LIFE_ERR_INVALID, "negative step count");
    if (b->status_code) return set_error(b->status_code, b->status_msg);
    if (nsteps == 0) return LIFE_OK;
    return run_batch(b, nsteps, nullptr, nullptr);
}

extern "C" int life_batch_sync(LifeBatch* b) {
    if (!b) return set_error(LIFE_ERR_INVALID, "batch is NULL");
    return check_status(b);
}

extern "C" int life_batch_case(LifeBatch* b, int32_t k, LifeCase** out) {
    if (!b || !out || k < 0 || k >= (int)b->cases.size()) return set_error(LIFE_ERR_INVALID, "no such case");
    CK(cudaStreamSynchronize(b->stream));
    *out = b->cases[k];
    return LIFE_OK;
}

extern "C" int life_batch_info(LifeBatch* b, LifeBatchInfo* info) {
    if (!b || !info) return set_error(LIFE_ERR_INVALID, "NULL argument");
    LifeBatchInfo I{};
    I.n_cases = (int32_t)b->cases.size();
    I.precision = b->prec;
    I.sites = b->sites;
    I.tile_w = b->tile_w;
    I.tile_h = b->tile_h;
    I.tiles = b->ntiles;
    I.grid = b->grid;
    I.kernel_nodes = b->kernel_nodes[0];
    size_t bytes = 0;
    for (LifeCase* c : b->cases) bytes += c->dev_bytes;
    I.device_bytes = bytes;
    *info = I;
    return LIFE_OK;
}

extern "C" int life_batch_set_tile(LifeBatch* b, int32_t tile_w, int32_t tile_h) {
    if (!b) return set_error(LIFE_ERR_INVALID, "batch is NULL");
    if (tile_w < 32 || tile_w > 256 || tile_w % 32 || tile_h < 1 || tile_h > 64)
        return set_error(LIFE_ERR_INVALID, "tile_w must be 32..256 in steps of 32 and tile_h 1..64");
    CK(cudaStreamSynchronize(b->stream));
    b->tile_w = tile_w;
    b->tile_h = tile_h;
    drop_graphs(b);
    return upload_case_table(b);
}

// Times the batched interior kernel alone (phase 0, `reps` launches after two
// warm-up launches) without touching any case's state: a copy of the case
// table sends every output of the launch (the populations, the outlet
// columns, the per-site densities and corner velocities) to scratch memory,
// so a later export or step sees exactly the state the last step left.
static int time_interior(LifeBatch* b, int reps, float* ms) {
    const int n = (int)b->cases.size();
    std::vector<BatchLatCase> h = b->h_cases;
    size_t total = 0;
    auto take = [&](size_t bytes) {
        const size_t at = total;
        total += (bytes + 255) / 256 * 256;
        return at;
    };
    std::vector<size_t> oP(n), oU(n), oF(n), oC(n), oR(n);
    for (int k = 0; k < n; k++) {
        const LifeCase* c = b->cases[k];
        oP[k] = take((size_t)9 * c->S * c->elem);
        oU[k] = take(sizeof(double) * 6 * c->Ny);
        oF[k] = take(sizeof(double) * 3 * c->Ny);
        oC[k] = take(sizeof(double) * 8);
        oR[k] = c->site_force ? take(sizeof(double) * c->S) : 0;
    }
    const size_t table = take(sizeof(BatchLatCase) * n);
    char* scratch = nullptr;
    CK(cudaMalloc(&scratch, total));
    for (int k = 0; k < n; k++)
        for (int p = 0; p < 2; p++) {
            h[k].B[p] = scratch + oP[k];
            h[k].L[p].outlet_u = reinterpret_cast<double*>(scratch + oU[k]);
            h[k].L[p].outlet_f_next = reinterpret_cast<double*>(scratch + oF[k]);
            h[k].L[p].corner_next = reinterpret_cast<double*>(scratch + oC[k]);
            if (b->cases[k]->site_force) h[k].L[p].rho_next = reinterpret_cast<double*>(scratch + oR[k]);
        }
    BatchLatCase* d = reinterpret_cast<BatchLatCase*>(scratch + table);
    cudaError_t e = cudaMemcpyAsync(d, h.data(), sizeof(BatchLatCase) * n, cudaMemcpyHostToDevice, b->stream);
    for (int r = 0; r < 2 && e == cudaSuccess; r++) e = launch_batch_interior(b, 0, b->stream, h.data(), d);
    if (e == cudaSuccess) e = cudaEventRecord(b->t0, b->stream);
    for (int r = 0; r < reps && e == cudaSuccess; r++) e = launch_batch_interior(b, 0, b->stream, h.data(), d);
    if (e == cudaSuccess) e = cudaEventRecord(b->t1, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_fail(e, "interior timing");
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, b->t0, b->t1));
    *ms = t / reps;
    return LIFE_OK;
}

extern "C" int life_batch_interior_ms(LifeBatch* b, int32_t reps, float* ms) {
    if (!b || !ms || reps <= 0) return set_error(LIFE_ERR_INVALID, "bad arguments");
    if (int rc = refill_steps(b, 4)) return rc;
    if (!b->ntiles)
        if (int rc = upload_case_table(b)) return rc;
    return time_interior(b, reps, ms);
}

extern "C" int life_batch_autotune(LifeBatch* b, int32_t* tile_w, int32_t* tile_h, float* best_ms) {
    if (!b) return set_error(LIFE_ERR_INVALID, "batch is NULL");
    if (int rc = refill_steps(b, 4)) return rc;
    int bw = b->tile_w, bh = b->tile_h;
    float best = 1e30f;
    for (int w : {64, 128, 256})
        for (int h : {1, 2, 4, 8}) {
            b->tile_w = w;
            b->tile_h = h;
            if (int rc = upload_case_table(b)) return rc;
            float ms = 0.f;
            if (int rc = time_interior(b, 5, &ms)) return rc;
            if (ms < best) {
                best = ms;
                bw = w;
                bh = h;
            }
        }
    if (int rc = life_batch_set_tile(b, bw, bh)) return rc;
    if (tile_w) *tile_w = bw;
    if (tile_h) *tile_h = bh;
    if (best_ms) *best_ms = best;
    return LIFE_OK;
}

extern "C" int life_batch_bench_steps(LifeBatch* b, int32_t nsteps, double* total_ms, int32_t* kernels_per_step) {
    if (!b || nsteps <= 0) return set_error(LIFE_ERR_INVALID, "bad arguments");
    if (b->status_code) return set_error(b->status_code, b->status_msg);
    if (graph_phase(b) < 0)
        if (int rc = build_graphs(b)) return rc;
    CK(cudaStreamSynchronize(b->stream));
    int rc = run_batch(b, nsteps, b->t0, b->t1);
    if (rc) return rc;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, b->t0, b->t1));
    if (total_ms) *total_ms = ms;
    if (kernels_per_step) *kernels_per_step = b->kernel_nodes[0];
    return LIFE_OK;
}
