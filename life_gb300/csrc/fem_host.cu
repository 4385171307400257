// Host side of the flexible bodies: upload of the FEM state built at start-up
// (objects.cpp), the per-step block Gauss-Seidel loop (ObjectsClass::
// objectKernel, reference src/Objects.cpp:26-60) and the FEM accessors.
#include <cuda_runtime.h>

#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "fem_kernels.h"

using namespace life;

namespace life {
// The subiteration loop of one step captured as a graph: a WHILE node whose
// body is one subiteration's kernels; the residual kernel sets the condition.
// Kernel arguments are fixed at capture, so one graph exists per
// (population buffer, parity of t) combination the case uses.
struct FsiGraph {
    cudaGraphExec_t exec = nullptr;
};
struct FemHost {
    FsiDev F{};
    std::vector<FemBodyDev> bodies;   // host copies of the device records
    std::vector<int> hostBody;        // host body index of each flexible body
    int* h_cont = nullptr;            // pinned flag (host-driven loop)
    cudaStream_t cap = nullptr;       // capture stream
    FsiGraph graph[4];
    bool host_loop = false;           // LIFE_FSI_HOSTLOOP=1: read the flag on the host instead
};
}  // namespace life

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

static int falloc(LifeCase* c, void** p, size_t bytes) { return case_dev_alloc(c, p, bytes); }
template <class T>
static int fallocT(LifeCase* c, T** p, size_t n) {
    return falloc(c, (void**)p, sizeof(T) * n);
}
template <class T>
static int upload(LifeCase* c, T** p, const std::vector<T>& h) {
    int rc = fallocT(c, p, h.size());
    if (rc) return rc;
    if (!h.empty()) {
        cudaError_t e = cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "upload");
    }
    return LIFE_OK;
}

static FemHost* fem_of(LifeCase* c) { return c->fem; }

int setup_fem(LifeCase* c) {
    FemHost* H = new FemHost();
    c->fem = H;
    HObjects& o = c->obj;
    FsiDev& F = H->F;
    int rc;
    // body marker ranges (contiguous after de-overlap)
    std::vector<int> start(o.b.size()), count(o.b.size()), flexMarkers;
    for (size_t b = 0; b < o.b.size(); b++) {
        const auto& nodes = o.b[b].nodes;
        start[b] = nodes.empty() ? 0 : nodes[0];
        count[b] = (int)nodes.size();
        for (size_t k = 0; k < nodes.size(); k++)
            if (nodes[k] != start[b] + (int)k) return set_error(LIFE_ERR_GEOMETRY, "body markers are not contiguous");
        if (o.b[b].flex)
            for (int k : nodes) flexMarkers.push_back(k);
    }
    std::vector<int> markerBody(o.m.size());
    for (size_t k = 0; k < o.m.size(); k++) markerBody[k] = o.m[k].body;
    if ((rc = upload(c, &F.flexMarkers, flexMarkers)) || (rc = upload(c, &F.markerBody, markerBody)) ||
        (rc = upload(c, &F.bodyStart, start)) || (rc = upload(c, &F.bodyCount, count)))
        return rc;
    F.nFlexMarkers = (int)flexMarkers.size();
    F.uni = c->p.uni_epsilon;
    F.simDOFs = o.simDOFs;
    const int N = (int)o.m.size();
    if (F.uni) {
        if ((rc = fallocT(c, &F.uniA, (size_t)N * N)) || (rc = fallocT(c, &F.uniB, (size_t)N)) ||
            (rc = fallocT(c, &F.uniPiv, (size_t)N)) || (rc = fallocT(c, &F.uniLmax, (size_t)N)))
            return rc;
    }
    // FEM bodies
    for (size_t b = 0; b < o.b.size(); b++) {
        if (!o.b[b].flex) continue;
        const HFem& f = *o.b[b].fem;
        FemBodyDev D{};
        D.n = f.dofs;
        D.nNodes = f.nNodes;
        D.nEl = f.nEl;
        D.bc = f.bc;
        D.nMark = count[b];
        D.mbase = start[b];
        D.body = (int)b;
        D.L0 = f.L0;
        D.angle0 = f.angle0;
        const int n = f.dofs;
        std::vector<double> pool((size_t)NVEC * n, 0.0);
        const std::vector<double>* src[NVEC] = {&f.U, &f.Udot, &f.Udotdot, &f.U_n, &f.U_nm1, &f.U_nm2, &f.Udot_n,
                                                &f.Udotdot_n, &f.U_km1, &f.R_k, &f.R_km1, &f.R, &f.F, &f.delU};
        for (int v = 0; v < NVEC; v++) {
            for (int i = 0; i < n; i++) pool[(size_t)v * n + i] = (*src[v])[i];
            D.slots[v] = v;
        }
        std::vector<double> node((size_t)f.nNodes * 6);
        for (int k = 0; k < f.nNodes; k++) {
            node[k * 6 + 0] = f.pos0[k * 2];
            node[k * 6 + 1] = f.pos0[k * 2 + 1];
            node[k * 6 + 2] = f.pos[k * 2];
            node[k * 6 + 3] = f.pos[k * 2 + 1];
            node[k * 6 + 4] = f.angle0n[k];
            node[k * 6 + 5] = f.anglen[k];
        }
        std::vector<double> el((size_t)f.nEl * EL_STRIDE, 0.0);
        std::vector<int> fStart(f.nEl + 1, 0), fNode, fEl;
        std::vector<double> fZ;
        for (int e = 0; e < f.nEl; e++) {
            const HElement& h = f.el[e];
            double* r = &el[(size_t)e * EL_STRIDE];
            r[EL_L0] = h.L0;
            r[EL_L] = h.L;
            r[EL_ANG] = h.angle;
            r[EL_A] = h.A;
            r[EL_I] = h.I;
            r[EL_E] = h.E;
            r[EL_RHO] = h.rho;
            r[EL_COS] = h.T[0][0];
            r[EL_SIN] = h.T[0][1];
            for (int q = 0; q < 36; q++) {
                r[EL_M + q] = h.M[q / 6][q % 6];
                r[EL_KL + q] = h.KL[q / 6][q % 6];
            }
            fStart[e] = (int)fNode.size();
            for (const auto& m : h.fmap) {
                fNode.push_back(m.node);
                fEl.push_back(e);
                fZ.push_back(m.z1);
                fZ.push_back(m.z2);
            }
        }
        fStart[f.nEl] = (int)fNode.size();
        D.nfmap = (int)fNode.size();
        if ((rc = upload(c, &D.pool, pool)) || (rc = fallocT(c, &D.lu_cache, fem_cache_doubles(n, D.bc, D.nNodes, D.nEl))) ||
            (rc = upload(c, &D.node, node)) || (rc = upload(c, &D.el, el)) ||
            (rc = fallocT(c, &D.elscr, (size_t)f.nEl * ES_STRIDE)) || (rc = upload(c, &D.fmapStart, fStart)) ||
            (rc = upload(c, &D.fmapEl, fEl)) || (rc = upload(c, &D.fmapNode, fNode)) || (rc = upload(c, &D.fmapZ, fZ)) ||
            (rc = fallocT(c, &D.rgscr, (size_t)D.nfmap * 6)) || (rc = upload(c, &D.mapEl, f.mapEl)) ||
            (rc = upload(c, &D.mapZeta, f.mapZeta)) || (rc = fallocT(c, &D.piv, (size_t)n)) ||
            (rc = fallocT(c, &D.lmax, (size_t)n)) || (rc = fallocT(c, &D.epsA, (size_t)D.nMark * D.nMark)) ||
            (rc = fallocT(c, &D.epsB, (size_t)D.nMark)))
            return rc;
        H->bodies.push_back(D);
        H->hostBody.push_back((int)b);
    }
    F.nFlex = (int)H->bodies.size();
    if ((rc = upload(c, &F.bodies, H->bodies))) return rc;
    // Each FEM CTA holds its body's LU band and matrices in shared memory.
    size_t smem = 0;
    for (const auto& D : H->bodies) smem = std::max(smem, fem_dynamic_smem(D.n, D.bc));
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > (size_t)optin)
        return set_error(LIFE_ERR_INVALID, "a flexible body has too many elements for the shared-memory FEM solve (" +
                                               std::to_string(smem) + " bytes needed)");
    F.fem_smem = smem;
    CK(fem_dynamic_configure(smem));
    F.s = c->d_fsi;
    F.status = c->d_status;
    if ((rc = fallocT(c, &F.cont, 1))) return rc;
    CK(cudaMallocHost(&H->h_cont, sizeof(int)));
    CK(cudaStreamCreateWithFlags(&H->cap, cudaStreamNonBlocking));
    if (const char* v = std::getenv("LIFE_FSI_HOSTLOOP")) H->host_loop = (v[0] == '1');
    F.Dx = c->Dx;
    F.Dt = c->Dt;
    F.Dm = c->Dm;
    F.gravityX = c->p.gravityX;
    F.gravityY = c->p.gravityY;
    F.ref_L = c->p.ref_L;
    F.alpha = c->p.alpha;
    F.delta = c->p.delta;
    F.relaxMax = c->p.relaxMax;
    F.subTol = c->p.subTol;
    F.Nx = c->Nx;
    F.Ny = c->Ny;
    return LIFE_OK;
}

void life::free_fem(LifeCase* c) {
    FemHost* H = fem_of(c);
    if (!H) return;
    for (auto& g : H->graph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (H->cap) cudaStreamDestroy(H->cap);
    if (H->h_cont) cudaFreeHost(H->h_cont);
    delete H;
    c->fem = nullptr;
}

static int build_fsi_graph(LifeCase* c, FemHost* H, int key, int t, const void* A, const LatDev& L) {
    cudaGraph_t graph = nullptr;
    CK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
    if (e == cudaSuccess) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(H->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t el = launch_fsi_subiteration(H->F, c->M, A, L, t, c->Dt / c->Dx, H->cap, nullptr, &h);
            e = cudaStreamEndCapture(H->cap, &body);
            if (el != cudaSuccess) e = el;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&H->graph[key].exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "FSI loop graph");
    return LIFE_OK;
}

// While a batch captures the case's stream, the WHILE node of the loop goes
// straight into the graph being captured: it is added after the capture's
// current dependencies, its body is captured on the case's side stream, and
// the capture continues after the node.
static int embed_fsi_loop(LifeCase* c, FemHost* H, int t, const void* A, const LatDev& L, cudaStream_t stream) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(stream, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(H->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    cudaError_t el = launch_fsi_subiteration(H->F, c->M, A, L, t, c->Dt / c->Dx, H->cap, nullptr, &h);
    cudaError_t e = cudaStreamEndCapture(H->cap, &body);
    if (el != cudaSuccess) return cuda_fail(el, "FSI loop body");
    if (e != cudaSuccess) return cuda_fail(e, "FSI loop body capture");
    size_t nn = 0;
    CK(cudaGraphGetNodes(body, nullptr, &nn));
    c->loop_body_kernels = (int)nn;
    CK(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    c->ibm_launches += 1;
    return LIFE_OK;
}

// The subiteration loop of one step on `stream`; the spread follows in
// ibm_apply().
int fem_fsi_loop(LifeCase* c, int t, const void* A, const LatDev& L, cudaStream_t stream) {
    FemHost* H = fem_of(c);
    cudaError_t e = launch_fsi_begin(H->F, t, stream, c->t_dev, c->t_off);
    if (e != cudaSuccess) return cuda_fail(e, "fsi_begin");
    c->ibm_launches += 1;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(stream, &cs));
    if (cs == cudaStreamCaptureStatusActive) return embed_fsi_loop(c, H, t, A, L, stream);
    if (!H->host_loop) {
        const int key = (A == c->P[0] ? 0 : 2) + (t & 1);
        if (!H->graph[key].exec)
            if (int rc = build_fsi_graph(c, H, key, t, A, L)) return rc;
        e = cudaGraphLaunch(H->graph[key].exec, stream);
        if (e != cudaSuccess) return cuda_fail(e, "FSI loop graph launch");
        c->ibm_launches += 1;
        return LIFE_OK;
    }
    for (int it = 0; it < 20; it++) {
        e = launch_fsi_subiteration(H->F, c->M, A, L, t, c->Dt / c->Dx, stream, &c->ibm_launches);
        if (e != cudaSuccess) return cuda_fail(e, "fsi_subiteration");
        e = cudaMemcpyAsync(H->h_cont, H->F.cont, sizeof(int), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_fail(e, "fsi_loop");
        if (!*H->h_cont) break;
    }
    return LIFE_OK;
}

extern "C" int life_case_get_fem(LifeCase* c, int32_t k, double* U, double* Udot, double* Udotdot, double* U_n,
                                 double* U_nm1, double* R_k, double* el_L, double* el_angle, double* node_pos,
                                 double* node_angle) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    FemHost* H = fem_of(c);
    if (!H || k < 0 || k >= (int)H->bodies.size()) return set_error(LIFE_ERR_INVALID, "no such flexible body");
    FemBodyDev D;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&D, H->F.bodies + k, sizeof D, cudaMemcpyDeviceToHost));
    const int n = D.n;
    auto vecout = [&](int name, double* dst) -> cudaError_t {
        if (!dst) return cudaSuccess;
        return cudaMemcpy(dst, D.pool + (size_t)D.slots[name] * n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    };
    CK(vecout(V_U, U));
    CK(vecout(V_Udot, Udot));
    CK(vecout(V_Udotdot, Udotdot));
    CK(vecout(V_Un, U_n));
    CK(vecout(V_Unm1, U_nm1));
    CK(vecout(V_Rk, R_k));
    std::vector<double> el((size_t)D.nEl * EL_STRIDE), node((size_t)D.nNodes * 6);
    CK(cudaMemcpy(el.data(), D.el, sizeof(double) * el.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(node.data(), D.node, sizeof(double) * node.size(), cudaMemcpyDeviceToHost));
    for (int e = 0; e < D.nEl; e++) {
        if (el_L) el_L[e] = el[(size_t)e * EL_STRIDE + EL_L];
        if (el_angle) el_angle[e] = el[(size_t)e * EL_STRIDE + EL_ANG];
    }
    for (int q = 0; q < D.nNodes; q++) {
        if (node_pos) {
            node_pos[q * 2] = node[q * 6 + 2];
            node_pos[q * 2 + 1] = node[q * 6 + 3];
        }
        if (node_angle) node_angle[q] = node[q * 6 + 5];
    }
    return LIFE_OK;
}

// Reference configuration of flexible body k's nodes (FEMNodeClass pos0 and
// angle0, written to FEM.restart by src/Objects.cpp:1345-1360).
extern "C" int life_case_get_fem0(LifeCase* c, int32_t k, double* node_pos0, double* node_angle0) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    FemHost* H = fem_of(c);
    if (!H || k < 0 || k >= (int)H->bodies.size()) return set_error(LIFE_ERR_INVALID, "no such flexible body");
    FemBodyDev D;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&D, H->F.bodies + k, sizeof D, cudaMemcpyDeviceToHost));
    std::vector<double> node((size_t)D.nNodes * 6);
    CK(cudaMemcpy(node.data(), D.node, sizeof(double) * node.size(), cudaMemcpyDeviceToHost));
    for (int q = 0; q < D.nNodes; q++) {
        if (node_pos0) {
            node_pos0[q * 2] = node[q * 6 + 0];
            node_pos0[q * 2 + 1] = node[q * 6 + 1];
        }
        if (node_angle0) node_angle0[q] = node[q * 6 + 4];
    }
    return LIFE_OK;
}

// The FEM half of ObjectsClass::readRestart (src/Objects.cpp:1055-1175) for
// flexible body k, then setElementTransform of its elements
// (src/Objects.cpp:1195-1200). NULL skips an array.
extern "C" int life_case_set_fem(LifeCase* c, int32_t k, const double* U, const double* Udot, const double* Udotdot,
                                 const double* U_n, const double* U_nm1, const double* R_k, const double* el_L,
                                 const double* el_angle, const double* node_pos0, const double* node_pos,
                                 const double* node_angle0, const double* node_angle) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    FemHost* H = fem_of(c);
    if (!H || k < 0 || k >= (int)H->bodies.size()) return set_error(LIFE_ERR_INVALID, "no such flexible body");
    FemBodyDev D;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&D, H->F.bodies + k, sizeof D, cudaMemcpyDeviceToHost));
    const int n = D.n;
    auto vecin = [&](int name, const double* src) -> cudaError_t {
        if (!src) return cudaSuccess;
        return cudaMemcpy(D.pool + (size_t)D.slots[name] * n, src, sizeof(double) * n, cudaMemcpyHostToDevice);
    };
    CK(vecin(V_U, U));
    CK(vecin(V_Udot, Udot));
    CK(vecin(V_Udotdot, Udotdot));
    CK(vecin(V_Un, U_n));
    CK(vecin(V_Unm1, U_nm1));
    CK(vecin(V_Rk, R_k));
    std::vector<double> el((size_t)D.nEl * EL_STRIDE), node((size_t)D.nNodes * 6);
    CK(cudaMemcpy(el.data(), D.el, sizeof(double) * el.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(node.data(), D.node, sizeof(double) * node.size(), cudaMemcpyDeviceToHost));
    for (int e = 0; e < D.nEl; e++) {
        if (el_L) el[(size_t)e * EL_STRIDE + EL_L] = el_L[e];
        if (el_angle) el[(size_t)e * EL_STRIDE + EL_ANG] = el_angle[e];
    }
    for (int q = 0; q < D.nNodes; q++) {
        if (node_pos0) {
            node[q * 6 + 0] = node_pos0[q * 2];
            node[q * 6 + 1] = node_pos0[q * 2 + 1];
        }
        if (node_pos) {
            node[q * 6 + 2] = node_pos[q * 2];
            node[q * 6 + 3] = node_pos[q * 2 + 1];
        }
        if (node_angle0) node[q * 6 + 4] = node_angle0[q];
        if (node_angle) node[q * 6 + 5] = node_angle[q];
    }
    CK(cudaMemcpy(D.el, el.data(), sizeof(double) * el.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(D.node, node.data(), sizeof(double) * node.size(), cudaMemcpyHostToDevice));
    CK(launch_fem_element_trig(D.el, D.nEl, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LIFE_OK;
}

// The Aitken factor of FEM.restart (src/Objects.cpp:1065-1073).
extern "C" int life_case_set_relax(LifeCase* c, double relax) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    if (!c->d_fsi) return set_error(LIFE_ERR_INVALID, "case has no immersed bodies");
    FsiScalars h{};
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&h, c->d_fsi, sizeof h, cudaMemcpyDeviceToHost));
    h.relax = relax;
    CK(cudaMemcpy(c->d_fsi, &h, sizeof h, cudaMemcpyHostToDevice));
    return LIFE_OK;
}

extern "C" int life_case_get_relax(LifeCase* c, double* relax) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    if (!c->d_fsi) {
        if (relax) *relax = c->p.relaxMax;
        return LIFE_OK;
    }
    FsiScalars h{};
    CK(cudaMemcpyAsync(&h, c->d_fsi, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (relax) *relax = h.relax;
    return LIFE_OK;
}
