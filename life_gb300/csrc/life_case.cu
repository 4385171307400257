// C-ABI implementation: case lifecycle, time stepping and field access.
//
// One LifeCase owns its device state on the device that was current when it
// was created, and one CUDA stream on which every kernel of the case runs in
// order. The state after step t is kept as P_{t+1} (post-collision
// populations, structure of arrays) plus the small side buffers the next step
// reads; see lbm_device.cuh.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/life_gb300.h"
#include "ibm_kernels.h"
#include "lbm_kernels.h"
#include "life_internal.h"
#include "objects.h"

using namespace life;

namespace {
thread_local std::string g_err;
const double PI = 3.14159265358979323846;
}  // namespace

namespace life {
int set_error(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* where) {
    return set_error(LIFE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
}  // namespace life

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

extern "C" int life_abi_version(void) { return LIFE_ABI_VERSION; }
extern "C" const char* life_last_error(void) { return g_err.c_str(); }

// The large buffers of a case (population planes, force fields: 1 MiB and
// up) come from the device's stream-ordered memory pool, set to keep what is
// freed: a case created after another was destroyed (a served request, a
// batch rebuilt) reuses that memory instead of mapping new pages. Allocation
// and release are ordered on one allocation stream per device; each
// allocation is complete before it is handed out, and a case's memory is
// released only after every stream that used it has drained. The many small buffers (per-body arrays) use cudaMalloc,
// which needs no synchronisation per allocation; so do devices without
// memory pools.
namespace {
struct DevicePool {
    bool init = false, pooled = false;
    cudaStream_t s = nullptr;
};
DevicePool g_pools[64];
std::mutex g_pool_mu;

DevicePool* device_pool(int dev) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    DevicePool& P = g_pools[dev];
    if (!P.init) {
        P.init = true;
        int ok = 0;
        if (cudaDeviceGetAttribute(&ok, cudaDevAttrMemoryPoolsSupported, dev) == cudaSuccess && ok) {
            cudaMemPool_t pool;
            unsigned long long keep = ~0ull;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess &&
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess &&
                cudaStreamCreateWithFlags(&P.s, cudaStreamNonBlocking) == cudaSuccess)
                P.pooled = true;
        }
        cudaGetLastError();
    }
    return &P;
}
}  // namespace

int life::case_dev_alloc(LifeCase* c, void** p, size_t bytes) {
    if (!bytes) bytes = 8;
    int dev = 0;
    cudaGetDevice(&dev);
    DevicePool* P = device_pool(dev);
    cudaError_t e;
    const bool pooled = P && P->pooled && bytes >= (1u << 20);
    if (pooled) {
        e = cudaMallocAsync(p, bytes, P->s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(P->s);
    } else {
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? LIFE_ERR_NOMEM : LIFE_ERR_CUDA,
                         std::string("device allocation (") + std::to_string(bytes) + " bytes): " +
                             cudaGetErrorString(e));
    }
    c->allocs.push_back(*p);
    c->alloc_pooled.push_back(pooled ? 1 : 0);
    c->dev_bytes += bytes;
    return LIFE_OK;
}

// Called with the case's device current and every stream that used the
// case's memory idle.
void life::case_dev_free_all(LifeCase* c) {
    int dev = 0;
    cudaGetDevice(&dev);
    DevicePool* P = device_pool(dev);
    for (size_t k = 0; k < c->allocs.size(); k++) {
        void* p = c->allocs[k];
        if (!p) continue;
        if (c->alloc_pooled[k] && P && P->pooled) cudaFreeAsync(p, P->s);
        else cudaFree(p);
    }
    c->allocs.clear();
    c->alloc_pooled.clear();
}

static int dev_alloc(LifeCase* c, void** p, size_t bytes) { return case_dev_alloc(c, p, bytes); }

template <class T>
static int dev_alloc_t(LifeCase* c, T** p, size_t count) {
    return dev_alloc(c, (void**)p, sizeof(T) * (count ? count : 1));
}

// Per-step scalars for absolute steps [t0, t0+n): inlet ramp
// (GridClass::getRampCoefficient, src/Grid.cpp:548-556) and the Womersley force
// (src/Grid.cpp:52-62), both with the C library's cos() as in the reference.
// The table is a ring of kStepRing entries (step t at t % kStepRing) with a
// fixed address, so captured graphs stay valid; n must not exceed the ring.
int life::ensure_steps(LifeCase* c, int t0, int n) {
    if (n > kStepRing) return set_error(LIFE_ERR_INVALID, "step table request larger than its ring");
    if (!c->d_steps) {
        if (int rc = dev_alloc_t(c, &c->d_steps, (size_t)kStepRing)) return rc;
        c->steps_cap = kStepRing;
    }
    const LifeCaseParams& p = c->p;
    std::vector<StepScalars> h(n);
    for (int k = 0; k < n; k++) {
        const int t = t0 + k;
        StepScalars s{};
        s.ramp = 1.0;
        if (p.has_inlet_ramp && c->Dt * t <= p.inlet_ramp) s.ramp = (1.0 - std::cos(PI * c->Dt * t / p.inlet_ramp)) / 2.0;
        if (p.has_womersley) {
            const double ph = std::cos(2.0 * PI * t * c->Dt /
                                       ((p.height_p * p.height_p * PI) / (2.0 * (p.womersley * p.womersley) * p.nu_p)));
            const double sc = (c->Dx * c->Dt) * (c->Dx * c->Dt);
            s.fx = (0.0 + p.dpdx * ph) * sc / c->Dm;
            s.fy = (0.0 + p.dpdy * ph) * sc / c->Dm;
            s.fx_f = (float)s.fx;
            s.fy_f = (float)s.fy;
            s.ax = p.dpdx * ph;
            s.ay = p.dpdy * ph;
            s.ax_f = (float)s.ax;
            s.ay_f = (float)s.ay;
        }
        h[k] = s;
    }
    // copy in at most two contiguous pieces of the ring
    const int first = t0 % kStepRing;
    const int n1 = n < kStepRing - first ? n : kStepRing - first;
    CK(cudaMemcpyAsync(c->d_steps + first, h.data(), sizeof(StepScalars) * n1, cudaMemcpyHostToDevice, c->stream));
    if (n1 < n)
        CK(cudaMemcpyAsync(c->d_steps, h.data() + n1, sizeof(StepScalars) * (n - n1), cudaMemcpyHostToDevice,
                           c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->steps_n = n;
    return LIFE_OK;
}

LatDev life::lattice_view(const LifeCase* c, int t) {
    LatDev L{};
    L.Nx = c->Nx;
    L.Ny = c->Ny;
    L.pitch = c->pitch;
    L.S = c->S;
    L.wall[0] = c->p.wall_left;
    L.wall[1] = c->p.wall_right;
    L.wall[2] = c->p.wall_bottom;
    L.wall[3] = c->p.wall_top;
    L.cm = c->p.central_moments;
    L.prec = c->p.precision;
    L.womersley = c->p.has_womersley;
    L.convective = c->p.wall_right == LIFE_CONVECTIVE;
    L.has_ibm = c->obj.hasIBM;
    L.omega = c->p.omega;
    L.cs = c->cs;
    L.Fx0 = c->Fx0;
    L.Fy0 = c->Fy0;
    L.omega_f = (float)c->p.omega;
    L.Fx0_f = (float)c->Fx0;
    L.Fy0_f = (float)c->Fy0;
    L.u0x = c->u0x;
    L.u0y = c->u0y;
    L.init_mode = c->init_mode;
    L.steps_cap = kStepRing;
    L.steps = c->d_steps;
    L.u_in = c->d_u_in;
    L.rho_in = c->d_rho_in;
    L.outlet_u = c->d_outlet_u;
    L.outlet_f_prev = c->d_outlet_f[(t - 1) & 1];
    L.outlet_f_next = c->d_outlet_f[t & 1];
    L.delU = c->d_delU;
    L.force_ibm = c->W.force_ibm;
    L.t_dev = c->t_dev;
    L.t_off = c->t_off;
    L.site_force = c->site_force;
    L.Drho = c->Drho;
    L.gx = c->p.gravityX;
    L.gy = c->p.gravityY;
    L.fsc = (c->Dx * c->Dt) * (c->Dx * c->Dt);
    L.Dm = c->Dm;
    L.Drho_f = (float)c->Drho;
    L.gx_f = (float)c->p.gravityX;
    L.gy_f = (float)c->p.gravityY;
    L.fscdm_f = (float)(L.fsc / c->Dm);
    L.rho_prev = c->d_rho_hist[(t - 1) & 1];
    L.rho_next = c->d_rho_hist[t & 1];
    L.corner_prev = c->d_corner_u[(t - 1) & 1];
    L.corner_next = c->d_corner_u[t & 1];
    L.tile_ctr = c->d_tile_ctr;
    return L;
}

static int validate(const LifeCaseParams* p) {
    if (!p) return set_error(LIFE_ERR_INVALID, "params is NULL");
    if (p->Nx < 4 || p->Ny < 4) return set_error(LIFE_ERR_INVALID, "lattice must be at least 4 x 4 sites");
    if (p->Ny > 65535) return set_error(LIFE_ERR_INVALID, "Ny above 65535 is not supported");
    for (int w : {p->wall_left, p->wall_right, p->wall_bottom, p->wall_top})
        if (w < LIFE_FLUID || w > LIFE_CONVECTIVE) return set_error(LIFE_ERR_INVALID, "unknown wall type");
    if (p->wall_left == LIFE_CONVECTIVE || p->wall_bottom == LIFE_CONVECTIVE || p->wall_top == LIFE_CONVECTIVE)
        return set_error(LIFE_ERR_INVALID, "Currently convective BC only supported for right boundary...exiting");
    if (p->wall_right == LIFE_CONVECTIVE && p->Nx < 4)
        return set_error(LIFE_ERR_INVALID, "convective outlet needs at least 4 columns");
    if (p->precision != LIFE_PREC_F64 && p->precision != LIFE_PREC_F32 && p->precision != LIFE_PREC_F16)
        return set_error(LIFE_ERR_INVALID, "unknown precision");
    if (p->omega <= 0.0) return set_error(LIFE_ERR_INVALID, "omega must be positive");
    return LIFE_OK;
}

static void free_case(LifeCase* c) {
    if (!c) return;
    int prev = -1;
    cudaGetDevice(&prev);
    if (c->device >= 0) cudaSetDevice(c->device);
    // the case's own streams drain before its memory returns to the pool. A
    // batch that steps the case (a user batch, a server group) synchronises
    // its stream before it lets go of its cases, so no other work can still
    // use the memory. (No device-wide synchronisation: another thread may be
    // capturing a graph.)
    for (cudaStream_t s : {c->stream, c->side, c->aux})
        if (s) cudaStreamSynchronize(s);
    if (c->self_batch) batch_free(c->self_batch);
    free_recorder(c);
    free_fem(c);
    case_dev_free_all(c);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_out) cudaEventDestroy(c->ev_out);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    if (c->ev_aux) cudaEventDestroy(c->ev_aux);
    if (c->aux) {
        cudaStreamSynchronize(c->aux);
        cudaStreamDestroy(c->aux);
    }
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (prev >= 0) cudaSetDevice(prev);
    delete c;
}

int upload_markers(LifeCase* c);
int setup_fem(LifeCase* c);
int ibm_step(LifeCase* c, int t, const void* A, void* B);

extern "C" int life_case_create(const LifeCaseParams* params, const LifeBodyDesc* bodies, int32_t n_bodies,
                                LifeCase** out) {
    if (!out) return set_error(LIFE_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (int rc = validate(params)) return rc;
    if (n_bodies < 0 || (n_bodies > 0 && !bodies)) return set_error(LIFE_ERR_INVALID, "bad body list");
    LifeCase* c = new LifeCase();
    c->p = *params;
    const LifeCaseParams& p = c->p;
    cudaGetDevice(&c->device);
    c->Nx = p.Nx;
    c->Ny = p.Ny;
    // Rows start on 128-byte boundaries for every storage form.
    c->pitch = (p.Nx + 63) / 64 * 64;
    c->S = (long long)c->pitch * p.Ny;
    // GridClass::GridClass (src/Grid.cpp:1243-1260)
    const double rho0 = 1.0;
    c->cs = 1.0 / std::sqrt(3.0);
    c->tau = 1.0 / p.omega;
    c->nu = (c->tau - 0.5) * (c->cs * c->cs);
    c->Dx = p.height_p / (p.Ny - 1);
    c->Dt = (c->Dx * c->Dx) * c->nu / p.nu_p;
    c->Dm = (p.rho_p / rho0) * (c->Dx * c->Dx * c->Dx);
    c->Drho = (p.rho_p / rho0);
    const double sc = (c->Dx * c->Dt) * (c->Dx * c->Dt);
    c->Fx0 = (rho0 * c->Drho * p.gravityX + p.dpdx) * sc / c->Dm;
    c->Fy0 = (rho0 * c->Drho * p.gravityY + p.dpdy) * sc / c->Dm;
    c->site_force = p.has_womersley && (p.gravityX != 0.0 || p.gravityY != 0.0);
    c->u0x = p.ux0_p * c->Dt / c->Dx;
    c->u0y = p.uy0_p * c->Dt / c->Dx;
    c->init_mode = p.has_inlet_ramp ? 0 : (p.profile >= 0 ? 1 : 2);
    c->elem = p.precision == LIFE_PREC_F64 ? 8 : (p.precision == LIFE_PREC_F32 ? 4 : 2);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    // The side stream (outlet, boundary perimeter) has the highest priority:
    // its few blocks are then dispatched ahead of the interior launch's
    // queued blocks and run beside them instead of after them.
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_aux, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
    for (const char* var : {"LIFE_CASE_HOSTLOOP", "LIFE_FSI_HOSTLOOP"})
        if (const char* v = std::getenv(var))
            if (v[0] == '1') c->host_steps = true;
    if (e != cudaSuccess) {
        free_case(c);
        return cuda_fail(e, "cudaStreamCreate");
    }
    // Immersed bodies on the host (geometryReadIn + initialiseObjects).
    Grid0 g{p.Nx, p.Ny, c->Dx, c->Dt, c->Dm, p.gravityX, p.gravityY, p.ref_L, p.alpha, p.delta};
    c->g0 = g;
    std::string err;
    // Large marker sets test their pairs for overlap on the device;
    // LIFE_OVERLAP_SCAN=device / host forces one side for every set.
    int scan_min = kOverlapScanMin;
    OverlapScan scan = device_overlap_scan;
    if (const char* v = std::getenv("LIFE_OVERLAP_SCAN")) {
        if (std::strcmp(v, "device") == 0) scan_min = 0;
        else if (std::strcmp(v, "host") == 0) scan = nullptr;
    }
    int rc = build_objects(g, p, bodies, n_bodies, c->obj, &err, scan, scan_min);
    if (rc) {
        free_case(c);
        return set_error(rc, err);
    }
    // Inlet profile (src/Grid.cpp:954-996)
    std::vector<double> u_in((size_t)p.Ny * 2), rho_in(p.Ny, rho0);
    for (int j = 0; j < p.Ny; j++) {
        const double Dt = c->Dt, Dx = c->Dx;
        double ux = 0.0, uy = 0.0;
        if (p.profile < 0) {
            ux = p.uxInlet_p * Dt / Dx;
            uy = p.uyInlet_p * Dt / Dx;
        } else if (p.profile == LIFE_PROFILE_PARABOLIC) {
            const double R = p.height_p / 2.0, Y = j * Dx - R;
            ux = 1.5 * (p.uxInlet_p * Dt / Dx) * (1.0 - (Y / R) * (Y / R));
            uy = 1.5 * (p.uyInlet_p * Dt / Dx) * (1.0 - (Y / R) * (Y / R));
        } else if (p.profile == LIFE_PROFILE_SHEAR) {
            const double H = p.height_p, Y = j * Dx;
            ux = (p.uxInlet_p * Dt / Dx) * (Y / H);
            uy = (p.uyInlet_p * Dt / Dx) * (Y / H);
        } else if (p.profile == LIFE_PROFILE_BOUNDARY_LAYER) {
            const double H = p.height_p, Y = j * Dx;
            ux = ((1.5 * p.uxInlet_p * Dt / Dx) / (H * H)) * Y * (2.0 * H - Y);
            uy = ((1.5 * p.uyInlet_p * Dt / Dx) / (H * H)) * Y * (2.0 * H - Y);
        }
        u_in[j * 2] = ux;
        u_in[j * 2 + 1] = uy;
    }
    // Device buffers
    const size_t plane = (size_t)c->S;
    if ((rc = dev_alloc(c, &c->P[0], plane * 9 * c->elem)) || (rc = dev_alloc(c, &c->P[1], plane * 9 * c->elem)) ||
        (rc = dev_alloc_t(c, &c->d_u_in, (size_t)p.Ny * 2)) || (rc = dev_alloc_t(c, &c->d_rho_in, (size_t)p.Ny)) ||
        (rc = dev_alloc_t(c, &c->d_outlet_u, (size_t)3 * p.Ny * 2)) ||
        (rc = dev_alloc_t(c, &c->d_outlet_f[0], (size_t)p.Ny * 3)) ||
        (rc = dev_alloc_t(c, &c->d_outlet_f[1], (size_t)p.Ny * 3)) ||
        (rc = dev_alloc_t(c, &c->d_delU, (size_t)p.Ny * 2)) || (rc = dev_alloc_t(c, &c->d_red, 4)) ||
        (rc = dev_alloc_t(c, &c->d_corner_u[0], 8)) || (rc = dev_alloc_t(c, &c->d_corner_u[1], 8)) ||
        (rc = dev_alloc_t(c, &c->d_tile_ctr, 2)) ||
        (c->site_force && ((rc = dev_alloc_t(c, &c->d_rho_hist[0], plane)) ||
                           (rc = dev_alloc_t(c, &c->d_rho_hist[1], plane))))) {
        free_case(c);
        return rc;
    }
    cudaMemcpyAsync(c->d_u_in, u_in.data(), sizeof(double) * u_in.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_rho_in, rho_in.data(), sizeof(double) * rho_in.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(c->d_delU, 0, sizeof(double) * p.Ny * 2, c->stream);
    cudaMemsetAsync(c->d_tile_ctr, 0, sizeof(int) * 2, c->stream);
    if (c->obj.hasIBM) {
        if ((rc = upload_markers(c))) {
            free_case(c);
            return rc;
        }
        if (c->obj.hasFlex && (rc = setup_fem(c))) {
            free_case(c);
            return rc;
        }
    }
    c->t = 0;
    c->t_set = 0;
    if ((rc = ensure_steps(c, 0, 2))) {
        free_case(c);
        return rc;
    }
    LatDev L = lattice_view(c, 0);
    e = launch_init(c->P[0], c->P[1], L, 0, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        free_case(c);
        return cuda_fail(e, "init");
    }
    c->cur = 0;
    *out = c;
    return LIFE_OK;
}

extern "C" int life_case_destroy(LifeCase* c) {
    free_case(c);
    return LIFE_OK;
}

static int check_device_status(LifeCase* c) {
    if (c->p.precision != LIFE_PREC_F64 && tma_timeouts() > 0 && c->status_code == 0) {
        c->status_code = LIFE_ERR_TIMEOUT;
        c->status_t = c->t;
        c->status_msg = "a shared-memory tile copy of the step kernel did not complete";
        return LIFE_OK;
    }
    if (!c->d_status) return LIFE_OK;
    int h[4];
    CK(cudaMemcpyAsync(h, c->d_status, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (h[0] != 0 && c->status_code == 0) {
        c->status_code = h[0];
        c->status_t = h[1];
    }
    return LIFE_OK;
}

// Runs nsteps time steps on the case's stream. With `timing`, CUDA events are
// recorded around every interior-lattice launch and around the whole range,
// and the launches of the library's kernels are counted.
struct StepTiming {
    std::vector<cudaEvent_t> ev;   // 2 per step: before/after the interior kernel
    cudaEvent_t start = nullptr, stop = nullptr;
    int launches = 0;
};

// Runs shorter than this, before any step graph exists, launch their kernels
// directly: capturing and instantiating the two step graphs costs about as
// much host time as a few large steps, and the same kernels run either way.
constexpr int kDirectMaxSteps = 64;

static int run_steps(LifeCase* c, int nsteps, StepTiming* tm) {
    int rc;
    const bool direct = !c->host_steps && !tm && nsteps < kDirectMaxSteps && !case_graphs_ready(c);
    if (!c->host_steps && !direct) {
        // the case's captured step graphs; the same kernels in the same order
        if ((rc = case_graph_steps(c, nsteps, tm ? tm->start : nullptr, tm ? tm->stop : nullptr))) return rc;
        if (tm) tm->launches = case_kernels_per_step(c) * nsteps;
        if (c->obj.hasFlex) {
            if ((rc = check_device_status(c))) return rc;
            if (c->status_code) {
                c->status_msg = "Subiteration scheme hit 20 iterations...exiting";
                return set_error(c->status_code, c->status_msg);
            }
        }
        return LIFE_OK;
    }
    rc = ensure_steps(c, c->t, (nsteps < kStepChunk ? nsteps : kStepChunk) + 2);
    if (rc) return rc;
    const bool conv = c->p.wall_right == LIFE_CONVECTIVE;
    if (tm) cudaEventRecord(tm->start, c->stream);
    for (int k = 0; k < nsteps; k++) {
        if (k > 0 && k % kStepChunk == 0) {
            const int left = nsteps - k;
            if ((rc = ensure_steps(c, c->t, (left < kStepChunk ? left : kStepChunk) + 2))) return rc;
        }
        const int tt = c->t + 1;
        LatDev L = lattice_view(c, tt);
        const void* A = c->P[c->cur];
        void* B = c->P[c->cur ^ 1];
        cudaError_t e;
        if (conv) {
            e = launch_outlet(L, c->d_delU, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "outlet");
            if (tm) tm->launches++;
        }
        if (direct && case_fused_step(c)) {
            // the one-launch step kernel of the step graphs
            e = launch_step_lowp(A, B, L, tt, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "step");
        } else {
            // The boundary-condition perimeter runs on a side stream,
            // overlapped with the interior kernel: both read only A and write
            // disjoint sites of B. The main stream waits for it before
            // anything reads B.
            cudaEventRecord(c->ev_fork, c->stream);
            cudaStreamWaitEvent(c->side, c->ev_fork, 0);
            e = launch_perimeter(A, B, L, tt, c->side);
            if (e != cudaSuccess) return cuda_fail(e, "perimeter step");
            cudaEventRecord(c->ev_join, c->side);
            if (tm) cudaEventRecord(tm->ev[2 * k], c->stream);
            e = L.prec == LIFE_PREC_F64 ? launch_interior_f64((const double*)A, (double*)B, L, tt, c->stream)
                                        : launch_interior_lowp(A, B, L, tt, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "interior step");
            if (tm) cudaEventRecord(tm->ev[2 * k + 1], c->stream);
            cudaStreamWaitEvent(c->stream, c->ev_join, 0);
            if (tm) tm->launches += 2;
        }
        if (c->obj.hasIBM) {
            int before = c->ibm_launches;
            if ((rc = ibm_step(c, tt, A, B))) return rc;
            if (tm) tm->launches += c->ibm_launches - before;
        }
        if (c->rec.every > 0) {
            e = launch_record(c, tt, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "observables recorder");
            if (tm) tm->launches++;
        }
        c->cur ^= 1;
        c->t = tt;
    }
    if (tm) cudaEventRecord(tm->stop, c->stream);
    if (c->obj.hasFlex) {
        if ((rc = check_device_status(c))) return rc;
        if (c->status_code) {
            c->status_msg = "Subiteration scheme hit 20 iterations...exiting";
            return set_error(c->status_code, c->status_msg);
        }
    }
    return LIFE_OK;
}

extern "C" int life_case_step(LifeCase* c, int32_t nsteps) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    if (nsteps < 0) return set_error(LIFE_ERR_INVALID, "negative step count");
    if (nsteps == 0) return LIFE_OK;
    if (c->status_code) return set_error(c->status_code, c->status_msg);
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c->device) cudaSetDevice(c->device);
    int rc = run_steps(c, nsteps, nullptr);
    if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return rc;
}

extern "C" int life_case_bench_steps(LifeCase* c, int32_t nsteps, double* total_ms, double* interior_ms,
                                     int32_t* launches) {
    if (!c || nsteps <= 0) return set_error(LIFE_ERR_INVALID, "bad arguments");
    if (c->status_code) return set_error(c->status_code, c->status_msg);
    StepTiming tm;
    tm.ev.resize(2 * (size_t)nsteps);
    for (auto& e : tm.ev) CK(cudaEventCreate(&e));
    CK(cudaEventCreate(&tm.start));
    CK(cudaEventCreate(&tm.stop));
    CK(cudaStreamSynchronize(c->stream));
    int rc = run_steps(c, nsteps, &tm);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    double tot = 0.0, inner = 0.0;
    if (rc == LIFE_OK && e == cudaSuccess) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, tm.start, tm.stop);
        tot = ms;
        if (c->host_steps) {
            for (int k = 0; k < nsteps; k++) {
                cudaEventElapsedTime(&ms, tm.ev[2 * k], tm.ev[2 * k + 1]);
                inner += ms;
            }
        } else {
            // inside a graph the interior launch is timed alone afterwards
            rc = case_interior_ms(c, 10, &ms);
            inner = (double)ms * nsteps;
        }
    }
    for (auto& ev : tm.ev) cudaEventDestroy(ev);
    cudaEventDestroy(tm.start);
    cudaEventDestroy(tm.stop);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "bench_steps");
    if (total_ms) *total_ms = tot;
    if (interior_ms) *interior_ms = inner / nsteps;
    if (launches) *launches = tm.launches;
    return LIFE_OK;
}

extern "C" int life_case_sync(LifeCase* c) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    CK(cudaStreamSynchronize(c->stream));
    if (int rc = check_device_status(c)) return rc;
    if (c->status_code) return set_error(c->status_code, c->status_msg);
    return LIFE_OK;
}

extern "C" int life_case_info(const LifeCase* c, LifeCaseInfo* info) {
    if (!c || !info) return set_error(LIFE_ERR_INVALID, "NULL argument");
    std::memset(info, 0, sizeof *info);
    info->Nx = c->Nx;
    info->Ny = c->Ny;
    info->n_bodies = (int)c->obj.b.size();
    info->n_markers = (int)c->obj.m.size();
    info->n_flex = c->obj.nFlex;
    info->sim_dofs = c->obj.simDOFs;
    info->precision = c->p.precision;
    info->t = c->t;
    info->Dx = c->Dx;
    info->Dt = c->Dt;
    info->Dm = c->Dm;
    info->Drho = c->Drho;
    info->tau = c->tau;
    info->nu = c->nu;
    info->c_s = c->cs;
    info->device_bytes = c->dev_bytes;
    return LIFE_OK;
}

extern "C" int life_case_status(LifeCase* c, LifeStatus* st) {
    if (!c || !st) return set_error(LIFE_ERR_INVALID, "NULL argument");
    if (int rc = check_device_status(c)) return rc;
    std::memset(st, 0, sizeof *st);
    st->code = c->status_code;
    st->t = c->status_t;
    if (c->d_fsi) {
        FsiScalars h{};
        CK(cudaMemcpyAsync(&h, c->d_fsi, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        st->last_subits = h.subIt;
        st->last_subres = h.subRes;
        st->relax = h.relax;
        st->last_nr_its = h.lastNR;
    }
    return LIFE_OK;
}

extern "C" int life_case_get_fields(LifeCase* c, double* rho, double* u, double* f, double* force_ibm) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const size_t n = (size_t)c->Nx * c->Ny;
    if (c->t == c->t_set && c->host_state) {
        if (rho) std::memcpy(rho, c->h_rho.data(), n * sizeof(double));
        if (u) std::memcpy(u, c->h_u.data(), n * 2 * sizeof(double));
        if (f) std::memcpy(f, c->h_f.data(), n * 9 * sizeof(double));
        if (force_ibm) std::memcpy(force_ibm, c->h_fibm.data(), n * 2 * sizeof(double));
        return LIFE_OK;
    }
    // staging buffers on the device: from the memory pool, ordered on the
    // case's stream (kernel, copies and release all run there), else cudaMalloc
    double *d_rho = nullptr, *d_u = nullptr, *d_f = nullptr, *d_fi = nullptr;
    int dev = 0;
    cudaGetDevice(&dev);
    DevicePool* P = device_pool(dev);
    const bool pooled = P && P->pooled;
    auto get = [&](double** p, size_t count) {
        return pooled ? cudaMallocAsync((void**)p, count * sizeof(double), c->stream)
                      : cudaMalloc((void**)p, count * sizeof(double));
    };
    auto cleanup = [&]() {
        for (double* p : {d_rho, d_u, d_f, d_fi})
            if (p) {
                if (pooled) cudaFreeAsync(p, c->stream);
                else cudaFree(p);
            }
    };
    if ((rho && get(&d_rho, n) != cudaSuccess) || (u && get(&d_u, n * 2) != cudaSuccess) ||
        (f && get(&d_f, n * 9) != cudaSuccess) || (force_ibm && get(&d_fi, n * 2) != cudaSuccess)) {
        cleanup();
        cudaStreamSynchronize(c->stream);
        cudaGetLastError();
        return set_error(LIFE_ERR_NOMEM, "no device memory for the field export");
    }
    LatDev L = lattice_view(c, c->t);
    const bool initial = (c->t == c->t_set);
    // Large lattices export into page-locked host buffers in column chunks,
    // each a contiguous range of the reference layout, so the copy of chunk k
    // (on the side stream) runs beside the export kernel of chunk k+1 (on the
    // case's stream). Copies to pageable memory block the host and would
    // serialise the chunks, so those take one copy per field.
    bool locked = true;
    for (const double* h : {(const double*)rho, (const double*)u, (const double*)f, (const double*)force_ibm}) {
        if (!h) continue;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, h) != cudaSuccess || a.type != cudaMemoryTypeHost) locked = false;
    }
    cudaGetLastError();
    const int chunks = (!initial && locked && n >= (1u << 20)) ? 8 : 1;
    cudaEvent_t ev = nullptr;
    cudaError_t e = chunks > 1 ? cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) : cudaSuccess;
    for (int k = 0; k < chunks && e == cudaSuccess; k++) {
        const int i0 = (int)((long long)c->Nx * k / chunks), i1 = (int)((long long)c->Nx * (k + 1) / chunks);
        const size_t o = (size_t)i0 * c->Ny, m = (size_t)(i1 - i0) * c->Ny;
        e = launch_export(c->P[c->cur ^ 1], L, c->t, initial, d_rho, d_u, d_f, d_fi, c->stream, i0,
                          chunks > 1 ? i1 : -1);
        cudaStream_t cs = c->stream;
        if (chunks > 1) {
            if (e == cudaSuccess) e = cudaEventRecord(ev, c->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, ev, 0);
            cs = c->side;
        }
        const size_t oo = chunks > 1 ? o : 0, mm = chunks > 1 ? m : n;
        if (e == cudaSuccess && rho)
            e = cudaMemcpyAsync(rho + oo, d_rho + oo, mm * sizeof(double), cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && u)
            e = cudaMemcpyAsync(u + 2 * oo, d_u + 2 * oo, mm * 2 * sizeof(double), cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && f)
            e = cudaMemcpyAsync(f + 9 * oo, d_f + 9 * oo, mm * 9 * sizeof(double), cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && force_ibm)
            e = cudaMemcpyAsync(force_ibm + 2 * oo, d_fi + 2 * oo, mm * 2 * sizeof(double), cudaMemcpyDeviceToHost, cs);
    }
    if (chunks > 1) {
        // the staging buffers are released on the case's stream after the copies
        const cudaError_t ew = ev ? cudaEventRecord(ev, c->side) : cudaSuccess;
        if (ew == cudaSuccess) {
            cudaStreamWaitEvent(c->stream, ev, 0);
        } else {
            cudaStreamSynchronize(c->side);
            if (e == cudaSuccess) e = ew;
        }
    }
    cleanup();
    const cudaError_t es = cudaStreamSynchronize(c->stream);
    if (chunks > 1) cudaStreamSynchronize(c->side);
    if (ev) cudaEventDestroy(ev);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) return cuda_fail(e, "get_fields");
    return LIFE_OK;
}

extern "C" int life_case_get_vtk_fields(LifeCase* c, double* density, double* pressure, double* velocity) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const size_t n = (size_t)c->Nx * c->Ny;
    VtiScale V{c->Drho, c->p.ref_P, c->p.rho_p, c->cs, c->Dm, c->Dx, c->Dt};
    if (c->t == c->t_set && c->host_state) {
        // a loaded restart state, before any step: the same conversions on
        // the host arrays (reference layout id = i*Ny + j)
        for (int j = 0; j < c->Ny; j++)
            for (int i = 0; i < c->Nx; i++) {
                const size_t id = (size_t)i * c->Ny + j, o = (size_t)j * c->Nx + i;
                const double rho = c->h_rho[id];
                if (density) density[o] = rho * V.Drho;
                if (pressure)
                    pressure[o] = V.ref_P + (rho - V.rho_p / V.Drho) * (V.cs * V.cs) * V.Dm / (V.Dx * (V.Dt * V.Dt));
                if (velocity) {
                    velocity[o * 3] = c->h_u[id * 2] * (V.Dx / V.Dt);
                    velocity[o * 3 + 1] = c->h_u[id * 2 + 1] * (V.Dx / V.Dt);
                    velocity[o * 3 + 2] = 0.0;
                }
            }
        return LIFE_OK;
    }
    double *d_dens = nullptr, *d_pres = nullptr, *d_vel = nullptr;
    cudaError_t e = cudaSuccess;
    if (density) e = cudaMallocAsync((void**)&d_dens, n * sizeof(double), c->stream);
    if (e == cudaSuccess && pressure) e = cudaMallocAsync((void**)&d_pres, n * sizeof(double), c->stream);
    if (e == cudaSuccess && velocity) e = cudaMallocAsync((void**)&d_vel, 3 * n * sizeof(double), c->stream);
    if (e == cudaSuccess) {
        const LatDev L = lattice_view(c, c->t);
        e = launch_export_vti(c->P[c->cur ^ 1], L, c->t, c->t == c->t_set, V, d_dens, d_pres, d_vel, c->stream);
    }
    if (e == cudaSuccess && density)
        e = cudaMemcpyAsync(density, d_dens, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && pressure)
        e = cudaMemcpyAsync(pressure, d_pres, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && velocity)
        e = cudaMemcpyAsync(velocity, d_vel, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    for (double* p : {d_dens, d_pres, d_vel})
        if (p) cudaFreeAsync(p, c->stream);
    const cudaError_t es = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) return cuda_fail(e, "life_case_get_vtk_fields");
    return LIFE_OK;
}

extern "C" int life_case_set_fields(LifeCase* c, int32_t t, const double* rho, const double* u, const double* f,
                                    const double* force_ibm) {
    if (!c || !rho || !u || !f) return set_error(LIFE_ERR_INVALID, "NULL argument");
    const size_t n = (size_t)c->Nx * c->Ny;
    c->h_rho.assign(rho, rho + n);
    c->h_u.assign(u, u + 2 * n);
    c->h_f.assign(f, f + 9 * n);
    if (force_ibm) c->h_fibm.assign(force_ibm, force_ibm + 2 * n);
    else c->h_fibm.assign(2 * n, 0.0);
    c->host_state = true;
    double *d_rho = nullptr, *d_u = nullptr, *d_f = nullptr, *d_fi = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_rho);
        cudaFree(d_u);
        cudaFree(d_f);
        cudaFree(d_fi);
    };
    if (cudaMalloc(&d_rho, n * 8) != cudaSuccess || cudaMalloc(&d_u, n * 16) != cudaSuccess ||
        cudaMalloc(&d_f, n * 72) != cudaSuccess || cudaMalloc(&d_fi, n * 16) != cudaSuccess) {
        cleanup();
        return set_error(LIFE_ERR_NOMEM, "no device memory for the field import");
    }
    cudaMemcpyAsync(d_rho, c->h_rho.data(), n * 8, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_u, c->h_u.data(), n * 16, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_f, c->h_f.data(), n * 72, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_fi, c->h_fibm.data(), n * 16, cudaMemcpyHostToDevice, c->stream);
    c->t = t;
    c->t_set = t;
    int rc = ensure_steps(c, t, 2);
    if (rc) {
        cleanup();
        return rc;
    }
    LatDev L = lattice_view(c, t);
    cudaError_t e = launch_state(c->P[0], L, t, d_rho, d_u, d_f, d_fi, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "set_fields");
    c->cur = 0;
    return LIFE_OK;
}

extern "C" int life_case_max_velocity(LifeCase* c, double* max_vel, int32_t* has_nan) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    unsigned long long h[2] = {0, 0};
    CK(cudaMemsetAsync(c->d_red, 0, 2 * sizeof(unsigned long long), c->stream));
    LatDev L = lattice_view(c, c->t);
    if (c->t == c->t_set) {
        // Before the first step the state is the initial (or restart) one:
        // export it and reduce on the host side of this call.
        std::vector<double> u((size_t)c->Nx * c->Ny * 2);
        if (int rc = life_case_get_fields(c, nullptr, u.data(), nullptr, nullptr)) return rc;
        double m = 0.0;
        int nan = 0;
        for (size_t k = 0; k < u.size() / 2; k++) {
            double v = std::sqrt(u[2 * k] * u[2 * k] + u[2 * k + 1] * u[2 * k + 1]);
            if (v != v) nan = 1;
            else if (v > m) m = v;
        }
        if (max_vel) *max_vel = m;
        if (has_nan) *has_nan = nan;
        return LIFE_OK;
    }
    CK(launch_maxvel(c->P[c->cur ^ 1], L, c->t, c->d_red, c->stream));
    CK(cudaMemcpyAsync(h, c->d_red, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double m;
    std::memcpy(&m, &h[0], sizeof m);
    if (max_vel) *max_vel = m;
    if (has_nan) *has_nan = h[1] ? 1 : 0;
    return LIFE_OK;
}
