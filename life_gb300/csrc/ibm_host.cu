// Host side of the immersed bodies: device upload of the markers, the
// per-step IBM sequence (ObjectsClass::objectKernel, reference
// src/Objects.cpp:26-60) and the marker/body accessors of the C-ABI.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "fem_kernels.h"
#include "ibm_kernels.h"
#include "life_internal.h"

using namespace life;

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

static int alloc_track(LifeCase* c, void** p, size_t bytes) { return case_dev_alloc(c, p, bytes); }
template <class T>
static int alloc_t(LifeCase* c, T** p, size_t n) {
    return alloc_track(c, (void**)p, sizeof(T) * n);
}

// removeOverlapMarkers' pair test on the device (objects.h OverlapScan): the
// close pairs, sorted into the reference's (n1, n2) loop order.
int life::device_overlap_scan(const double* pos, int nm, double Dx, std::vector<std::pair<int, int>>* pairs,
                              std::string* err) {
    (void)err;
    pairs->clear();
    if (nm < 2) return LIFE_OK;
    double* d_pos = nullptr;
    int* d_count = nullptr;
    int2* d_out = nullptr;
    int cap = 1 << 16, count = 0;
    cudaError_t e = cudaMalloc(&d_pos, sizeof(double) * 2 * (size_t)nm);
    if (e == cudaSuccess) e = cudaMalloc(&d_count, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(d_pos, pos, sizeof(double) * 2 * (size_t)nm, cudaMemcpyHostToDevice);
    for (int pass = 0; e == cudaSuccess && pass < 2; pass++) {
        if (d_out) cudaFree(d_out);
        d_out = nullptr;
        e = cudaMalloc(&d_out, sizeof(int2) * (size_t)cap);
        if (e == cudaSuccess) e = cudaMemset(d_count, 0, sizeof(int));
        if (e == cudaSuccess) e = launch_overlap_pairs(d_pos, nm, Dx, d_count, d_out, cap, 0);
        if (e == cudaSuccess) e = cudaMemcpy(&count, d_count, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess || count <= cap) break;
        cap = count;  // the first list was too short: run again with room for all
    }
    std::vector<int2> h;
    if (e == cudaSuccess && count > cap) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
        h.resize(count);
        if (count) e = cudaMemcpy(h.data(), d_out, sizeof(int2) * (size_t)count, cudaMemcpyDeviceToHost);
    }
    cudaFree(d_out);
    cudaFree(d_count);
    cudaFree(d_pos);
    if (e != cudaSuccess) return cuda_fail(e, "marker overlap scan");
    pairs->reserve(count);
    for (const int2& q : h) pairs->emplace_back(q.x, q.y);
    std::sort(pairs->begin(), pairs->end());
    return LIFE_OK;
}

// Copies the host marker table to the device arrays.
int push_markers(LifeCase* c) {
    const auto& m = c->obj.m;
    const int n = (int)m.size();
    std::vector<double> pos(2 * n), vel(2 * n), force(2 * n), eps(n), ds(n), sd(9 * n);
    std::vector<int> ns(n), si(9 * n), sj(9 * n), body(n);
    for (int k = 0; k < n; k++) {
        for (int d = 0; d < 2; d++) {
            pos[2 * k + d] = m[k].pos[d];
            vel[2 * k + d] = m[k].vel[d];
            force[2 * k + d] = m[k].force[d];
        }
        eps[k] = m[k].eps;
        ds[k] = m[k].ds;
        ns[k] = m[k].nsupp;
        body[k] = m[k].body;
        for (int s = 0; s < 9; s++) {
            si[9 * k + s] = m[k].si[s];
            sj[9 * k + s] = m[k].sj[s];
            sd[9 * k + s] = m[k].sd[s];
        }
    }
    MarkerDev& M = c->M;
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(M.pos, pos.data(), 16 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.vel, vel.data(), 16 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.force, force.data(), 16 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.eps, eps.data(), 8 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.ds, ds.data(), 8 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.nsupp, ns.data(), 4 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.si, si.data(), 36 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.sj, sj.data(), 36 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.sd, sd.data(), 72 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(M.body, body.data(), 4 * n, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    return LIFE_OK;
}

int upload_markers(LifeCase* c) {
    const int n = (int)c->obj.m.size();
    MarkerDev& M = c->M;
    M.n = n;
    int rc;
    if ((rc = alloc_t(c, &M.pos, 2 * n)) || (rc = alloc_t(c, &M.vel, 2 * n)) || (rc = alloc_t(c, &M.force, 2 * n)) ||
        (rc = alloc_t(c, &M.eps, n)) || (rc = alloc_t(c, &M.ds, n)) || (rc = alloc_t(c, &M.nsupp, n)) ||
        (rc = alloc_t(c, &M.si, 9 * n)) || (rc = alloc_t(c, &M.sj, 9 * n)) || (rc = alloc_t(c, &M.sd, 9 * n)) ||
        (rc = alloc_t(c, &M.bbox, n)) || (rc = alloc_t(c, &M.body, n)))
        return rc;
    if ((rc = push_markers(c))) return rc;
    IbmScratch& W = c->W;
    W.ntx = (c->Nx + 15) / 16;
    W.nty = (c->Ny + 15) / 16;
    W.max_tiles = W.ntx * W.nty;
    if ((rc = alloc_t(c, &W.force_ibm, (size_t)2 * c->S)) || (rc = alloc_t(c, &W.sites, (size_t)9 * n + 1)) ||
        (rc = alloc_t(c, &W.sites_prev, (size_t)9 * n + 1)) || (rc = alloc_t(c, &W.nsites, 1)) ||
        (rc = alloc_t(c, &W.nsites_prev, 1)) || (rc = alloc_t(c, &W.tile_flag, (size_t)W.max_tiles)) ||
        (rc = alloc_t(c, &W.tiles, (size_t)W.max_tiles)) || (rc = alloc_t(c, &W.ntiles, 1)))
        return rc;
    CK(cudaMemsetAsync(W.force_ibm, 0, sizeof(double) * 2 * c->S, c->stream));
    CK(cudaMemsetAsync(W.nsites, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(W.nsites_prev, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(W.tile_flag, 0, sizeof(unsigned) * W.max_tiles, c->stream));
    CK(cudaMemsetAsync(W.ntiles, 0, sizeof(int), c->stream));
    // bodies as contiguous marker ranges (markers are stored body by body);
    // one range over all markers if that ever does not hold
    std::vector<int> start(1, 0);
    bool contiguous = true;
    for (int k = 1; k < n; k++) {
        const int b0 = c->obj.m[k - 1].body, b1 = c->obj.m[k].body;
        if (b1 != b0) {
            if (b1 < b0) contiguous = false;
            start.push_back(k);
        }
    }
    start.push_back(n);
    if (!contiguous || n == 0) start = {0, n};
    W.nbodies = (int)start.size() - 1;
    std::vector<int> box_of((size_t)std::max(n, 1), 0);
    for (int r = 0; r < W.nbodies; r++)
        for (int k = start[r]; k < start[r + 1]; k++) box_of[k] = r;
    int *d_start = nullptr, *d_box_of = nullptr;
    if ((rc = alloc_t(c, &d_start, start.size())) || (rc = alloc_t(c, &d_box_of, box_of.size())) ||
        (rc = alloc_t(c, &W.body_box, (size_t)W.nbodies)))
        return rc;
    W.body_start = d_start;
    W.box_of = d_box_of;
    CK(cudaMemcpyAsync(d_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_box_of, box_of.data(), sizeof(int) * box_of.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if ((rc = alloc_t(c, &c->d_fsi, 1)) || (rc = alloc_t(c, &c->d_status, 4))) return rc;
    FsiScalars f{};
    f.relax = c->p.relaxMax;
    CK(cudaMemcpyAsync(c->d_fsi, &f, sizeof f, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_status, 0, 4 * sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LIFE_OK;
}

// One step of ObjectsClass::objectKernel on the device, in two parts. The
// forces (interpolation and forceCalc, or the whole FSI subiteration loop)
// read only the step's input populations A, so they can run beside the
// lattice step; the spread writes the support sites of B and follows both.
int ibm_forces(LifeCase* c, int t, const void* A, cudaStream_t s) {
    LatDev L = lattice_view(c, t);
    if (c->obj.hasFlex) return fem_fsi_loop(c, t, A, L, s);
    cudaError_t e = launch_ibm_interp(A, L, t, c->M, c->Dt / c->Dx, s);
    if (e != cudaSuccess) return cuda_fail(e, "ibm_interp");
    c->ibm_launches += 1;
    return LIFE_OK;
}

int ibm_apply(LifeCase* c, int t, const void* A, void* B, cudaStream_t s) {
    LatDev L = lattice_view(c, t);
    cudaError_t e = launch_ibm_spread(A, B, L, t, c->M, c->W, s);
    if (e != cudaSuccess) return cuda_fail(e, "ibm_spread");
    c->ibm_launches += 3;
    std::swap(c->W.sites, c->W.sites_prev);
    std::swap(c->W.nsites, c->W.nsites_prev);
    return LIFE_OK;
}

int ibm_step(LifeCase* c, int t, const void* A, void* B) {
    if (int rc = ibm_forces(c, t, A, c->stream)) return rc;
    return ibm_apply(c, t, A, B, c->stream);
}

extern "C" int life_case_get_markers(LifeCase* c, double* pos, double* vel, double* force, double* epsilon,
                                     double* ds, int32_t* body_index) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const int n = c->M.n;
    if (n == 0) return LIFE_OK;
    cudaStream_t s = c->stream;
    if (pos) CK(cudaMemcpyAsync(pos, c->M.pos, 16 * n, cudaMemcpyDeviceToHost, s));
    if (vel) CK(cudaMemcpyAsync(vel, c->M.vel, 16 * n, cudaMemcpyDeviceToHost, s));
    if (force) CK(cudaMemcpyAsync(force, c->M.force, 16 * n, cudaMemcpyDeviceToHost, s));
    if (epsilon) CK(cudaMemcpyAsync(epsilon, c->M.eps, 8 * n, cudaMemcpyDeviceToHost, s));
    if (ds) CK(cudaMemcpyAsync(ds, c->M.ds, 8 * n, cudaMemcpyDeviceToHost, s));
    if (body_index) CK(cudaMemcpyAsync(body_index, c->M.body, 4 * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return LIFE_OK;
}

// The IBM half of ObjectsClass::readRestart (src/Objects.cpp:981-1053):
// marker positions, velocities and forces in global marker order (NULL
// skips a field), then findSupport + computeDs of every marker and
// computeEpsilon (src/Objects.cpp:1181-1192), on the host as at start-up.
// Rigid bodies keep their construction epsilon in the reference (it skips
// them after step 0); recomputing it from the same positions gives the same
// values.
extern "C" int life_case_set_markers(LifeCase* c, const double* pos, const double* vel, const double* force) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const int n = (int)c->obj.m.size();
    if (n == 0) return LIFE_OK;
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < n; k++) {
        HMarker& m = c->obj.m[k];
        for (int d = 0; d < 2; d++) {
            if (pos) m.pos[d] = pos[2 * k + d];
            if (vel) m.vel[d] = vel[2 * k + d];
            if (force) m.force[d] = force[2 * k + d];
        }
    }
    std::string err;
    for (int k = 0; k < n; k++)
        if (int rc = host_find_support(c->g0, c->obj.m[k], &err)) return set_error(rc, err);
    for (int k = 0; k < n; k++) host_compute_ds(c->g0, c->obj, k);
    if (int rc = host_compute_epsilon(c->g0, c->obj, c->p.uni_epsilon != 0, true, &err)) return set_error(rc, err);
    if (int rc = push_markers(c)) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return LIFE_OK;
}

extern "C" int life_case_get_bodies(LifeCase* c, int32_t* ids, int32_t* flexible, int32_t* n_markers,
                                    int32_t* n_fem_nodes) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    for (size_t k = 0; k < c->obj.b.size(); k++) {
        const HBody& b = c->obj.b[k];
        if (ids) ids[k] = b.ID;
        if (flexible) flexible[k] = b.flex;
        if (n_markers) n_markers[k] = (int)b.nodes.size();
        if (n_fem_nodes) n_fem_nodes[k] = b.fem ? b.fem->nNodes : 0;
    }
    return LIFE_OK;
}

extern "C" int life_case_get_body_nodes(LifeCase* c, int32_t* kind, int32_t* marker_index) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    size_t q = 0;
    for (size_t k = 0; k < c->obj.b.size(); k++) {
        const HBody& b = c->obj.b[k];
        if (kind) kind[k] = b.kind;
        for (int m : b.nodes) {
            if (marker_index) marker_index[q] = m;
            q++;
        }
    }
    return LIFE_OK;
}

// ObjectsClass::writeTotalForces (src/Objects.cpp:517-528): sequential sum
// over markers, in lattice units scaled to newtons.
extern "C" int life_case_total_force(LifeCase* c, double* fx, double* fy) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const int n = c->M.n;
    std::vector<double> force(2 * n), eps(n), ds(n);
    if (n) {
        int rc = life_case_get_markers(c, nullptr, nullptr, force.data(), eps.data(), ds.data(), nullptr);
        if (rc) return rc;
    }
    const double forceScale = c->Dm * c->Dx / (c->Dt * c->Dt) * 1.0 / c->Dx;
    double F[2] = {0.0, 0.0};
    for (int k = 0; k < n; k++)
        for (int d = 0; d < 2; d++) F[d] -= force[2 * k + d] * 1.0 * eps[k] * ds[k] * forceScale;
    if (fx) *fx = F[0];
    if (fy) *fy = F[1];
    return LIFE_OK;
}

// SplitMix64 (Steele, Lea and Flood 2014), mapped to [0, 1) with 53 bits:
// the draws of the CANOPY keyword.
static double canopy_draw(uint64_t& state) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1p-53;
}

extern "C" int life_parse_geometry(const char* text, LifeBodyDesc* out, int32_t cap, int32_t* n) {
    if (!text || !n) return set_error(LIFE_ERR_INVALID, "NULL argument");
    // Skip the leading comment lines (src/Objects.cpp:338-353).
    const char* p = text;
    while (*p == '#') {
        while (*p && *p != '\n') p++;
        if (*p == '\n') p++;
    }
    std::vector<std::string> tok;
    std::string cur;
    for (; *p; p++) {
        if (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') {
            if (!cur.empty()) tok.push_back(cur);
            cur.clear();
        } else {
            cur += *p;
        }
    }
    if (!cur.empty()) tok.push_back(cur);
    int count = 0;
    size_t q = 0;
    try {
        while (q < tok.size()) {
            LifeBodyDesc d{};
            if (tok[q] == "CIRCLE") {
                if (q + 8 > tok.size()) return set_error(LIFE_ERR_GEOMETRY, "truncated CIRCLE line");
                d.kind = LIFE_BODY_CIRCLE;
                d.number = std::stoi(tok[q + 1]);
                d.id = std::stoi(tok[q + 2]);
                d.x = std::stod(tok[q + 3]);
                d.y = std::stod(tok[q + 4]);
                d.dx = std::stod(tok[q + 5]);
                d.dy = std::stod(tok[q + 6]);
                d.radius = std::stod(tok[q + 7]);
                q += 8;
            } else if (tok[q] == "FILAMENT") {
                if (q + 15 > tok.size()) return set_error(LIFE_ERR_GEOMETRY, "truncated FILAMENT line");
                d.kind = LIFE_BODY_FILAMENT;
                d.number = std::stoi(tok[q + 1]);
                d.id = std::stoi(tok[q + 2]);
                d.x = std::stod(tok[q + 3]);
                d.y = std::stod(tok[q + 4]);
                d.dx = std::stod(tok[q + 5]);
                d.dy = std::stod(tok[q + 6]);
                d.length = std::stod(tok[q + 7]);
                d.height = std::stod(tok[q + 8]);
                d.angle_deg = std::stod(tok[q + 9]);
                if (tok[q + 10] == "FLEXIBLE") d.flexible = 1;
                else if (tok[q + 10] == "RIGID") d.flexible = 0;
                else return set_error(LIFE_ERR_GEOMETRY, "Not a proper flexible type set...exiting");
                d.n_elements = tok[q + 11] == "CONFORMING" ? 0 : (int)std::stod(tok[q + 11]);
                d.clamped = tok[q + 12] == "CLAMPED" ? 1 : 0;
                d.rho = std::stod(tok[q + 13]);
                d.E = std::stod(tok[q + 14]);
                q += 15;
            } else if (tok[q] == "CANOPY") {
                // CANOPY NUMBER STARTID STARTX STARTY SPACING_X SPACING_Y
                //        LENGTH_MIN LENGTH_MAX HEIGHT ANGLE N_ELEMENTS|CONFORMING
                //        CLAMPED|SUPPORTED DENSITY_PER_LENGTH YOUNG_MIN YOUNG_MAX SEED
                // NUMBER flexible stalks, stalk k at START + k SPACING with
                // length L_k = LMIN + (LMAX - LMIN) r, density DPL L_k and
                // Young's modulus Y_k L_k^3, Y_k = YMIN (YMAX / YMIN)^r'
                // (log-uniform), r and r' the next two draws of SplitMix64
                // seeded with SEED; each stalk becomes one FILAMENT body.
                if (q + 17 > tok.size()) return set_error(LIFE_ERR_GEOMETRY, "truncated CANOPY line");
                const int number = std::stoi(tok[q + 1]), id0 = std::stoi(tok[q + 2]);
                const double sx = std::stod(tok[q + 3]), sy = std::stod(tok[q + 4]);
                const double dx = std::stod(tok[q + 5]), dy = std::stod(tok[q + 6]);
                const double lmin = std::stod(tok[q + 7]), lmax = std::stod(tok[q + 8]);
                const double height = std::stod(tok[q + 9]), angle = std::stod(tok[q + 10]);
                const int nel = tok[q + 11] == "CONFORMING" ? 0 : (int)std::stod(tok[q + 11]);
                const int clamped = tok[q + 12] == "CLAMPED" ? 1 : 0;
                const double dpl = std::stod(tok[q + 13]);
                const double ymin = std::stod(tok[q + 14]), ymax = std::stod(tok[q + 15]);
                uint64_t state = std::stoull(tok[q + 16]);
                if (number < 0 || !(lmin > 0.0) || lmax < lmin || !(ymin > 0.0) || ymax < ymin)
                    return set_error(LIFE_ERR_GEOMETRY, "bad CANOPY parameters");
                q += 17;
                for (int k = 0; k < number; k++) {
                    LifeBodyDesc s{};
                    s.kind = LIFE_BODY_FILAMENT;
                    s.number = 1;
                    s.id = id0 + k;
                    s.x = sx + k * dx;
                    s.y = sy + k * dy;
                    const double rl = canopy_draw(state), ry = canopy_draw(state);
                    s.length = lmin + (lmax - lmin) * rl;
                    s.height = height;
                    s.angle_deg = angle;
                    s.flexible = 1;
                    s.n_elements = nel;
                    s.clamped = clamped;
                    s.rho = dpl * s.length;
                    s.E = (ymin * std::pow(ymax / ymin, ry)) * (s.length * s.length * s.length);
                    if (out && count < cap) out[count] = s;
                    count++;
                }
                continue;
            } else {
                return set_error(LIFE_ERR_GEOMETRY, "unknown geometry keyword '" + tok[q] + "'");
            }
            if (out && count < cap) out[count] = d;
            count++;
        }
    } catch (...) {
        return set_error(LIFE_ERR_GEOMETRY, "malformed number in geometry.config");
    }
    *n = count;
    return LIFE_OK;
}

extern "C" int life_case_get_support(LifeCase* c, int32_t* nsupp, int32_t* si, int32_t* sj, double* sd) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    const int n = c->M.n;
    if (n == 0) return LIFE_OK;
    cudaStream_t s = c->stream;
    if (nsupp) CK(cudaMemcpyAsync(nsupp, c->M.nsupp, 4 * n, cudaMemcpyDeviceToHost, s));
    if (si) CK(cudaMemcpyAsync(si, c->M.si, 36 * n, cudaMemcpyDeviceToHost, s));
    if (sj) CK(cudaMemcpyAsync(sj, c->M.sj, 36 * n, cudaMemcpyDeviceToHost, s));
    if (sd) CK(cudaMemcpyAsync(sd, c->M.sd, 72 * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return LIFE_OK;
}

// ObjectsClass::computeEpsilon for one marker set on caller-provided device
// buffers; the n x n system and pivots live in memory allocated per call.
extern "C" int life_ibm_epsilon(const double* pos, const int32_t* nsupp, const int32_t* si, const int32_t* sj,
                                const double* sd, const double* ds, int32_t n, double Dx, double* eps,
                                void* stream) {
    if (n < 0 || (n > 0 && (!pos || !nsupp || !si || !sj || !sd || !ds || !eps)))
        return set_error(LIFE_ERR_INVALID, "bad arguments");
    if (n == 0) return LIFE_OK;
    if (!(Dx > 0.0)) return set_error(LIFE_ERR_INVALID, "Dx must be positive");
    cudaStream_t s = (cudaStream_t)stream;
    double *A = nullptr, *b = nullptr;
    int *piv = nullptr, *lmax = nullptr;
    cudaError_t e = cudaMalloc(&A, sizeof(double) * (size_t)n * n);
    if (e == cudaSuccess) e = cudaMalloc(&b, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&piv, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc(&lmax, sizeof(int) * n);
    if (e == cudaSuccess) {
        MarkerDev M{};
        M.n = n;
        M.pos = const_cast<double*>(pos);
        M.nsupp = const_cast<int*>(nsupp);
        M.si = const_cast<int*>(si);
        M.sj = const_cast<int*>(sj);
        M.sd = const_cast<double*>(sd);
        M.ds = const_cast<double*>(ds);
        M.eps = eps;
        e = launch_epsilon_markers(M, n, Dx, A, b, piv, lmax, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFree(A);
    cudaFree(b);
    cudaFree(piv);
    cudaFree(lmax);
    if (e != cudaSuccess) return cuda_fail(e, "life_ibm_epsilon");
    return LIFE_OK;
}
