// Observables recorder: the rows that ObjectsClass::writeTotalForces and
// ObjectsClass::writeTips append every tinfo steps (reference
// src/Objects.cpp:491-594), gathered on the device while the steps run, so a
// run records its force and tip histories without any host synchronisation.
//
// A row at step t holds the total force on all markers,
//   F[d] = - sum_n force_n[d] * 1.0 * eps_n * ds_n * forceScale
// summed in global marker order with the reference's operation order
// (src/Objects.cpp:518-528), and, for every flexible body in body order, the
// position and velocity of its last marker (src/Objects.cpp:576-588).
//
// The kernel runs at the end of every step (a node of the case's step graph);
// it writes a row only when t is a multiple of the recording interval, into a
// device buffer of `capacity` rows that life_case_records drains. Rows that
// find the buffer full are counted as dropped.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/life_gb300.h"
#include "life_internal.h"

using namespace life;

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

namespace {

// One warp. Lanes 0 and 1 run the x and y force sums (two independent
// sequential chains in marker order); lanes 2.. gather the tips.
__global__ void k_record(RecorderDev R, MarkerDev M, int t_host, const int* t_dev, int t_off) {
    const int t = t_dev ? *t_dev + t_off : t_host;
    if (t % R.every != 0) return;
    __shared__ int s_row;
    if (threadIdx.x == 0) {
        const int row = R.count[0];
        s_row = row < R.capacity ? row : -1;
        if (row < R.capacity) R.count[0] = row + 1;
        else R.count[1] += 1;
    }
    __syncwarp();
    const int row = s_row;
    if (row < 0) return;
    double* out = R.rows + (size_t)row * R.cols;
    const int lane = threadIdx.x;
    if (lane < 2) {
        double F = 0.0;
        for (int n = 0; n < M.n; n++) F -= M.force[2 * n + lane] * 1.0 * M.eps[n] * M.ds[n] * R.force_scale;
        out[lane] = F;
    }
    for (int q = lane; q < R.n_tips; q += 32) {
        const int m = R.tip[q];
        out[2 + 4 * q + 0] = M.pos[2 * m];
        out[2 + 4 * q + 1] = M.pos[2 * m + 1];
        out[2 + 4 * q + 2] = M.vel[2 * m];
        out[2 + 4 * q + 3] = M.vel[2 * m + 1];
    }
    if (lane == 0) R.t[row] = t;
}

}  // namespace

namespace life {

cudaError_t launch_record(const LifeCase* c, int t, cudaStream_t s) {
    if (c->rec.every <= 0) return cudaSuccess;
    k_record<<<1, 32, 0, s>>>(c->rec, c->M, t, c->t_dev, c->t_off);
    return cudaGetLastError();
}

void free_recorder(LifeCase* c) {
    if (c->rec.rows) cudaFree(c->rec.rows);
    if (c->rec.t) cudaFree(c->rec.t);
    if (c->rec.count) cudaFree(c->rec.count);
    if (c->rec.tip) cudaFree(c->rec.tip);
    const int gen = c->rec_gen;
    c->rec = RecorderDev{};
    c->rec_gen = gen + 1;
}

}  // namespace life

extern "C" int life_case_record(LifeCase* c, int32_t every, int32_t capacity) {
    if (!c) return set_error(LIFE_ERR_INVALID, "case is NULL");
    if (every > 0 && capacity <= 0) return set_error(LIFE_ERR_INVALID, "recorder capacity must be positive");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c->device) cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream));
    free_recorder(c);
    int rc = LIFE_OK;
    if (every > 0) {
        std::vector<int> tips;
        for (const HBody& b : c->obj.b)
            if (b.flex && !b.nodes.empty()) tips.push_back(b.nodes.back());
        RecorderDev& R = c->rec;
        R.every = every;
        R.capacity = capacity;
        R.n_tips = (int)tips.size();
        R.cols = 2 + 4 * R.n_tips;
        R.force_scale = c->Dm * c->Dx / (c->Dt * c->Dt) * 1.0 / c->Dx;
        cudaError_t e = cudaMalloc(&R.rows, sizeof(double) * (size_t)capacity * R.cols);
        if (e == cudaSuccess) e = cudaMalloc(&R.t, sizeof(int) * (size_t)capacity);
        if (e == cudaSuccess) e = cudaMalloc(&R.count, sizeof(int) * 2);
        if (e == cudaSuccess) e = cudaMalloc(&R.tip, sizeof(int) * std::max<size_t>(1, tips.size()));
        if (e == cudaSuccess) e = cudaMemsetAsync(R.count, 0, sizeof(int) * 2, c->stream);
        if (e == cudaSuccess && !tips.empty())
            e = cudaMemcpyAsync(R.tip, tips.data(), sizeof(int) * tips.size(), cudaMemcpyHostToDevice, c->stream);
        // the row of the current state, as the reference writes one before
        // its first step (src/main.cpp:61)
        if (e == cudaSuccess) {
            const int* td = c->t_dev;
            c->t_dev = nullptr;
            e = launch_record(c, c->t, c->stream);
            c->t_dev = td;
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            free_recorder(c);
            rc = cuda_fail(e, "life_case_record");
        }
    }
    if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return rc;
}

extern "C" int life_case_records(LifeCase* c, int32_t max_rows, int32_t* n_rows, int32_t* n_cols, int32_t* t,
                                 double* rows, int32_t* dropped) {
    if (!c || !n_rows) return set_error(LIFE_ERR_INVALID, "NULL argument");
    *n_rows = 0;
    if (n_cols) *n_cols = c->rec.cols;
    if (dropped) *dropped = 0;
    if (c->rec.every <= 0) return set_error(LIFE_ERR_INVALID, "no recorder on this case (life_case_record)");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c->device) cudaSetDevice(c->device);
    int cnt[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(cnt, c->rec.count, sizeof cnt, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    int rc = LIFE_OK;
    if (e == cudaSuccess && !t && !rows) {
        // query: how many rows are waiting, nothing drained
        *n_rows = cnt[0];
        if (dropped) *dropped = cnt[1];
    } else if (e == cudaSuccess && cnt[0] > max_rows) {
        rc = set_error(LIFE_ERR_INVALID, "life_case_records: " + std::to_string(cnt[0]) + " rows recorded, buffer holds " +
                                             std::to_string(max_rows));
    } else if (e == cudaSuccess) {
        const int n = cnt[0];
        if (n > 0 && t) e = cudaMemcpyAsync(t, c->rec.t, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && n > 0 && rows)
            e = cudaMemcpyAsync(rows, c->rec.rows, sizeof(double) * (size_t)n * c->rec.cols, cudaMemcpyDeviceToHost,
                                c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->rec.count, 0, sizeof(int) * 2, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess) {
            *n_rows = n;
            if (dropped) *dropped = cnt[1];
        }
    }
    if (e != cudaSuccess) rc = cuda_fail(e, "life_case_records");
    if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return rc;
}
