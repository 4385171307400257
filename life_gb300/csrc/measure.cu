// Measurement helper with no counterpart in the reference: the FP64 rate the
// GPU sustains, the denominator of the FP64 lattice kernels' roofline (the
// FP64 form's interior kernel is bound by the SM's FP64 unit, not by HBM).
//
// Every thread runs eight independent chains of fused multiply-adds,
// x = x * a + b, which keep the FP64 pipe busy without touching memory; the
// grid covers every SM with several blocks. One FMA counts as two FLOPs.
#include <cuda_runtime.h>

#include "../../include/life_gb300.h"
#include "life_internal.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double a, double b, double* sink) {
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += x[k];
    // the store is never taken (s stays finite), but the compiler cannot know
    if (s == -1.0) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" int life_measure_fp64_rate(double* gflops) {
    if (!gflops) return life::set_error(LIFE_ERR_INVALID, "NULL argument");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return life::cuda_fail(e, "life_measure_fp64_rate");
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double* sink = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaMalloc(&sink, sizeof(double) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(t0, 0);
        k_fp64_rate<<<blocks, threads>>>(iters, 0.999999, 1e-6, sink);
        cudaEventRecord(t1, 0);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(t1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (sink) cudaFree(sink);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (e != cudaSuccess) return life::cuda_fail(e, "life_measure_fp64_rate");
    const double flops = 2.0 * kChains * (double)iters * threads * blocks;
    *gflops = flops / (best * 1e-3) / 1e9;
    return LIFE_OK;
}
