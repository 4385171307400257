// life_ibm_epsilon_noalloc: the epsilon solve of life_ibm_epsilon without any
// device allocation, for callers that cannot call cudaMalloc -- code whose
// device memory all comes from another allocator's pool (a framework's caching
// allocator, a fixed arena sized at start-up) or that runs in a loop where the
// implicit device synchronisation of cudaMalloc/cudaFree is not allowed.
//
// The n x n system, right-hand side and pivot arrays live in one file-scope
// device array sized for LIFE_NOALLOC_MAX_MARKERS markers. Every GPU that
// loads the library holds that array until the process exits. All calls share
// it and it keeps the last call's contents; the kernel overwrites every entry
// it reads (the matrix is cleared, the right-hand side set to 1) before using
// it. Calls whose work overlaps on the GPU (different streams, or different
// host threads without ordering) race on the array and must be serialised by
// the caller.
//
// Host code cannot use the array's name as a device address: in host code it
// names a host-side stand-in. The device address is fetched with
// cudaGetSymbolAddress once per device, with that device current, by the first
// call made on it; that first call should come before any stream capture on
// the device. The address is kept for the life of the process, so the library
// must not be used on a device across a cudaDeviceReset.
//
// The call is stream-ordered: it queues the kernel on the caller's stream and
// returns without waiting. eps is ready once the caller's stream has reached
// that point (cudaStreamSynchronize, an event, or later work on the stream).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fem_kernels.h"

using namespace life;

#define LIFE_NOALLOC_MAX_MARKERS 256
#define LIFE_NOALLOC_MAX_DEVICES 64

namespace {
constexpr size_t kN = LIFE_NOALLOC_MAX_MARKERS;
constexpr size_t kOffB = kN * kN * sizeof(double);                 // right-hand side
constexpr size_t kOffPiv = kOffB + kN * sizeof(double);            // pivots
constexpr size_t kOffLmax = kOffPiv + kN * sizeof(int);            // last multiplier rows
constexpr size_t kBytes = kOffLmax + kN * sizeof(int);

// 516 KiB: the n x n epsilon system for n <= 256 plus its vectors.
static __device__ __align__(256) unsigned char g_epsilon_scratch[kBytes];

std::mutex g_mu;
unsigned char* g_addr[LIFE_NOALLOC_MAX_DEVICES] = {nullptr};

int scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_epsilon_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_epsilon_scratch)");
        g_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_addr[device];
    return LIFE_OK;
}
}  // namespace

extern "C" int life_ibm_epsilon_noalloc(const double* pos, const int32_t* nsupp, const int32_t* si,
                                        const int32_t* sj, const double* sd, const double* ds, int32_t n,
                                        double Dx, double* eps, void* stream) {
    if (n > LIFE_NOALLOC_MAX_MARKERS)
        return set_error(LIFE_ERR_INVALID, "life_ibm_epsilon_noalloc: " + std::to_string(n) +
                                               " markers exceed the static maximum of " +
                                               std::to_string(LIFE_NOALLOC_MAX_MARKERS) +
                                               "; use life_ibm_epsilon for larger sets");
    if (n < 0 || (n > 0 && (!pos || !nsupp || !si || !sj || !sd || !ds || !eps)))
        return set_error(LIFE_ERR_INVALID, "bad arguments");
    if (n == 0) return LIFE_OK;
    if (!(Dx > 0.0)) return set_error(LIFE_ERR_INVALID, "Dx must be positive");
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (device < 0 || device >= LIFE_NOALLOC_MAX_DEVICES)
        return set_error(LIFE_ERR_INVALID, "device index beyond the supported range");
    unsigned char* base = nullptr;
    if (int rc = scratch_address(device, &base)) return rc;
    MarkerDev M{};
    M.n = n;
    M.pos = const_cast<double*>(pos);
    M.nsupp = const_cast<int*>(nsupp);
    M.si = const_cast<int*>(si);
    M.sj = const_cast<int*>(sj);
    M.sd = const_cast<double*>(sd);
    M.ds = const_cast<double*>(ds);
    M.eps = eps;
    cudaStream_t s = (cudaStream_t)stream;
    e = launch_epsilon_markers(M, n, Dx, reinterpret_cast<double*>(base), reinterpret_cast<double*>(base + kOffB),
                               reinterpret_cast<int*>(base + kOffPiv), reinterpret_cast<int*>(base + kOffLmax), s);
    if (e != cudaSuccess) return cuda_fail(e, "life_ibm_epsilon_noalloc");
    return LIFE_OK;
}
