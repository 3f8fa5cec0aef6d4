// Allocation-free sum of a device array (pd_reduce_sum_static).
//
// Some callers cannot allocate device memory: code that runs while another
// component owns the CUDA allocator (a memory pool handed out up front, a
// host runtime that forbids cudaMalloc on its threads), callers that reach
// this library through a foreign-function interface without a CUDA context
// object of ours, or code paths that must not allocate for real-time reasons.
// This entry point gives them the deterministic FP64 sum without a context and
// without any allocation: its block partial sums live in a fixed array in the
// library's own device memory.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds it (64 KiB) until the process exits.  Host code cannot use the
// symbol's name as a device address; the first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and caches
// it.  That first call should therefore come before any stream capture that
// includes this entry point.
#include <mutex>

#include "pd_internal.cuh"

namespace pdg {
namespace {

constexpr int kStaticThreads = 256;
constexpr int kStaticItems = 16;                                  // elements per thread
constexpr int64_t kStaticChunk = (int64_t)kStaticThreads * kStaticItems;  // elements per block
constexpr int kStaticPartials = 8192;                             // blocks one call may use

__device__ __align__(256) double g_static_partials[kStaticPartials];

// Pass 1: block b sums elements [b*chunk, (b+1)*chunk) in a fixed order.
__global__ void k_static_partials(const double* __restrict__ x, int64_t n, double* __restrict__ part) {
    __shared__ double sm[kStaticThreads / 32];
    const int64_t base = blockIdx.x * kStaticChunk;
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < kStaticItems; k++) {
        const int64_t i = base + (int64_t)k * kStaticThreads + threadIdx.x;
        if (i < n) v += x[i];
    }
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < kStaticThreads / 32; w++) r += sm[w];
        part[blockIdx.x] = r;
    }
}

// Pass 2: one block sums the partials of pass 1 in a fixed order.
__global__ void k_static_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    __shared__ double sm[kStaticThreads / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < nparts; i += kStaticThreads) v += part[i];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < kStaticThreads / 32; w++) r += sm[w];
        *out = r;
    }
}

constexpr int kMaxDevices = 64;
std::mutex g_lock;
double* g_partials_addr[kMaxDevices] = {};

// Device address of g_static_partials on the current device (looked up once per device).
int static_scratch(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PD_ERR_CUDA;
    std::lock_guard<std::mutex> g(g_lock);
    if (!g_partials_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_partials) != cudaSuccess || !p) return PD_ERR_CUDA;
        g_partials_addr[dev] = static_cast<double*>(p);
    }
    *out = g_partials_addr[dev];
    return PD_OK;
}

}  // namespace
}  // namespace pdg

extern "C" int pd_reduce_sum_static(const double* dev_x, int64_t n, double* dev_result, void* stream) {
    using namespace pdg;
    if (!dev_x || !dev_result || n < 0) return PD_ERR_ARG;
    if (n > (int64_t)kStaticPartials * kStaticChunk) return PD_ERR_ARG;  // more partials than the array holds
    double* part = nullptr;
    int rc = static_scratch(&part);
    if (rc) return rc;
    cudaStream_t s = st(stream);
    const int nparts = (int)((n + kStaticChunk - 1) / kStaticChunk);
    if (nparts > 0) k_static_partials<<<nparts, kStaticThreads, 0, s>>>(dev_x, n, part);
    k_static_final<<<1, kStaticThreads, 0, s>>>(part, nparts, dev_result);
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}
