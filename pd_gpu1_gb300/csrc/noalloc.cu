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
// symbol's name as a device address.  The address belongs to the CUDA context
// (the module is loaded once per context), so the first call in each context,
// with that context current, looks it up with cudaGetSymbolAddress and caches
// it under the context's unique id (cuCtxGetId): a context created later on
// the same device, for instance the primary context rebuilt after
// cudaDeviceReset, or a driver-API caller's own context, gets its own lookup.
// That first call should come before any stream capture that includes this
// entry point.
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

// Address cache keyed by context id.  The id comes from the driver's
// cuCtxGetCurrent + cuCtxGetId, reached through the runtime's entry-point
// query so that the library needs no link to the driver library.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
constexpr int kCacheSlots = 64;
std::mutex g_lock;
struct CacheSlot {
    unsigned long long ctx_id;
    double* addr;
};
CacheSlot g_cache[kCacheSlots] = {};
int g_cache_next = 0;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

// Unique id of the current context (0: none could be had; the caller then
// looks the address up without caching it).
unsigned long long current_ctx_id() {
    if (!g_ctx_current || !g_ctx_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return 0;
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != 0 || !ctx || g_ctx_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of g_static_partials in the current context (looked up once
// per context).
int static_scratch(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PD_ERR_CUDA;
    // cudaGetDevice does not create the primary context; the runtime call
    // below does, so the id is read after it on a first call
    std::lock_guard<std::mutex> g(g_lock);
    unsigned long long id = current_ctx_id();
    if (id) {
        for (const CacheSlot& c : g_cache)
            if (c.ctx_id == id) {
                *out = c.addr;
                return PD_OK;
            }
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_partials) != cudaSuccess || !p) return PD_ERR_CUDA;
    if (!id) id = current_ctx_id();
    if (id) {
        g_cache[g_cache_next] = CacheSlot{id, static_cast<double*>(p)};
        g_cache_next = (g_cache_next + 1) % kCacheSlots;
    }
    *out = static_cast<double*>(p);
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
    // launched through cudaLaunchKernel so that the status is this call's own:
    // an error left by the caller's earlier work is neither returned nor cleared
    if (nparts > 0) {
        void* a1[] = {(void*)&dev_x, (void*)&n, (void*)&part};
        if (cudaLaunchKernel((const void*)k_static_partials, dim3(nparts), dim3(kStaticThreads), a1, 0, s) !=
            cudaSuccess)
            return PD_ERR_CUDA;
    }
    int np = nparts;
    void* a2[] = {(void*)&part, (void*)&np, (void*)&dev_result};
    if (cudaLaunchKernel((const void*)k_static_final, dim3(1), dim3(kStaticThreads), a2, 0, s) != cudaSuccess)
        return PD_ERR_CUDA;
    return PD_OK;
}
