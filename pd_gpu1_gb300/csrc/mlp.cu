// Per-node MLP of the learned ADR warm start (no reference counterpart: the
// reference runs a fixed number of ADR steps, Solve_Plate_Tensile.cu:106).
//
// Network: 8 -> 128 -> 128 -> 128 -> 2, GELU (erf form) on the hidden layers,
// 34,434 parameters.  Weights are BF16 operands of the tensor cores with FP32
// master copies for the optimizer; every product is a BF16 x BF16 -> FP32
// tcgen05.mma (kind::f16) issued by one thread, operands staged in shared
// memory in the canonical K-major layout without swizzle, accumulators in
// tensor memory read back with tcgen05.ld for the fused epilogues:
//   forward   Z = H W^T + b, H' = GELU(Z)            (epilogue: bias, GELU, BF16)
//   backward  dH = dZ' W, dZ = dH * GELU'(Z)         (epilogue: GELU', BF16)
//             dW = dZ^T H (split over row blocks)    (epilogue: FP32 partials)
// One kernel template serves every product: D[M x N] = A[M x K] * B[N x K]^T
// with A and B read through arbitrary element strides, so transposed operands
// (dZ^T, H^T, W) are gathered by the loader instead of being stored twice.
//
// Padding: the 8 inputs are padded to K = 16 and the 2 outputs to N = 16 with
// zero weights; tiles are 128 rows (M) by 16 or 128 columns (N).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "pd_internal.cuh"

namespace pdg {
namespace mlp {

constexpr int kIn = 8, kInPad = 16, kHid = 128, kOut = 2, kOutPad = 16;
constexpr int kParams = kHid * kIn + kHid + 2 * (kHid * kHid + kHid) + kOut * kHid + kOut;  // 34,434
constexpr int kTileM = 128;
constexpr int kChunkK = 64;
constexpr int kThreads = 128;
constexpr long long kSpinLimit = 1ll << 24;  // bounded mbarrier wait

enum Epi { E_F32 = 0, E_GELU = 1, E_BWD = 2, E_PARTIAL = 3 };

struct GemmArgs {
    const __nv_bfloat16* A;
    int64_t sam, sak;  // element strides of A(m, k)
    const __nv_bfloat16* B;
    int64_t sbn, sbk;  // element strides of B(n, k)
    int64_t M, N, K;
    int64_t k_per_split;
    int epi;
    float* D;            // E_F32: [M][ldd]; E_PARTIAL: [split][M][ldd]
    int64_t ldd;
    const float* bias;   // E_F32 / E_GELU: [N]
    float* Z;            // E_GELU: pre-activation [M][ldh]
    __nv_bfloat16* H;    // E_GELU: activation [M][ldh]; E_BWD: dZ [M][ldh]
    int64_t ldh;
    const float* Zin;    // E_BWD: pre-activation [M][ldh]
    int* err;
    long long spin_limit;  // iterations of each bounded mbarrier wait
    int issue;             // 0: issue neither the products nor their commit (bounded-wait self-check)
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: canonical K-major layout, no swizzle.
// Core matrices are 8 rows x 16 bytes stored contiguously (128 B); lbo is the
// byte distance between core matrices adjacent in K, sbo between core matrices
// adjacent in M/N (8-row groups).  Version field (bits 46-47) = 1.
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3fffu);
    d |= (uint64_t)((lbo >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fffu) << 32;
    d |= (uint64_t)1 << 46;
    return d;  // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Byte offset of element (row r, column k) of a K-major tile with kChunkK columns.
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    constexpr uint32_t lbo = 128, sbo = (kChunkK / 8) * 128;
    return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 3) * lbo + (uint32_t)(r & 7) * 16 + (uint32_t)(k & 7) * 2;
}

// Stage rows [r0, r0 + rows) x columns [k0, k0 + kChunkK) of X(r, k) =
// X[r * sr + k * sk] into a K-major tile, zero outside [0, R) x [0, Kmax).
__device__ void load_tile(unsigned char* tile, const __nv_bfloat16* X, int64_t sr, int64_t sk, int64_t r0, int rows,
                          int64_t R, int64_t k0, int64_t Kmax) {
    const int groups = rows * (kChunkK / 8);
    if (sk == 1) {  // 8 consecutive k per 16-byte vector
        for (int g = threadIdx.x; g < groups; g += kThreads) {
            const int r = g / (kChunkK / 8), kg = (g % (kChunkK / 8)) * 8;
            const int64_t gr = r0 + r, gk = k0 + kg;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gr < R) {
                const __nv_bfloat16* src = X + gr * sr + gk;
                if (gk + 8 <= Kmax && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    v = *reinterpret_cast<const uint4*>(src);
                } else {
                    unsigned short e[8];
                    for (int j = 0; j < 8; j++)
                        e[j] = gk + j < Kmax ? __bfloat16_as_ushort(src[j]) : (unsigned short)0;
                    v = make_uint4(e[0] | (e[1] << 16), e[2] | (e[3] << 16), e[4] | (e[5] << 16), e[6] | (e[7] << 16));
                }
            }
            *reinterpret_cast<uint4*>(tile + tile_off(r, kg)) = v;
        }
    } else {  // element by element (strided k)
        for (int g = threadIdx.x; g < rows * kChunkK; g += kThreads) {
            const int k = g / rows, r = g % rows;  // consecutive threads: consecutive rows
            const int64_t gr = r0 + r, gk = k0 + k;
            unsigned short e = 0;
            if (gr < R && gk < Kmax) e = __bfloat16_as_ushort(X[gr * sr + gk * sk]);
            *reinterpret_cast<unsigned short*>(tile + tile_off(r, k)) = e;
        }
    }
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, long long limit) {
    for (long long it = 0; it < limit; it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}

// D[M x N] = A[M x K] * B[N x K]^T for one 128 x NT tile and one K range.
template <int NT>
__global__ void __launch_bounds__(kThreads) k_gemm(GemmArgs g) {
    static_assert(NT == 16 || NT == 128, "tile width");
    constexpr uint32_t kCols = NT < 32 ? 32 : NT;  // TMEM allocation: power of two >= 32
    constexpr uint32_t kIdesc = make_idesc(kTileM, NT);
    __shared__ __align__(1024) unsigned char sa[kTileM * kChunkK * 2];
    __shared__ __align__(1024) unsigned char sb[NT * kChunkK * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kTileM, n0 = (int64_t)blockIdx.y * NT;
    const int64_t kb = (int64_t)blockIdx.z * g.k_per_split;
    const int64_t ke = kb + g.k_per_split < g.K ? kb + g.k_per_split : g.K;
    const uint32_t bar_a = smem_addr(&bar);

    if (threadIdx.x == 0) {
        failed = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    uint32_t phase = 0;
    int chunks = 0;
    for (int64_t k0 = kb; k0 < ke; k0 += kChunkK, chunks++) {
        if (chunks > 0) {  // the previous chunk's products have read the tiles
            if (!mbar_wait(bar_a, phase, g.spin_limit)) failed = 1;
            phase ^= 1;
        }
        __syncthreads();
        if (failed) break;
        load_tile(sa, g.A, g.sam, g.sak, m0, kTileM, g.M, k0, ke);
        load_tile(sb, g.B, g.sbn, g.sbk, n0, NT, g.N, k0, ke);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0 && g.issue) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int ksteps = (int)((ke - k0 < kChunkK ? ke - k0 : kChunkK) + 15) / 16;
            for (int j = 0; j < ksteps; j++) {
                const uint64_t da = make_desc(smem_addr(sa) + j * 256, 128, (kChunkK / 8) * 128);
                const uint64_t db = make_desc(smem_addr(sb) + j * 256, 128, (kChunkK / 8) * 128);
                const uint32_t acc = (chunks > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_a)
                         : "memory");
        }
    }
    if (chunks > 0 && !failed) {
        if (!mbar_wait(bar_a, phase, g.spin_limit)) failed = 1;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (!failed && chunks > 0) {
        // epilogue: thread (warp w, lane l) owns row m0 + 32 w + l
        const int64_t m = m0 + 32 * warp + lane;
        for (int c0 = 0; c0 < NT; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (m >= g.M) continue;
            if (g.epi == E_GELU && !g.Z && n0 + c0 + 16 <= g.N && (g.ldh & 7) == 0) {
                // inference: the row's 16 activations as BF16 in two 16-byte stores
                // (the pre-activation is kept only for the backward pass)
                uint32_t h[8];
                for (int j = 0; j < 8; j++) {
                    const float z0 = __uint_as_float(v[2 * j]) + g.bias[n0 + c0 + 2 * j];
                    const float z1 = __uint_as_float(v[2 * j + 1]) + g.bias[n0 + c0 + 2 * j + 1];
                    const __nv_bfloat162 b2 = __floats2bfloat162_rn(gelu(z0), gelu(z1));
                    h[j] = *reinterpret_cast<const uint32_t*>(&b2);
                }
                uint4* dst = reinterpret_cast<uint4*>(g.H + m * g.ldh + n0 + c0);
                dst[0] = make_uint4(h[0], h[1], h[2], h[3]);
                dst[1] = make_uint4(h[4], h[5], h[6], h[7]);
                continue;
            }
            for (int j = 0; j < 16; j++) {
                const int64_t n = n0 + c0 + j;
                if (n >= g.N) break;
                const float d = __uint_as_float(v[j]);
                switch (g.epi) {
                    case E_F32:
                        g.D[m * g.ldd + n] = d + (g.bias ? g.bias[n] : 0.0f);
                        break;
                    case E_PARTIAL:
                        g.D[((int64_t)blockIdx.z * g.M + m) * g.ldd + n] = d;
                        break;
                    case E_GELU: {
                        const float z = d + g.bias[n];
                        if (g.Z) g.Z[m * g.ldh + n] = z;
                        g.H[m * g.ldh + n] = __float2bfloat16_rn(gelu(z));
                        break;
                    }
                    default: {  // E_BWD
                        const float z = g.Zin[m * g.ldh + n];
                        g.H[m * g.ldh + n] = __float2bfloat16_rn(d * gelu_grad(z));
                        break;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    if (threadIdx.x == 0 && failed) atomicExch(g.err, 1);
}

// Sum of split-K partials [splits][rows][cols] -> out, fixed order.
__global__ void k_reduce_splits(const float* __restrict__ part, int splits, int64_t n, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < splits; k++) s += part[(int64_t)k * n + i];
        out[i] = s;
    }
}

// Column sums of a BF16 [M][cols] matrix (bias gradients), one thread per column.
__global__ void k_colsum(const __nv_bfloat16* __restrict__ x, int64_t M, int cols, int64_t rows_per_block,
                         float* __restrict__ part) {
    const int c = threadIdx.x;
    if (c >= cols) return;
    const int64_t r0 = blockIdx.x * rows_per_block;
    const int64_t r1 = r0 + rows_per_block < M ? r0 + rows_per_block : M;
    float s = 0.0f;
    for (int64_t r = r0; r < r1; r++) s += __bfloat162float(x[r * cols + c]);
    part[(int64_t)blockIdx.x * cols + c] = s;
}

// Loss gradient of the mean squared error over the 2 outputs: dY = 2 (Y - T) / (2 M),
// stored as BF16 [M][16] (columns 2..15 zero); per-block loss partial sums.
__global__ void k_loss(const float* __restrict__ Y, const float* __restrict__ T, int64_t M,
                       __nv_bfloat16* __restrict__ dY, float* __restrict__ part) {
    __shared__ float sm[kThreads / 32];
    float l = 0.0f;
    const float scale = 1.0f / (float)M;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < M; r += (int64_t)gridDim.x * blockDim.x) {
        for (int j = 0; j < kOutPad; j++) {
            float d = 0.0f;
            if (j < kOut) {
                const float e = Y[r * kOutPad + j] - T[r * kOut + j];
                l += e * e;
                d = e * scale;  // d/dy of sum(e^2) / (2 M)
            }
            dY[r * kOutPad + j] = __float2bfloat16_rn(d);
        }
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int k = 0; k < kThreads / 32; k++) s += sm[k];
        part[blockIdx.x] = s;
    }
}

// Features of the free nodes (see pd_warm_features).  hist (may be null):
// the previous increment's departure from proportionality per unit load, x
// then y (2 n), and its damage increase (n); kHistScale brings the departure
// (of the order of 1e-5 on the warm-start plates, its change from one
// increment to the next 1e-6) near one.
constexpr double kHistScale = 65536.0;
__global__ void k_features(int64_t n, const double* __restrict__ y, const double* __restrict__ ux,
                           const double* __restrict__ uy, const double* __restrict__ dmg,
                           const double* __restrict__ hist, double inv_u, double inc, double edge,
                           __nv_bfloat16* __restrict__ X) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float f[kInPad];
        f[0] = (float)(ux[i] * inv_u);
        f[1] = (float)(uy[i] * inv_u);
        f[2] = (float)inc;
        f[3] = (float)dmg[i];
        f[4] = fabs(y[i]) > edge ? 1.0f : 0.0f;
        f[5] = hist ? (float)(hist[i] * kHistScale) : 0.0f;
        f[6] = hist ? (float)(hist[n + i] * kHistScale) : 0.0f;
        f[7] = hist ? (float)hist[2 * n + i] : 0.0f;
        for (int j = kIn; j < kInPad; j++) f[j] = 0.0f;
        for (int j = 0; j < kInPad; j++) X[i * kInPad + j] = __float2bfloat16_rn(f[j]);
    }
}

// The history of a converged increment: its departure from proportionality
// per unit load, ((u - up) - up delta / Up) / Up per component, and the
// damage it added.
__global__ void k_warm_record(int64_t n, const double* __restrict__ ux, const double* __restrict__ uy,
                              const double* __restrict__ dmg, const double* __restrict__ up,
                              const double* __restrict__ dmgp, double ratio, double inv_up, double* __restrict__ hist) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        hist[i] = ((ux[i] - up[i]) - up[i] * ratio) * inv_up;
        hist[n + i] = ((uy[i] - up[n + i]) - up[n + i] * ratio) * inv_up;
        hist[2 * n + i] = dmg[i] - dmgp[i];
    }
}

// Candidates of the free nodes: du = u (delta / U) + U (h + net / kHistScale),
// the skip term (the proportional, secant, increment) plus the previous
// increment's departure from proportionality per unit load h (zero without a
// history) and the network's correction of it; the skip term alone is
// written as the second candidate.  The network predicts how the departure
// changes from one increment to the next, so its output, and with it the
// BF16 network's node-to-node rounding noise, is a small correction on top of
// smooth FP64 terms.
__global__ void k_scale_out(int64_t n, const float* __restrict__ y, double U, double ratio,
                            const double* __restrict__ ux, const double* __restrict__ uy,
                            const double* __restrict__ hist, double* __restrict__ du) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double sx = ux[i] * ratio, sy = uy[i] * ratio;
        const double hx = hist ? hist[i] : 0.0, hy = hist ? hist[n + i] : 0.0;
        du[i] = fma(U, hx + (double)y[i * kOut] * (1.0 / kHistScale), sx);
        du[n + i] = fma(U, hy + (double)y[i * kOut + 1] * (1.0 / kHistScale), sy);
        du[2 * n + i] = sx;
        du[3 * n + i] = sy;
    }
}

// The network's correction U * net of the free nodes (x components, then y).
__global__ void k_correction(int64_t n, const float* __restrict__ y, double U, double* __restrict__ corr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        corr[i] = U * (double)y[i * kOut] * (1.0 / kHistScale);
        corr[n + i] = U * (double)y[i * kOut + 1] * (1.0 / kHistScale);
    }
}

// One smoothing pass of the correction over the bond family: each free node
// takes the mean of its own value and those of its intact neighbours (the
// prescribed boundary rows count with a zero correction).  One warp per SELL
// slice, lane per row, as the force kernels walk it.
// cols: the neighbour ids of the slots, cols[slot * stride] (the first word of
// the layout's per-slot record).
__global__ void k_smooth(int64_t nslices, int64_t n, const int* __restrict__ width, const int64_t* __restrict__ base,
                         const int64_t* __restrict__ fbase, const int* __restrict__ cols, int stride,
                         const uint32_t* __restrict__ bits, const double* __restrict__ in, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < nslices;
         s += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t r = s * 32 + lane;
        if (s * 32 >= n) continue;
        const bool row = r < n;
        double sx = row ? in[r] : 0.0, sy = row ? in[n + r] : 0.0;
        int cnt = 1;
        const int W = width[s];
        const int64_t b = base[s];
        for (int k = 0; k < W; k++) {
            const bool alive = row && ((bits[fbase[s] + k] >> lane) & 1u);
            if (alive) {
                const int c = cols[(b + (int64_t)k * 32 + lane) * stride];
                if (c < n) {
                    sx += in[c];
                    sy += in[n + c];
                }
                cnt++;
            }
        }
        if (row) {
            out[r] = sx / cnt;
            out[n + r] = sy / cnt;
        }
    }
}

// Candidates from a smoothed correction: the skip term u * delta / U plus
// the correction, and the skip term alone.
__global__ void k_combine(int64_t n, const double* __restrict__ corr, double U, double ratio,
                          const double* __restrict__ ux, const double* __restrict__ uy, const double* __restrict__ hist,
                          double* __restrict__ du) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double sx = ux[i] * ratio, sy = uy[i] * ratio;
        const double hx = hist ? hist[i] : 0.0, hy = hist ? hist[n + i] : 0.0;
        du[i] = fma(U, hx, sx) + corr[i];
        du[n + i] = fma(U, hy, sy) + corr[n + i];
        du[2 * n + i] = sx;
        du[3 * n + i] = sy;
    }
}

// ---- fused forward pass (inference) ------------------------------------------
//
// All four layers per 128-row tile in one persistent kernel: the BF16
// weights stay in shared memory (loaded once per CTA by the tensor memory
// accelerator), each layer's product goes to the same 128 TMEM columns, and
// its epilogue (bias, GELU, BF16) writes the activations back into shared
// memory as the next product's A operand, so activations never leave the SM.
// The input tiles arrive by TMA as well, one tile ahead: the next tile's rows
// are requested as soon as the first layer's product has read the current
// ones, and land while layers 2-4 run.  The products, their order of K steps
// and the epilogue arithmetic are those of k_gemm, so the outputs equal the
// layer-by-layer pass bit for bit.
//
// TMA layout: every operand loaded by TMA comes in boxes of 8 columns (16
// bytes) by all rows of the operand, so one box is a column of core matrices
// (8 rows x 16 bytes each, 128 bytes apart: SBO = 128) and consecutive boxes
// are the next 8 columns of K (LBO = rows x 16 bytes).  Every box starts at a
// column that is a multiple of 8 BF16 elements (16 bytes).
// Shared memory: W1 4 KB, W2 and W3 32 KB each, W4 4 KB, the activation tile
// 32 KB (two 64-wide K chunks, written by the epilogues), the input tile 4 KB
// and the biases: 110 KB, two CTAs per SM.
constexpr int kFusedSmem = 4096 + 2 * 32768 + 4096 + 32768 + 4096 + 2048;  // + the biases (1,600 bytes)
// Eight warps: warps w and w + 4 read the same 32 TMEM lanes (a warp reaches
// the lane quarter w % 4), the first the columns [0, 64) of each layer, the
// second [64, 128), so sixteen warps per SM share the epilogues.
constexpr int kFusedThreads = 256;
constexpr uint32_t kWeightBytes = 4096 + 2 * 32768 + 4096, kXBytes = 4096;

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t v[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One 2-D tile (x = column, y = row) of a tensor map into shared memory;
// completion is counted in bytes on the mbarrier.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

struct FusedArgs {
    CUtensorMap mX;   // [M][16] input rows, boxes of 8 columns x 128 rows
    CUtensorMap mW1;  // [128][16], 8 x 128
    CUtensorMap mW2;  // [128][128], 8 x 128
    CUtensorMap mW3;  // [128][128], 8 x 128
    CUtensorMap mW4;  // [16][128], 8 x 16
    int64_t M;
    const float *b1, *b2, *b3, *b4;
    float* Y;  // [M][2]
    int* err;
    long long spin_limit;
};

__global__ void __launch_bounds__(kFusedThreads) k_mlp_fused(const __grid_constant__ FusedArgs g) {
    extern __shared__ __align__(1024) unsigned char fsm[];
    unsigned char* sW1 = fsm;                  // 2 boxes x 2 KB (128 rows)
    unsigned char* sW2 = sW1 + 4096;           // 16 boxes x 2 KB
    unsigned char* sW3 = sW2 + 32768;          // 16 boxes x 2 KB
    unsigned char* sW4 = sW3 + 32768;          // 16 boxes x 256 B (16 rows)
    unsigned char* sH = sW4 + 4096;            // 2 chunks x 16 KB, K-major tiles (tile_off)
    unsigned char* sX = sH + 32768;            // 2 boxes x 2 KB
    float* sb = reinterpret_cast<float*>(sX + 4096);  // b1, b2, b3 (128 each), b4 (16)
    __shared__ __align__(8) uint64_t bar, tbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lane quarter, column half
    const uint32_t bar_a = smem_addr(&bar), tbar_a = smem_addr(&tbar);
    const uint32_t a0 = smem_addr(sH), x0 = smem_addr(sX), w1 = smem_addr(sW1), w2 = smem_addr(sW2),
                   w3 = smem_addr(sW3), w4 = smem_addr(sW4);
    const int64_t ntiles = (g.M + kTileM - 1) / kTileM;

    if (threadIdx.x == 0) {
        failed = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tbar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    // the weights and the first input tile, by TMA (the grid never exceeds the tiles)
    if (threadIdx.x == 0) {
        mbar_expect_tx(tbar_a, kWeightBytes + kXBytes);
        for (int b = 0; b < 2; b++) {
            tma_load_2d(w1 + b * 2048, &g.mW1, 8 * b, 0, tbar_a);
            tma_load_2d(x0 + b * 2048, &g.mX, 8 * b, (int)(blockIdx.x * kTileM), tbar_a);
        }
        for (int b = 0; b < 16; b++) {
            tma_load_2d(w2 + b * 2048, &g.mW2, 8 * b, 0, tbar_a);
            tma_load_2d(w3 + b * 2048, &g.mW3, 8 * b, 0, tbar_a);
            tma_load_2d(w4 + b * 256, &g.mW4, 8 * b, 0, tbar_a);
        }
    }
    for (int i = threadIdx.x; i < kHid; i += kFusedThreads) {
        sb[i] = g.b1[i];
        sb[kHid + i] = g.b2[i];
        sb[2 * kHid + i] = g.b3[i];
        if (i < kOutPad) sb[3 * kHid + i] = g.b4[i];
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t kIdH = make_idesc(kTileM, kHid), kIdO = make_idesc(kTileM, kOutPad);
    uint32_t phase = 0, tphase = 0;
    bool pending = true;  // a TMA transaction on tbar not yet waited for (uniform across the CTA)
    const int r = 32 * quarter + lane;  // this thread's row of the tile
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t m = tile * kTileM + r;
        // this tile's input rows (and, on the first tile, the weights)
        if (mbar_wait(tbar_a, tphase, g.spin_limit)) {
            tphase ^= 1;
            pending = false;
        } else {
            failed = 1;
        }
        for (int layer = 0; layer < 4; layer++) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            if (failed) break;
            if (threadIdx.x == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if (layer == 0) {
                    mma_f16(tmem, make_desc(x0, 2048, 128), make_desc(w1, 2048, 128), kIdH, 0u);
                } else {
                    for (int c = 0; c < 2; c++)
                        for (int j = 0; j < kChunkK / 16; j++) {
                            const int kk = c * (kChunkK / 16) + j;  // K step of 16 columns = two boxes
                            const uint64_t db = layer == 1   ? make_desc(w2 + kk * 4096, 2048, 128)
                                                : layer == 2 ? make_desc(w3 + kk * 4096, 2048, 128)
                                                             : make_desc(w4 + kk * 512, 256, 128);
                            mma_f16(tmem, make_desc(a0 + c * 16384 + j * 256, 128, 1024), db,
                                    layer == 3 ? kIdO : kIdH, (c > 0 || j > 0) ? 1u : 0u);
                        }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 bar_a)
                             : "memory");
            }
            if (!mbar_wait(bar_a, phase, g.spin_limit)) failed = 1;
            phase ^= 1;
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (failed) break;
            if (layer == 0 && tile + gridDim.x < ntiles) {
                // the first product has read the input tile: request the next one
                if (threadIdx.x == 0) {
                    mbar_expect_tx(tbar_a, kXBytes);
                    for (int b = 0; b < 2; b++)
                        tma_load_2d(x0 + b * 2048, &g.mX, 8 * b, (int)((tile + gridDim.x) * kTileM), tbar_a);
                }
                pending = true;
            }
            const uint32_t trow = tmem + ((uint32_t)(32 * quarter) << 16);
            if (layer < 3) {
                // bias, GELU, BF16 -> the next product's A operand (this warp's
                // half of the columns)
                const float* bias = sb + layer * kHid;
                for (int c0 = half * (kHid / 2); c0 < (half + 1) * (kHid / 2); c0 += 16) {
                    uint32_t v[16];
                    tmem_ld16(trow + (uint32_t)c0, v);
                    uint32_t h[8];
                    for (int jj = 0; jj < 8; jj++) {
                        const float z0 = __uint_as_float(v[2 * jj]) + bias[c0 + 2 * jj];
                        const float z1 = __uint_as_float(v[2 * jj + 1]) + bias[c0 + 2 * jj + 1];
                        const __nv_bfloat162 b2 = __floats2bfloat162_rn(gelu(z0), gelu(z1));
                        h[jj] = *reinterpret_cast<const uint32_t*>(&b2);
                    }
                    unsigned char* chunk = sH + (c0 / kChunkK) * 16384;
                    *reinterpret_cast<uint4*>(chunk + tile_off(r, c0 % kChunkK)) = make_uint4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<uint4*>(chunk + tile_off(r, c0 % kChunkK + 8)) =
                        make_uint4(h[4], h[5], h[6], h[7]);
                }
            } else if (half == 0) {
                uint32_t v[16];
                tmem_ld16(trow, v);
                if (m < g.M)
                    *reinterpret_cast<float2*>(g.Y + m * kOut) =
                        make_float2(__uint_as_float(v[0]) + sb[3 * kHid], __uint_as_float(v[1]) + sb[3 * kHid + 1]);
            }
        }
        if (failed) break;
    }
    // a copy still in flight lands before the CTA's shared memory goes away
    if (pending) mbar_wait(tbar_a, tphase, g.spin_limit);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
    if (threadIdx.x == 0 && failed) atomicExch(g.err, 1);
}

}  // namespace mlp
}  // namespace pdg

using namespace pdg;
using namespace pdg::mlp;

// Parameter layout (flat FP32, PyTorch order): W1[128][8], b1[128], W2[128][128],
// b2[128], W3[128][128], b3[128], W4[2][128], b4[2].
namespace {
constexpr int oW1 = 0, ob1 = oW1 + kHid * kIn, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kHid * kHid, oW4 = ob3 + kHid, ob4 = oW4 + kOut * kHid, oEnd = ob4 + kOut;
static_assert(oEnd == kParams, "parameter count");

// master parameters -> padded BF16 operands and FP32 biases
__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* W1, __nv_bfloat16* W2, __nv_bfloat16* W3,
                       __nv_bfloat16* W4, float* b1, float* b2, float* b3, float* b4) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kHid * kHid; i += gridDim.x * blockDim.x) {
        W2[i] = __float2bfloat16_rn(p[oW2 + i]);
        W3[i] = __float2bfloat16_rn(p[oW3 + i]);
        if (i < kHid * kInPad) {
            const int o = i / kInPad, c = i % kInPad;
            W1[i] = __float2bfloat16_rn(c < kIn ? p[oW1 + o * kIn + c] : 0.0f);
        }
        if (i < kOutPad * kHid) {
            const int o = i / kHid, c = i % kHid;
            W4[i] = __float2bfloat16_rn(o < kOut ? p[oW4 + o * kHid + c] : 0.0f);
        }
        if (i < kHid) {
            b1[i] = p[ob1 + i];
            b2[i] = p[ob2 + i];
            b3[i] = p[ob3 + i];
        }
        if (i < kOutPad) b4[i] = i < kOut ? p[ob4 + i] : 0.0f;
    }
}

// padded gradients -> flat gradient vector
__global__ void k_unpack_grad(const float* gW1, const float* gb1, const float* gW2, const float* gb2,
                              const float* gW3, const float* gb3, const float* gW4, const float* gb4, float* g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        float v;
        if (i < ob1) v = gW1[(i / kIn) * kInPad + i % kIn];
        else if (i < oW2) v = gb1[i - ob1];
        else if (i < ob2) v = gW2[i - oW2];
        else if (i < oW3) v = gb2[i - ob2];
        else if (i < ob3) v = gW3[i - oW3];
        else if (i < oW4) v = gb3[i - ob3];
        else if (i < ob4) v = gW4[i - oW4];  // rows 0, 1 of the [16][128] gradient
        else v = gb4[i - ob4];
        g[i] = v;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        m1[i] = b1 * m1[i] + (1.0f - b1) * gi;
        m2[i] = b2 * m2[i] + (1.0f - b2) * gi * gi;
        p[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + eps);
    }
}
}  // namespace

struct pd_mlp {
    int64_t max_rows = 0;
    int* err = nullptr;
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // master, gradient, Adam moments
    __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W4 = nullptr;
    float *b1 = nullptr, *b2 = nullptr, *b3 = nullptr, *b4 = nullptr;
    float *gW1 = nullptr, *gW2 = nullptr, *gW3 = nullptr, *gW4 = nullptr;
    float *gb1 = nullptr, *gb2 = nullptr, *gb3 = nullptr, *gb4 = nullptr;
    // activations for max_rows rows
    float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Y = nullptr;
    __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dY = nullptr, *dZ = nullptr, *dZb = nullptr;
    float* part = nullptr;  // split-K partials / column-sum partials
    int64_t part_floats = 0;
    int64_t step = 0;
    int64_t launches = 0;  // kernels launched on this handle
    std::string errmsg;
};

namespace {

constexpr int64_t kRowsPerSplit = 1024;

int launch_gemm(pd_mlp* n, const GemmArgs& a0, int nt, cudaStream_t s, int splits = 1) {
    GemmArgs a = a0;
    a.err = n->err;
    if (a.k_per_split <= 0) a.k_per_split = a.K;
    if (a.spin_limit <= 0) a.spin_limit = kSpinLimit;
    const dim3 grid((unsigned)((a.M + kTileM - 1) / kTileM), (unsigned)((a.N + nt - 1) / nt), (unsigned)splits);
    if (nt == 16)
        k_gemm<16><<<grid, kThreads, 0, s>>>(a);
    else
        k_gemm<128><<<grid, kThreads, 0, s>>>(a);
    n->launches++;
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

GemmArgs gemm(const __nv_bfloat16* A, int64_t sam, int64_t sak, const __nv_bfloat16* B, int64_t sbn, int64_t sbk,
              int64_t M, int64_t N, int64_t K) {
    GemmArgs a{};
    a.A = A, a.sam = sam, a.sak = sak, a.B = B, a.sbn = sbn, a.sbk = sbk, a.M = M, a.N = N, a.K = K;
    a.k_per_split = K;
    a.spin_limit = kSpinLimit;
    a.issue = 1;
    return a;
}

// forward over M rows of X (BF16 [M][16]); Y (FP32 [M][16]) receives the outputs;
// keep_z: store the pre-activations for a backward pass
int forward(pd_mlp* n, const __nv_bfloat16* X, int64_t M, cudaStream_t s, bool keep_z = true) {
    int rc;
    GemmArgs a = gemm(X, kInPad, 1, n->W1, kInPad, 1, M, kHid, kInPad);
    a.epi = E_GELU, a.bias = n->b1, a.Z = keep_z ? n->Z1 : nullptr, a.H = n->H1, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    a = gemm(n->H1, kHid, 1, n->W2, kHid, 1, M, kHid, kHid);
    a.epi = E_GELU, a.bias = n->b2, a.Z = keep_z ? n->Z2 : nullptr, a.H = n->H2, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    a = gemm(n->H2, kHid, 1, n->W3, kHid, 1, M, kHid, kHid);
    a.epi = E_GELU, a.bias = n->b3, a.Z = keep_z ? n->Z3 : nullptr, a.H = n->H3, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    a = gemm(n->H3, kHid, 1, n->W4, kHid, 1, M, kOutPad, kHid);
    a.epi = E_F32, a.bias = n->b4, a.D = n->Y, a.ldd = kOutPad;
    return launch_gemm(n, a, 16, s);
}

// dW[out][in] = sum over rows of dZ[m][out] * Hin[m][in]  (split over row blocks)
int weight_grad(pd_mlp* n, const __nv_bfloat16* dZ, int64_t ldz, int64_t nout, const __nv_bfloat16* Hin,
                int64_t ldi, int64_t nin, int64_t M, float* out, cudaStream_t s) {
    const int splits = (int)((M + kRowsPerSplit - 1) / kRowsPerSplit);
    GemmArgs a = gemm(dZ, 1, ldz, Hin, 1, ldi, nout, nin, M);
    a.epi = E_PARTIAL, a.D = n->part, a.ldd = nin, a.k_per_split = kRowsPerSplit;
    int rc = launch_gemm(n, a, nin <= 16 ? 16 : 128, s, splits);
    if (rc) return rc;
    const int64_t cnt = nout * nin;
    k_reduce_splits<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(n->part, splits, cnt, out);
    n->launches++;
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

int bias_grad(pd_mlp* n, const __nv_bfloat16* dZ, int64_t M, int cols, float* out, cudaStream_t s) {
    const int64_t rpb = 256;
    const int blocks = (int)((M + rpb - 1) / rpb);
    k_colsum<<<blocks, 128, 0, s>>>(dZ, M, cols, rpb, n->part);
    k_reduce_splits<<<1, 128, 0, s>>>(n->part, blocks, cols, out);
    n->launches += 2;
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

// forward + backward over M rows; gradient into n->g (flat), loss (mean of
// squared errors over rows and outputs, halved) into *loss
int grad(pd_mlp* n, const __nv_bfloat16* X, const float* T, int64_t M, float* loss, cudaStream_t s) {
    int rc = forward(n, X, M, s);
    if (rc) return rc;
    const int lb = (int)std::min<int64_t>((M + kThreads - 1) / kThreads, 1024);
    k_loss<<<lb, kThreads, 0, s>>>(n->Y, T, M, n->dY, n->part);
    n->launches++;
    // layer 4: dW4 = dY^T H3, db4 = colsum dY, dH3 = dY W4 -> dZ3
    std::vector<float> lp(lb);
    cudaMemcpyAsync(lp.data(), n->part, lb * sizeof(float), cudaMemcpyDeviceToHost, s);
    if ((rc = weight_grad(n, n->dY, kOutPad, kOutPad, n->H3, kHid, kHid, M, n->gW4, s))) return rc;
    if ((rc = bias_grad(n, n->dY, M, kOutPad, n->gb4, s))) return rc;
    GemmArgs a = gemm(n->dY, kOutPad, 1, n->W4, 1, kHid, M, kHid, kOutPad);
    a.epi = E_BWD, a.Zin = n->Z3, a.H = n->dZ, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    // layer 3: dW3 = dZ3^T H2, db3, dH2 = dZ3 W3 -> dZ2
    if ((rc = weight_grad(n, n->dZ, kHid, kHid, n->H2, kHid, kHid, M, n->gW3, s))) return rc;
    if ((rc = bias_grad(n, n->dZ, M, kHid, n->gb3, s))) return rc;
    a = gemm(n->dZ, kHid, 1, n->W3, 1, kHid, M, kHid, kHid);
    a.epi = E_BWD, a.Zin = n->Z2, a.H = n->dZb, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    // layer 2: dW2 = dZ2^T H1, db2, dH1 = dZ2 W2 -> dZ1
    if ((rc = weight_grad(n, n->dZb, kHid, kHid, n->H1, kHid, kHid, M, n->gW2, s))) return rc;
    if ((rc = bias_grad(n, n->dZb, M, kHid, n->gb2, s))) return rc;
    a = gemm(n->dZb, kHid, 1, n->W2, 1, kHid, M, kHid, kHid);
    a.epi = E_BWD, a.Zin = n->Z1, a.H = n->dZ, a.ldh = kHid;
    if ((rc = launch_gemm(n, a, 128, s))) return rc;
    // layer 1: dW1 = dZ1^T X, db1
    if ((rc = weight_grad(n, n->dZ, kHid, kHid, X, kInPad, kInPad, M, n->gW1, s))) return rc;
    if ((rc = bias_grad(n, n->dZ, M, kHid, n->gb1, s))) return rc;
    k_unpack_grad<<<64, 256, 0, s>>>(n->gW1, n->gb1, n->gW2, n->gb2, n->gW3, n->gb3, n->gW4, n->gb4, n->g);
    n->launches++;
    int herr = 0;
    cudaMemcpyAsync(&herr, n->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return PD_ERR_CUDA;
    if (herr) return PD_ERR_TIMEOUT;
    if (loss) {
        double l = 0.0;
        for (float v : lp) l += v;
        *loss = (float)(l / (2.0 * (double)M));
    }
    return PD_OK;
}

}  // namespace

extern "C" {

pd_mlp* pd_mlp_create(int64_t max_rows, int* status) {
    auto fail = [&](int st) -> pd_mlp* {
        if (status) *status = st;
        return nullptr;
    };
    if (max_rows < 1) return fail(PD_ERR_ARG);
    pd_mlp* n = new pd_mlp();
    n->max_rows = max_rows;
    const int64_t R = (max_rows + kTileM - 1) / kTileM * kTileM;
    const int64_t splits = (R + kRowsPerSplit - 1) / kRowsPerSplit;
    n->part_floats = std::max<int64_t>(splits * kHid * kHid, (R / 128 + 1) * 128 + 1024);
    bool ok = true;
    auto al = [&](auto*& ptr, int64_t count) {
        if (ok) ok = cudaMalloc(&ptr, std::max<int64_t>(count, 1) * sizeof(*ptr)) == cudaSuccess;
        if (ok) cudaMemset(ptr, 0, std::max<int64_t>(count, 1) * sizeof(*ptr));
    };
    al(n->err, 1);
    al(n->p, kParams), al(n->g, kParams), al(n->m1, kParams), al(n->m2, kParams);
    al(n->W1, kHid * kInPad), al(n->W2, kHid * kHid), al(n->W3, kHid * kHid), al(n->W4, kOutPad * kHid);
    al(n->b1, kHid), al(n->b2, kHid), al(n->b3, kHid), al(n->b4, kOutPad);
    al(n->gW1, kHid * kInPad), al(n->gW2, kHid * kHid), al(n->gW3, kHid * kHid), al(n->gW4, kOutPad * kHid);
    al(n->gb1, kHid), al(n->gb2, kHid), al(n->gb3, kHid), al(n->gb4, kOutPad);
    al(n->Z1, R * kHid), al(n->Z2, R * kHid), al(n->Z3, R * kHid), al(n->Y, R * kOutPad);
    al(n->H1, R * kHid), al(n->H2, R * kHid), al(n->H3, R * kHid), al(n->dY, R * kOutPad);
    al(n->dZ, R * kHid), al(n->dZb, R * kHid);
    al(n->part, n->part_floats);
    if (!ok) {
        pd_mlp_destroy(n);
        return fail(PD_ERR_NOMEM);
    }
    if (status) *status = PD_OK;
    return n;
}

int pd_mlp_destroy(pd_mlp* n) {
    if (!n) return PD_ERR_ARG;
    void* ptrs[] = {n->err, n->p,   n->g,   n->m1,  n->m2,  n->W1,  n->W2,  n->W3, n->W4, n->b1,
                    n->b2,  n->b3,  n->b4,  n->gW1, n->gW2, n->gW3, n->gW4, n->gb1, n->gb2, n->gb3,
                    n->gb4, n->Z1,  n->Z2,  n->Z3,  n->Y,   n->H1,  n->H2,  n->H3, n->dY, n->dZ,
                    n->dZb, n->part};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete n;
    return PD_OK;
}

int pd_mlp_num_params(void) { return kParams; }

int pd_mlp_set_params(pd_mlp* n, const float* host, int64_t count) {
    if (!n || !host || count != kParams) return PD_ERR_ARG;
    if (cudaMemcpy(n->p, host, kParams * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return PD_ERR_CUDA;
    cudaMemset(n->m1, 0, kParams * sizeof(float));
    cudaMemset(n->m2, 0, kParams * sizeof(float));
    n->step = 0;
    k_pack<<<64, 256>>>(n->p, n->W1, n->W2, n->W3, n->W4, n->b1, n->b2, n->b3, n->b4);
    n->launches++;
    return cudaDeviceSynchronize() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

int pd_mlp_get_params(pd_mlp* n, float* host, int64_t count) {
    if (!n || !host || count != kParams) return PD_ERR_ARG;
    return cudaMemcpy(host, n->p, kParams * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? PD_OK
                                                                                                 : PD_ERR_CUDA;
}

int pd_mlp_forward_layers(pd_mlp* n, const void* dev_x, int64_t M, float* dev_y, void* stream) {
    if (!n || !dev_x || !dev_y || M < 1) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    for (int64_t r0 = 0; r0 < M; r0 += n->max_rows) {
        const int64_t m = std::min<int64_t>(n->max_rows, M - r0);
        int rc = forward(n, reinterpret_cast<const __nv_bfloat16*>(dev_x) + r0 * kInPad, m, s, false);
        if (rc) return rc;
        if (cudaMemcpy2DAsync(dev_y + r0 * kOut, kOut * sizeof(float), n->Y, kOutPad * sizeof(float),
                              kOut * sizeof(float), m, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return PD_ERR_CUDA;
    }
    int herr = 0;
    cudaMemcpyAsync(&herr, n->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return PD_ERR_CUDA;
    return herr ? PD_ERR_TIMEOUT : PD_OK;
}

namespace {
// cuTensorMapEncodeTiled, looked up through the runtime (no link against the
// driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

// A row-major [rows][cols] BF16 matrix read in boxes of 8 columns (16 bytes)
// by box_rows rows; rows past the end read as zero.
bool bf16_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * sizeof(__nv_bfloat16)};
    const cuuint32_t box[2] = {8, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

int pd_mlp_forward(pd_mlp* n, const void* dev_x, int64_t M, float* dev_y, void* stream) {
    if (!n || !dev_x || !dev_y || M < 1 || M > INT32_MAX - kTileM) return PD_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(dev_x) & 15) || (reinterpret_cast<uintptr_t>(dev_y) & 7)) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    // the fused pass: two CTAs per SM, persistent over the 128-row tiles
    static int configured = 0;
    if (!configured) {
        if (cudaFuncSetAttribute((const void*)k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kFusedSmem) != cudaSuccess)
            return PD_ERR_CUDA;
        configured = 1;
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t ntiles = (M + kTileM - 1) / kTileM;
    FusedArgs a;
    if (!bf16_map(&a.mX, dev_x, (uint64_t)M, kInPad, kTileM) || !bf16_map(&a.mW1, n->W1, kHid, kInPad, kHid) ||
        !bf16_map(&a.mW2, n->W2, kHid, kHid, kHid) || !bf16_map(&a.mW3, n->W3, kHid, kHid, kHid) ||
        !bf16_map(&a.mW4, n->W4, kOutPad, kHid, kOutPad)) {
        n->errmsg = "tensor map encoding failed";
        return PD_ERR_CUDA;
    }
    a.M = M;
    a.b1 = n->b1, a.b2 = n->b2, a.b3 = n->b3, a.b4 = n->b4;
    a.Y = dev_y, a.err = n->err, a.spin_limit = kSpinLimit;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ntiles, 2 * (int64_t)sms));
    k_mlp_fused<<<grid, kFusedThreads, kFusedSmem, s>>>(a);
    n->launches++;
    if (cudaGetLastError() != cudaSuccess) return PD_ERR_CUDA;
    int herr = 0;
    cudaMemcpyAsync(&herr, n->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return PD_ERR_CUDA;
    return herr ? PD_ERR_TIMEOUT : PD_OK;
}

int pd_mlp_grad(pd_mlp* n, const void* dev_x, const float* dev_t, int64_t M, float* host_grad, float* loss,
                void* stream) {
    if (!n || !dev_x || !dev_t || M < 1 || M > n->max_rows) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    int rc = grad(n, reinterpret_cast<const __nv_bfloat16*>(dev_x), dev_t, M, loss, s);
    if (rc) return rc;
    if (host_grad && cudaMemcpy(host_grad, n->g, kParams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
        return PD_ERR_CUDA;
    return PD_OK;
}

int pd_mlp_train_step(pd_mlp* n, const void* dev_x, const float* dev_t, int64_t M, float lr, float* loss,
                      void* stream) {
    if (!n || !dev_x || !dev_t || M < 1 || M > n->max_rows || !(lr > 0.0f)) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    int rc = grad(n, reinterpret_cast<const __nv_bfloat16*>(dev_x), dev_t, M, loss, s);
    if (rc) return rc;
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)n->step), c2 = 1.0f - std::pow(b2, (float)n->step);
    k_adam<<<64, 256, 0, s>>>(n->p, n->g, n->m1, n->m2, lr, b1, b2, 1e-8f, c1, c2);
    k_pack<<<64, 256, 0, s>>>(n->p, n->W1, n->W2, n->W3, n->W4, n->b1, n->b2, n->b3, n->b4);
    n->launches += 2;
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

// Warm-start features of the free nodes (BF16 [N_int][16], columns 8..15 zero):
//   0, 1  previous displacement / accumulated boundary displacement U
//   2     load increment / U
//   3     damage
//   4     1 within one horizon of a loaded edge
//   5, 6  the previous increment's departure from proportionality per unit
//         load (pd_warm_record), times kHistScale; 0 without a history
//   7     the damage the previous increment added; 0 without a history
int pd_warm_features(pd_ctx* c, double U, double delta, void* dev_x, void* stream) {
    if (!c || !dev_x || !(U > 0.0) || c->p.dim != 2) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    const int64_t n = c->p.N_int;
    const double hy = c->p.ny * c->p.dx / 2.0;
    k_features<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
        n, c->nf[PD_F_Y], c->nf[PD_F_UX], c->nf[PD_F_UY], c->nf[PD_F_DMG], c->warm_hist, 1.0 / U, delta / U,
        hy - c->p.delta, reinterpret_cast<__nv_bfloat16*>(dev_x));
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "pd_warm_features");
}

// Record the increment just solved as the history of the next prediction:
// dev_u_prev (2 N_int: x then y) and dev_dmg_prev (N_int) are the free nodes'
// displacement and damage before it, U_prev the accumulated boundary
// displacement before it.  U_prev <= 0 (no proportional reference yet)
// clears the history.
int pd_warm_record(pd_ctx* c, double U_prev, double delta, const double* dev_u_prev, const double* dev_dmg_prev,
                   void* stream) {
    if (!c || c->p.dim != 2) return PD_ERR_ARG;
    if (!(U_prev > 0.0)) {
        if (c->warm_hist) cudaFree(c->warm_hist);
        c->warm_hist = nullptr;
        return PD_OK;
    }
    if (!dev_u_prev || !dev_dmg_prev) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    const int64_t n = c->p.N_int;
    if (!c->warm_hist && cudaMalloc(&c->warm_hist, 3 * n * sizeof(double)) != cudaSuccess) {
        c->warm_hist = nullptr;
        return set_err(c, PD_ERR_NOMEM, "warm-start history");
    }
    int rc = pd_damage(c, stream);
    if (rc) return rc;
    k_warm_record<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
        n, c->nf[PD_F_UX], c->nf[PD_F_UY], c->nf[PD_F_DMG], dev_u_prev, dev_dmg_prev, delta / U_prev, 1.0 / U_prev,
        c->warm_hist);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "pd_warm_record");
}

// Candidate increments of the free nodes: features, forward pass, then
// du = u * delta / U + U * output (x components, then y components), and the
// skip term u * delta / U alone.
int pd_warm_predict(pd_ctx* c, pd_mlp* n, double U, double delta, int smooth_passes, double* dev_du, void* stream) {
    if (!c || !n || !dev_du || smooth_passes < 0) return PD_ERR_ARG;
    if (smooth_passes > 0 && (c->p.model != PD_MODEL_BOND || !c->family))
        return set_err(c, PD_ERR_STATE, "smoothing the correction needs a bond-based family");
    cudaStream_t s = st(stream);
    const int64_t ni = c->p.N_int;
    void* x = nullptr;
    float* y = nullptr;
    if (cudaMallocAsync(&x, ni * kInPad * 2, s) != cudaSuccess) return set_err(c, PD_ERR_NOMEM, "warm features");
    if (cudaMallocAsync(&y, ni * kOut * sizeof(float), s) != cudaSuccess) {
        cudaFreeAsync(x, s);
        return set_err(c, PD_ERR_NOMEM, "warm outputs");
    }
    int rc = pd_warm_features(c, U, delta, x, s);
    const int64_t l0 = n->launches;
    if (!rc) rc = pd_mlp_forward(n, x, ni, y, s);
    c->launches += n->launches - l0;  // the network's kernels count as the context's
    const unsigned g = (unsigned)std::min<int64_t>((ni + 255) / 256, 4096);
    if (!rc && smooth_passes == 0) {
        k_scale_out<<<g, 256, 0, s>>>(ni, y, U, delta / U, c->nf[PD_F_UX], c->nf[PD_F_UY], c->warm_hist, dev_du);
        c->launches++;
        rc = cuda_err(c, cudaGetLastError(), "pd_warm_predict");
    } else if (!rc) {
        // the correction, smoothed over the family, then the candidates
        double* cb = nullptr;
        if ((rc = make_ready(c, s)) == PD_OK &&
            (rc = cuda_err(c, cudaMallocAsync(&cb, 4 * ni * sizeof(double), s), "warm correction")) == PD_OK) {
            k_correction<<<g, 256, 0, s>>>(ni, y, U, cb);
            c->launches++;
            const Sell& S = c->sell;
            const int64_t ns = (ni + 31) / 32;
            const unsigned gs = (unsigned)std::min<int64_t>((ns * 32 + 255) / 256, 65535);
            for (int k = 0; k < smooth_passes; k++) {
                const double* in = cb + (k & 1) * 2 * ni;
                double* out = cb + ((k + 1) & 1) * 2 * ni;
                const int* cols = S.rec16 ? reinterpret_cast<const int*>(S.rec16) : reinterpret_cast<const int*>(S.rec);
                const int stride = S.rec16 ? (int)(sizeof(bt::Rec) / 4) : (int)(sizeof(BondRec) / 4);
                k_smooth<<<gs, 256, 0, s>>>(ns, ni, S.width, S.base, S.fbase, cols, stride, S.bits, in, out);
                c->launches++;
            }
            k_combine<<<g, 256, 0, s>>>(ni, cb + (smooth_passes & 1) * 2 * ni, U, delta / U, c->nf[PD_F_UX],
                                        c->nf[PD_F_UY], c->warm_hist, dev_du);
            c->launches++;
            rc = cuda_err(c, cudaGetLastError(), "pd_warm_predict");
            cudaFreeAsync(cb, s);
        }
    } else {
        set_err(c, rc, rc == PD_ERR_TIMEOUT ? "tensor-core wait gave up" : "MLP forward failed");
    }
    cudaFreeAsync(x, s);
    cudaFreeAsync(y, s);
    cudaStreamSynchronize(s);
    return rc;
}

// Self-test of the tensor-core product: D[M x N] = A[M x K] * B[N x K]^T for
// row-major BF16 A and B (FP32 D), through the same kernel and loader.
int pd_mlp_gemm(const void* dev_a, const void* dev_b, int64_t M, int64_t N, int64_t K, float* dev_d, int transpose_a,
                void* stream) {
    return pd_mlp_gemm_wait_check(dev_a, dev_b, M, N, K, dev_d, transpose_a, 0, 1, stream);
}

// The same product with the bounded mbarrier wait's iteration limit given
// (spin_limit <= 0: the library's limit) and, with issue = 0, no product and
// no commit issued: the wait then never completes, gives up after spin_limit
// iterations, and the call returns PD_ERR_TIMEOUT with the context usable.
int pd_mlp_gemm_wait_check(const void* dev_a, const void* dev_b, int64_t M, int64_t N, int64_t K, float* dev_d,
                           int transpose_a, long long spin_limit, int issue, void* stream) {
    if (!dev_a || !dev_b || !dev_d || M < 1 || N < 1 || K < 1 || (N != 16 && N % 128 != 0)) return PD_ERR_ARG;
    pd_mlp tmp;
    if (cudaMalloc(&tmp.err, sizeof(int)) != cudaSuccess) return PD_ERR_NOMEM;
    cudaMemset(tmp.err, 0, sizeof(int));
    cudaStream_t s = st(stream);
    const __nv_bfloat16* A = reinterpret_cast<const __nv_bfloat16*>(dev_a);
    // transpose_a: A is stored K x M (the loader gathers A(m, k) = A[k][m])
    GemmArgs a = transpose_a ? gemm(A, 1, M, reinterpret_cast<const __nv_bfloat16*>(dev_b), K, 1, M, N, K)
                             : gemm(A, K, 1, reinterpret_cast<const __nv_bfloat16*>(dev_b), K, 1, M, N, K);
    a.epi = E_F32, a.D = dev_d, a.ldd = N;
    a.spin_limit = spin_limit > 0 ? spin_limit : kSpinLimit;
    a.issue = issue ? 1 : 0;
    int rc = launch_gemm(&tmp, a, N == 16 ? 16 : 128, s);
    int herr = 0;
    cudaMemcpyAsync(&herr, tmp.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(tmp.err);
    tmp.err = nullptr;
    if (rc) return rc;
    if (e != cudaSuccess) return PD_ERR_CUDA;
    return herr ? PD_ERR_TIMEOUT : PD_OK;
}

}  // extern "C"
