// Bond-family build: replaces find_neighbor_gpu / kernel_find_neighbor_2D/3D
// (Neighbor.cu:7-40, :82-90), an all-pairs O(N^2) search that appends both
// directions of every pair to a padded ELL list through atomics (row order
// nondeterministic) and does not guard against rows longer than MN.
//
// Here: nodes are binned into a uniform grid of cells no smaller than the
// horizon, the cells are numbered in Morton order (so a cell's neighbours sit
// close in the sorted node list), a count pass sizes every row, a scan turns
// the counts into CSR offsets, a fill pass writes the rows and a per-row sort
// puts them in ascending order — the row order of the reference's CPU search
// (Neighbor.cu:42-80).  The family predicate is the reference's expression,
// |xj - xi|^2 < delta^2, and this file is compiled without FMA contraction, so
// the membership test rounds exactly like the reference's host code.
#include "pd_internal.cuh"

namespace pdg {
namespace {

__global__ void k_bbox(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                       int64_t n, int dim, double* __restrict__ part) {
    __shared__ double sm[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double c[3] = {x[i], y[i], dim == 3 ? z[i] : 0.0};
        for (int a = 0; a < 3; a++) {
            lo[a] = fmin(lo[a], c[a]);
            hi[a] = fmax(hi[a], c[a]);
        }
    }
    for (int a = 0; a < 3; a++) {
        sm[a][threadIdx.x] = lo[a];
        sm[3 + a][threadIdx.x] = hi[a];
    }
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int a = 0; a < 3; a++) {
                sm[a][threadIdx.x] = fmin(sm[a][threadIdx.x], sm[a][threadIdx.x + off]);
                sm[3 + a][threadIdx.x] = fmax(sm[3 + a][threadIdx.x], sm[3 + a][threadIdx.x + off]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = sm[threadIdx.x][0];
}

struct Grid {
    double lo[3];
    double inv_h;
    int64_t nc[3];
    int morton;  // 1: keys are Morton codes of the cell coordinates
    int bits;    // bits per axis of the Morton code
};

__device__ __forceinline__ uint64_t spread2(uint64_t v) {
    v &= 0xffffffffull;
    v = (v | (v << 16)) & 0x0000ffff0000ffffull;
    v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
    v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}

__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__device__ __forceinline__ int64_t cell_key(const Grid& g, int dim, int64_t cx, int64_t cy, int64_t cz) {
    if (g.morton) {
        if (dim == 2) return (int64_t)(spread2((uint64_t)cx) | (spread2((uint64_t)cy) << 1));
        return (int64_t)(spread3((uint64_t)cx) | (spread3((uint64_t)cy) << 1) | (spread3((uint64_t)cz) << 2));
    }
    return (cz * g.nc[1] + cy) * g.nc[0] + cx;
}

__device__ __forceinline__ void cell_of(const Grid& g, int dim, double x, double y, double z, int64_t* c) {
    const double v[3] = {x, y, z};
    for (int a = 0; a < 3; a++) {
        int64_t k = 0;
        if (a < dim) {
            k = (int64_t)floor((v[a] - g.lo[a]) * g.inv_h);
            if (k < 0) k = 0;
            if (k >= g.nc[a]) k = g.nc[a] - 1;
        }
        c[a] = k;
    }
}

// Grouped 2-D builds (a batch of specimens sharing one coordinate frame):
// the third cell axis is the node's group, so a node only visits cells of its
// own group; padding nodes (group -1) sit in a layer of their own past the
// last group and have no family.
__device__ __forceinline__ void group_cell(const Grid& g, const int* __restrict__ grp, int64_t i, int64_t* c) {
    if (grp) c[2] = grp[i] >= 0 ? grp[i] : g.nc[2] - 1;
}

__global__ void k_cell_count(const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z, const int* __restrict__ grp, int64_t n, int dim, Grid g,
                             int64_t* __restrict__ key, int* __restrict__ count) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t c[3];
    cell_of(g, dim, x[i], y[i], dim == 3 ? z[i] : 0.0, c);
    group_cell(g, grp, i, c);
    const int64_t k = cell_key(g, dim, c[0], c[1], c[2]);
    key[i] = k;
    atomicAdd(&count[k], 1);
}

__global__ void k_cell_scatter(int64_t n, const int64_t* __restrict__ key, const int64_t* __restrict__ start,
                               int* __restrict__ cursor, int* __restrict__ order) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t k = key[i];
    order[start[k] + atomicAdd(&cursor[k], 1)] = (int)i;
}

// The family predicate of Neighbor.cu:16 / :33 / :51 / :72.  With contraction
// disabled for this file the expression rounds exactly like the reference's
// host build: three products, two sums, one compare.
__device__ __forceinline__ bool in_family(const double* __restrict__ x, const double* __restrict__ y,
                                          const double* __restrict__ z, int dim, int64_t i, int64_t j,
                                          double delta2) {
    const double dx = x[j] - x[i];
    const double dy = y[j] - y[i];
    if (dim == 2) return dx * dx + dy * dy < delta2;
    const double dz = z[j] - z[i];
    return dx * dx + dy * dy + dz * dz < delta2;
}

// One thread per node; FILL=false counts the row, FILL=true writes it.
template <bool FILL>
__global__ void k_family(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                         const int* __restrict__ grp, int64_t n, int dim, Grid g, double delta2,
                         const int64_t* __restrict__ start, const int* __restrict__ count,
                         const int* __restrict__ order, int* __restrict__ NN, const int64_t* __restrict__ rowptr,
                         int* __restrict__ NL) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (grp && grp[i] < 0) {
        if (!FILL) NN[i] = 0;
        return;
    }
    int64_t c[3];
    cell_of(g, dim, x[i], y[i], dim == 3 ? z[i] : 0.0, c);
    group_cell(g, grp, i, c);
    int cnt = 0;
    int64_t out = FILL ? rowptr[i] : 0;
    const int64_t z0 = dim == 3 ? -1 : 0, z1 = dim == 3 ? 1 : 0;
    for (int64_t dz = z0; dz <= z1; dz++)
        for (int64_t dy = -1; dy <= 1; dy++)
            for (int64_t dx = -1; dx <= 1; dx++) {
                const int64_t a0 = c[0] + dx, a1 = c[1] + dy, a2 = c[2] + dz;
                if (a0 < 0 || a1 < 0 || a2 < 0 || a0 >= g.nc[0] || a1 >= g.nc[1] || a2 >= g.nc[2]) continue;
                const int64_t k = cell_key(g, dim, a0, a1, a2);
                const int64_t b = start[k], e = b + count[k];
                for (int64_t t = b; t < e; t++) {
                    const int j = order[t];
                    if (j == i || !in_family(x, y, z, dim, i, j, delta2)) continue;
                    if (FILL) NL[out++] = j;
                    cnt++;
                }
            }
    if (!FILL) NN[i] = cnt;
}

// Ascending order within each row (insertion sort: rows hold at most a few
// hundred entries and this runs once per setup).
__global__ void k_row_sort(int64_t n, const int64_t* __restrict__ rowptr, int* __restrict__ NL) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int* r = NL + rowptr[i];
    const int len = (int)(rowptr[i + 1] - rowptr[i]);
    for (int a = 1; a < len; a++) {
        const int v = r[a];
        int b = a - 1;
        while (b >= 0 && r[b] > v) {
            r[b + 1] = r[b];
            b--;
        }
        r[b + 1] = v;
    }
}

__global__ void k_fill_bonds(int64_t B, double* scr, double* e, int* fail) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < B; q += (int64_t)gridDim.x * blockDim.x) {
        scr[q] = 1.0;
        e[q] = 0.0;
        fail[q] = 1;  // kernel_initial_fail (Initial.cu:6-14)
    }
}

__global__ void k_max_int(const int* __restrict__ v, int64_t n, int* out) {
    int m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, v[i]);
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

template <typename T>
void free_ptr(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

namespace {

// ---- exclusive scan of int32 counts into int64 offsets ----------------------
//
// Three passes over tiles of kScanTile counts: the sum of every tile, an
// exclusive scan of the tile sums in one block, then every tile rescanned
// from its offset.  Integer sums: exact and independent of the launch.
constexpr int kScanThreads = 512, kScanItems = 8, kScanTile = kScanThreads * kScanItems;
constexpr int kScanWarps = kScanThreads / 32;

// Inclusive scan of one value per thread over the block (every thread
// calls it); total receives the block's sum.
__device__ int64_t block_inclusive_scan(int64_t v, int64_t* sm, int64_t& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += t;
    }
    if (lane == 31) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        int64_t q = lane < kScanWarps ? sm[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, q, off);
            if (lane >= off) q += t;
        }
        if (lane < kScanWarps) sm[lane] = q;
    }
    __syncthreads();
    total = sm[kScanWarps - 1];
    const int64_t r = v + (w > 0 ? sm[w - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(const int* __restrict__ in, int64_t n,
                                                                 int64_t* __restrict__ tile_sum) {
    __shared__ int64_t sm[kScanWarps];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v = 0;
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) v += in[base + k];
    int64_t total;
    block_inclusive_scan(v, sm, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// One block: the tile sums become their exclusive prefix sums, in place.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_offsets(int64_t* __restrict__ tile_sum, int64_t ntiles) {
    __shared__ int64_t sm[kScanWarps];
    int64_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += kScanThreads) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < ntiles ? tile_sum[i] : 0;
        int64_t total;
        const int64_t inc = block_inclusive_scan(v, sm, total);
        if (i < ntiles) tile_sum[i] = carry + inc - v;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ in, int64_t n,
                                                             const int64_t* __restrict__ tile_off,
                                                             int64_t* __restrict__ out) {
    __shared__ int64_t sm[kScanWarps];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int c[kScanItems];
    int64_t v = 0;
    for (int k = 0; k < kScanItems; k++) {
        c[k] = base + k < n ? in[base + k] : 0;
        v += c[k];
    }
    int64_t total;
    const int64_t inc = block_inclusive_scan(v, sm, total);
    int64_t run = tile_off[blockIdx.x] + inc - v;
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) {
            out[base + k] = run;
            run += c[k];
        }
}

}  // namespace

// Exclusive scan of n int32 counts into int64 offsets out[0 .. n) (the
// callers form out[n] themselves).
static int scan_counts(pd_ctx* c, const int* in, int64_t* out, int64_t n, cudaStream_t s) {
    if (n <= 0) return PD_OK;
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    int64_t* tiles = nullptr;
    cudaError_t e = cudaMallocAsync(&tiles, ntiles * sizeof(int64_t), s);
    if (e != cudaSuccess) return cuda_err(c, e, "scan alloc");
    k_scan_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tiles);
    k_scan_tile_offsets<<<1, kScanThreads, 0, s>>>(tiles, ntiles);
    k_scan_apply<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, tiles, out);
    cudaFreeAsync(tiles, s);
    c->launches += 3;
    return cuda_err(c, cudaGetLastError(), "scan");
}

int build_family(pd_ctx* c, cudaStream_t s) {
    const pd_params& p = c->p;
    const int64_t N = p.N;
    const int dim = p.dim;
    double* X = c->nf[PD_F_X];
    double* Y = c->nf[PD_F_Y];
    double* Z = c->nf[PD_F_Z];
    const int* grp = c->batch.node_group;
    if (grp && dim != 2) return set_err(c, PD_ERR_ARG, "grouped family builds are 2-D");
    // until this build succeeds the context holds no valid family: every
    // failure below leaves it refused by the stages that need one
    c->family = false;
    c->volcorr = c->surfcorr = c->weights = false;
    c->prepared = false;
    cudaError_t e;

    // bounding box
    const int nb = (int)std::min<int64_t>(1024, (N + 255) / 256);
    double* part = c->partials;
    k_bbox<<<nb, 256, 0, s>>>(X, Y, Z, N, dim, part);
    c->launches++;
    std::vector<double> hp((size_t)nb * 6);
    if ((e = cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_err(c, e, "bbox copy");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_err(c, e, "bbox");
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = 0; b < nb; b++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], hp[b * 6 + a]);
            hi[a] = std::max(hi[a], hp[b * 6 + 3 + a]);
        }
    Grid g{};
    const double h = p.delta * 1.0001;  // cell edge no smaller than the horizon
    g.inv_h = 1.0 / h;
    int64_t ncell = 1;
    int maxbits = 0;
    for (int a = 0; a < 3; a++) {
        g.lo[a] = a < dim ? lo[a] : 0.0;
        g.nc[a] = a < dim ? (int64_t)std::floor((hi[a] - lo[a]) / h) + 1 : 1;
        if (a == 2 && grp) g.nc[2] = c->batch.count + 1;  // groups, then the padding layer
        ncell *= g.nc[a];
        int b = 0;
        while ((int64_t(1) << b) < g.nc[a]) b++;
        maxbits = std::max(maxbits, b);
    }
    if (ncell > (int64_t(1) << 31)) return set_err(c, PD_ERR_ARG, "domain too large for the cell grid");
    // Morton keys when their padded range stays small, row-major otherwise
    const int64_t mrange = int64_t(1) << (maxbits * dim);
    g.morton = (!grp && maxbits * dim <= 30 && mrange <= 8 * ncell + 1024) ? 1 : 0;
    g.bits = maxbits;
    const int64_t nkeys = g.morton ? mrange : ncell;

    int* count = nullptr;
    int* cursor = nullptr;
    int64_t* start = nullptr;
    int64_t* key = nullptr;
    int* order = nullptr;
    int* dmax = nullptr;
    auto cleanup = [&]() {
        cudaFreeAsync(count, s);
        cudaFreeAsync(cursor, s);
        cudaFreeAsync(start, s);
        cudaFreeAsync(key, s);
        cudaFreeAsync(order, s);
        cudaFreeAsync(dmax, s);
    };
    if ((e = cudaMallocAsync(&count, (nkeys + 1) * sizeof(int), s)) != cudaSuccess ||
        (e = cudaMallocAsync(&cursor, nkeys * sizeof(int), s)) != cudaSuccess ||
        (e = cudaMallocAsync(&start, (nkeys + 1) * sizeof(int64_t), s)) != cudaSuccess ||
        (e = cudaMallocAsync(&key, N * sizeof(int64_t), s)) != cudaSuccess ||
        (e = cudaMallocAsync(&order, N * sizeof(int), s)) != cudaSuccess ||
        (e = cudaMallocAsync(&dmax, sizeof(int), s)) != cudaSuccess) {
        cleanup();
        return set_err(c, PD_ERR_NOMEM, "cell list allocation failed");
    }
    cudaMemsetAsync(count, 0, (nkeys + 1) * sizeof(int), s);
    cudaMemsetAsync(cursor, 0, nkeys * sizeof(int), s);
    cudaMemsetAsync(dmax, 0, sizeof(int), s);
    const int T = 256;
    const unsigned gN = (unsigned)((N + T - 1) / T);
    k_cell_count<<<gN, T, 0, s>>>(X, Y, Z, grp, N, dim, g, key, count);
    c->launches++;
    int rc = scan_counts(c, count, start, nkeys, s);
    if (rc) {
        cleanup();
        return rc;
    }
    k_cell_scatter<<<gN, T, 0, s>>>(N, key, start, cursor, order);
    c->launches++;

    const double delta2 = p.delta * p.delta;
    k_family<false><<<gN, T, 0, s>>>(X, Y, Z, grp, N, dim, g, delta2, start, count, order, c->NN, nullptr, nullptr);
    c->launches++;
    rc = scan_counts(c, c->NN, c->rowptr, N, s);
    if (rc) {
        cleanup();
        return rc;
    }
    k_max_int<<<std::min<int64_t>(1024, (N + T - 1) / T), T, 0, s>>>(c->NN, N, dmax);
    c->launches++;
    int64_t last_off = 0;
    int last_cnt = 0, maxnn = 0;
    cudaMemcpyAsync(&last_off, c->rowptr + (N - 1), sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&last_cnt, c->NN + (N - 1), sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&maxnn, dmax, sizeof(int), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
        cleanup();
        return cuda_err(c, e, "family count");
    }
    const int64_t B = last_off + last_cnt;
    cudaMemcpyAsync(c->rowptr + N, &B, sizeof(int64_t), cudaMemcpyHostToDevice, s);

    // (re)allocate the bond arrays
    free_ptr(c->NL);
    free_ptr(c->idist);
    free_ptr(c->fac);
    free_ptr(c->scr);
    free_ptr(c->w);
    free_ptr(c->e);
    free_ptr(c->fail);
    const size_t nb8 = (size_t)std::max<int64_t>(B, 1) * 8, nb4 = (size_t)std::max<int64_t>(B, 1) * 4;
    if (cudaMalloc(&c->NL, nb4) || cudaMalloc(&c->idist, nb8) || cudaMalloc(&c->fac, nb8) ||
        cudaMalloc(&c->scr, nb8) || cudaMalloc(&c->w, nb8) || cudaMalloc(&c->e, nb8) || cudaMalloc(&c->fail, nb4)) {
        cleanup();
        return set_err(c, PD_ERR_NOMEM, "bond array allocation failed");
    }
    c->B = B;
    k_family<true><<<gN, T, 0, s>>>(X, Y, Z, grp, N, dim, g, delta2, start, count, order, nullptr, c->rowptr, c->NL);
    k_row_sort<<<gN, T, 0, s>>>(N, c->rowptr, c->NL);
    cudaMemsetAsync(c->idist, 0, nb8, s);
    cudaMemsetAsync(c->fac, 0, nb8, s);
    cudaMemsetAsync(c->w, 0, nb8, s);
    k_fill_bonds<<<(unsigned)std::min<int64_t>(152 * 32, (B + T - 1) / T + 1), T, 0, s>>>(B, c->scr, c->e, c->fail);
    c->launches += 3;
    cleanup();
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(c, e, "family kernels");
    c->bits_current = false;
    c->csr_fail_current = true;
    if (p.MN > 0 && maxnn > p.MN) {
        // the arrays hold the oversized family, but it is not the reference's
        // (whose rows stop at MN): the context stays without a family
        return set_err(c, PD_ERR_FAMILY,
                       "a node has " + std::to_string(maxnn) + " neighbours, more than MN=" + std::to_string(p.MN));
    }
    c->family = true;
    return PD_OK;
}

}  // namespace pdg
