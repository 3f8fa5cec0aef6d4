// Node-parallel passes: time integration, loading, damage, reductions.
//
//   launch_prologue     kernel_quick_load + kernel_integrate_2D_1/3D_1 +
//                       kernel_cy_integrate_1 of the first step of a run, and the
//                       current-position buffer P = x + u
//   launch_adr_update   kernel_integrate (Integrate.cu:54-106) with the damping
//                       coefficient read from device memory, the next step's
//                       boundary loading, and P
//   launch_verlet1/2    kernel_integrate_2D_1/_2, 3D_1/_2 (Integrate.cu:174-266)
//   launch_damage       kernel_cal_dmg_2D/3D (Base_Function.cu:149-217)
//   reduce_sum          sum (Reduce.cu:52-65) with a fixed summation order
//
// Every loop over rows < N_int stops at N_int; the reference's Verlet launches
// are sized for N_int but test i < N (Integrate.cu:178, :206), which only
// touches boundary rows whose force and acceleration are zero.
#include "pd_internal.cuh"

namespace pdg {
namespace {

constexpr int T = 256;

inline unsigned grid_for(pd_ctx* c, int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + T - 1) / T, (int64_t)c->num_sms * 16));
}

struct NodeArgs {
    KParams P;
    double *x, *y, *z, *ux, *uy, *uz, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz, *bx, *by, *bz;
    double *vhx, *vhy, *vhz, *fox, *foy, *foz;
    double2* pxy;  // current positions, x and y interleaved
    double* pz;
    const double* cn;
    CylDev* cyl;
    double adr_c0, adr_c1;  // 1.0 * dt / mass and 2.0 * dt / mass (host IEEE operations, the same bits)
};

NodeArgs node_args(pd_ctx* c) {
    NodeArgs a;
    a.P = kparams(c->p);
    double** f = c->nf;
    a.x = f[PD_F_X], a.y = f[PD_F_Y], a.z = f[PD_F_Z];
    a.ux = f[PD_F_UX], a.uy = f[PD_F_UY], a.uz = f[PD_F_UZ];
    a.vx = f[PD_F_VX], a.vy = f[PD_F_VY], a.vz = f[PD_F_VZ];
    a.ax = f[PD_F_AX], a.ay = f[PD_F_AY], a.az = f[PD_F_AZ];
    a.fx = f[PD_F_FX], a.fy = f[PD_F_FY], a.fz = f[PD_F_FZ];
    a.bx = f[PD_F_BX], a.by = f[PD_F_BY], a.bz = f[PD_F_BZ];
    a.vhx = f[PD_F_VHX], a.vhy = f[PD_F_VHY], a.vhz = f[PD_F_VHZ];
    a.fox = f[PD_F_FOX], a.foy = f[PD_F_FOY], a.foz = f[PD_F_FOZ];
    a.pxy = c->posxy[c->parity], a.pz = c->posz[c->parity];
    a.cn = c->cn;
    a.cyl = c->cyl;
    a.adr_c0 = 1.0 * c->p.dt / c->p.mass;
    a.adr_c1 = 2.0 * c->p.dt / c->p.mass;
    return a;
}

__global__ void k_refresh_pos(NodeArgs A) {
    const KParams& P = A.P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        A.pxy[i] = make_double2(A.x[i] + A.ux[i], A.y[i] + A.uy[i]);
        if (P.dim == 3) A.pz[i] = A.z[i] + A.uz[i];
    }
}

__device__ __forceinline__ void quick_load_row(const KParams& P, int64_t i, double load, double* uy) {
    const int64_t k = i - P.N_int;
    if (k < 3 * (int64_t)P.nx)
        uy[i] += load * P.dt;
    else if (k < 6 * (int64_t)P.nx)
        uy[i] -= load * P.dt;
}

// First step of a run: boundary loading, first Verlet half, impactor advance, P.
__global__ void k_prologue(NodeArgs A, double load, int first_verlet, int cyl_step) {
    const KParams& P = A.P;
    const double hdt = P.dt / 2.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= P.N_int) {
            if (load != 0.0) quick_load_row(P, i, load, A.uy);
        } else if (first_verlet) {
            A.vx[i] = fma(hdt, A.ax[i], A.vx[i]);
            A.vy[i] = fma(hdt, A.ay[i], A.vy[i]);
            if (P.dim == 3) A.vz[i] = fma(hdt, A.az[i], A.vz[i]);
            A.ux[i] = fma(A.vx[i], P.dt, A.ux[i]);
            A.uy[i] = fma(A.vy[i], P.dt, A.uy[i]);
            if (P.dim == 3) A.uz[i] = fma(A.vz[i], P.dt, A.uz[i]);
        }
        A.pxy[i] = make_double2(A.x[i] + A.ux[i], A.y[i] + A.uy[i]);
        if (P.dim == 3) A.pz[i] = A.z[i] + A.uz[i];
    }
    if (cyl_step && blockIdx.x == 0 && threadIdx.x == 0) {
        CylDev& cy = *A.cyl;
        for (int a = 0; a < 3; a++) {
            cy.vel[a] = fma(hdt, cy.acc[a], cy.vel[a]);
            cy.disp[a] = fma(cy.vel[a], P.dt, cy.disp[a]);
        }
    }
}

// kernel_integrate (Integrate.cu:54-106), same operand order.
__global__ void k_adr_update(NodeArgs A, int ct, int do_next, double load) {
    const KParams& P = A.P;
    // per step: 2 - cn dt, 2 + cn dt and its IEEE reciprocal, once per block
    // (per node the division goes through div_recip, bit for bit the
    // quotient); dt / mass comes from the host
    __shared__ double sk[3];
    if (threadIdx.x == 0) {
        const double cn = *A.cn;
        sk[0] = 2.0 - cn * P.dt;
        sk[1] = 2.0 + cn * P.dt;
        sk[2] = 1.0 / sk[1];
    }
    __syncthreads();
    const double num = sk[0], den = sk[1], rden = sk[2];
    const double c0 = A.adr_c0;  // ct == 0
    const double c1 = A.adr_c1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < P.N_int) {
            double* vh[3] = {A.vhx, A.vhy, A.vhz};
            double* v[3] = {A.vx, A.vy, A.vz};
            double* u[3] = {A.ux, A.uy, A.uz};
            double* fo[3] = {A.fox, A.foy, A.foz};
            const double* f[3] = {A.fx, A.fy, A.fz};
            const double* b[3] = {A.bx, A.by, A.bz};
            for (int a = 0; a < P.dim; a++) {
                const double vho = vh[a][i];
                const double fb = f[a][i] + b[a][i];
                double vhn;
                if (ct == 0)
                    vhn = c0 * fb / 2.0;
                else
                    vhn = div_recip(num * vho + c1 * fb, den, rden);
                v[a][i] = 0.5 * (vho + vhn);
                u[a][i] = fma(vhn, P.dt, u[a][i]);
                vh[a][i] = vhn;
                fo[a][i] = f[a][i];
            }
        } else if (do_next && load != 0.0) {
            quick_load_row(P, i, load, A.uy);
        }
        A.pxy[i] = make_double2(A.x[i] + A.ux[i], A.y[i] + A.uy[i]);
        if (P.dim == 3) A.pz[i] = A.z[i] + A.uz[i];
    }
}

__global__ void k_verlet1(NodeArgs A) {
    const KParams& P = A.P;
    const double hdt = P.dt / 2.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N_int;
         i += (int64_t)gridDim.x * blockDim.x) {
        A.vx[i] = fma(hdt, A.ax[i], A.vx[i]);
        A.vy[i] = fma(hdt, A.ay[i], A.vy[i]);
        if (P.dim == 3) A.vz[i] = fma(hdt, A.az[i], A.vz[i]);
        A.ux[i] = fma(A.vx[i], P.dt, A.ux[i]);
        A.uy[i] = fma(A.vy[i], P.dt, A.uy[i]);
        if (P.dim == 3) A.uz[i] = fma(A.vz[i], P.dt, A.uz[i]);
    }
}

__global__ void k_verlet2(NodeArgs A) {
    const KParams& P = A.P;
    const double hdt = P.dt / 2.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N_int;
         i += (int64_t)gridDim.x * blockDim.x) {
        A.ax[i] = div_recip(A.fx[i] + A.bx[i], P.dens, P.rdens);
        A.ay[i] = div_recip(A.fy[i] + A.by[i], P.dens, P.rdens);
        A.vx[i] = fma(hdt, A.ax[i], A.vx[i]);
        A.vy[i] = fma(hdt, A.ay[i], A.vy[i]);
        if (P.dim == 3) {
            A.az[i] = div_recip(A.fz[i] + A.bz[i], P.dens, P.rdens);
            A.vz[i] = fma(hdt, A.az[i], A.vz[i]);
        }
    }
}

__global__ void k_quick_load(NodeArgs A, double load) {
    const KParams& P = A.P;
    const int64_t n = 6 * (int64_t)P.nx;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = P.N_int + k;
        if (i < P.N) quick_load_row(P, i, load, A.uy);
    }
}

__global__ void k_load_tensile(NodeArgs A) {
    const KParams& P = A.P;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < P.ny) {
        A.bx[i * P.nx] = -0.001 * P.emod / P.dx;
        A.bx[i * P.nx + P.nx - 1] = 0.001 * P.emod / P.dx;
    }
}

// kernel_cal_dmg_2D/3D (Base_Function.cu:149-217): dmg = 1 - (sum of vol fac
// over intact bonds) / (sum of vol fac over all bonds), vol cancelled.  One
// thread per row summing its bonds in order: the reference's warp per node
// with a shuffle tree spends about 25 FP64 warp instructions per row, most of
// them on lanes without a bond, and on this GPU's FP64 pipe that took 2.2 ms
// per call on the 1.6M-node plate; here it is two FP64 additions per bond.
// The sums differ from the reference's order by rounding only (relative
// 1e-16).  The intact flag of bond q comes from the CSR flags or (BITS)
// straight from the step loop's SELL words: slot k of row r is bond
// rowptr[r] + k, and word fbase[r / 32] + k holds the flags of slot k of the
// slice's 32 rows (the same word for the 32 lanes of a warp), so no
// conversion pass is needed.  Both forms give the same bits.
template <bool BITS>
__global__ void k_damage(KParams P, const int64_t* __restrict__ rowptr, const int* __restrict__ fail,
                         const int64_t* __restrict__ fbase, const uint32_t* __restrict__ bits,
                         const double* __restrict__ fac, double* __restrict__ dmg) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P.N_int) return;
    const int64_t q0 = rowptr[i], n = rowptr[i + 1] - q0;
    const uint32_t* wb = BITS ? bits + fbase[i >> 5] : nullptr;
    double d1 = 0.0, d2 = 0.0;
    for (int64_t k = 0; k < n; k++) {
        const double f = fac[q0 + k];
        const bool alive = BITS ? ((wb[k] >> (i & 31)) & 1u) != 0u : fail[q0 + k] != 0;
        d2 += f;
        if (alive) d1 += f;
    }
    dmg[i] = 1.0 - d1 / d2;
}

// Deterministic two-pass sum: block partials in block order, then one block.
__global__ void k_sum_partials(const double* __restrict__ x, int64_t n, double* __restrict__ part) {
    __shared__ double sm[T / 32];
    double v = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v += x[i];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < T / 32; k++) r += sm[k];
        part[blockIdx.x] = r;
    }
}

__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double sm[T / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < T / 32; k++) r += sm[k];
        *out = r;
    }
}

// Squared residual |F + b|^2 of the free nodes, block partials in a fixed order.
__global__ void k_residual_partials(NodeArgs A, double* __restrict__ part) {
    __shared__ double sm[T / 32];
    const KParams& P = A.P;
    double v = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N_int;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double rx = A.fx[i] + A.bx[i], ry = A.fy[i] + A.by[i];
        v += rx * rx + ry * ry;
        if (P.dim == 3) {
            const double rz = A.fz[i] + A.bz[i];
            v += rz * rz;
        }
    }
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < T / 32; k++) r += sm[k];
        part[blockIdx.x] = r;
    }
}

__global__ void k_finite(NodeArgs A, int* bad) {
    const KParams& P = A.P;
    int b = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        b |= !isfinite(A.ux[i]) | !isfinite(A.uy[i]) | !isfinite(A.fx[i]) | !isfinite(A.fy[i]);
        if (P.dim == 3) b |= !isfinite(A.uz[i]) | !isfinite(A.fz[i]);
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Dependent FMA chains, 8 per thread: the FP64 issue rate of this GPU.
__global__ void k_fp64_probe(double* out, double a, double b, int iters) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// div_recip against the IEEE division on the same operands: counts the
// pairs whose bit patterns differ (y formed here as the update kernels form
// it, 1.0 / d).
__global__ void k_div_check(const double* __restrict__ n, const double* __restrict__ d, int64_t count,
                            unsigned long long* __restrict__ mismatches) {
    unsigned long long bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const double ni = n[i], di = d[i];
        const double q = div_recip(ni, di, 1.0 / di);
        const double r = ni / di;
        // bit patterns equal, or both NaN (a NaN's payload is not compared)
        if (__double_as_longlong(q) != __double_as_longlong(r) && !(q != q && r != r)) bad++;
    }
    for (int off = 16; off > 0; off >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, off);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatches, bad);
}

}  // namespace

int div_check(const double* n, const double* d, int64_t count, unsigned long long* mismatches, cudaStream_t s) {
    if (!n || !d || !mismatches || count < 0) return PD_ERR_ARG;
    cudaMemsetAsync(mismatches, 0, sizeof(unsigned long long), s);
    if (count > 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int64_t want = (count + T - 1) / T;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
        k_div_check<<<grid, T, 0, s>>>(n, d, count, mismatches);
    }
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

int fp64_probe(double* gfma_per_s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, iters = 4096;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * T * 8) != cudaSuccess) return PD_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(a);
        k_fp64_probe<<<blocks, T>>>(out, 0.999999, 1e-7, iters);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        best = std::min(best, ms);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *gfma_per_s = (double)blocks * T * iters * 8 / (best * 1e-3) / 1e9;
    return cudaGetLastError() == cudaSuccess ? PD_OK : PD_ERR_CUDA;
}

int refresh_pos(pd_ctx* c, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_refresh_pos<<<grid_for(c, A.P.N), T, 0, s>>>(A);
    c->launches++;
    c->pos_valid = true;
    return cuda_err(c, cudaGetLastError(), "refresh_pos");
}

int launch_prologue(pd_ctx* c, double load, int first_verlet, int cyl_step, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_prologue<<<grid_for(c, A.P.N), T, 0, s>>>(A, load, first_verlet, cyl_step);
    c->launches++;
    c->pos_valid = true;
    return cuda_err(c, cudaGetLastError(), "prologue");
}

int launch_adr_update(pd_ctx* c, int ct, int do_next, double load, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_adr_update<<<grid_for(c, A.P.N), T, 0, s>>>(A, ct, do_next, load);
    c->launches++;
    c->pos_valid = true;
    return cuda_err(c, cudaGetLastError(), "adr_update");
}

int launch_verlet1(pd_ctx* c, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_verlet1<<<grid_for(c, A.P.N_int), T, 0, s>>>(A);
    c->launches++;
    c->pos_valid = false;
    return cuda_err(c, cudaGetLastError(), "verlet1");
}

int launch_verlet2(pd_ctx* c, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_verlet2<<<grid_for(c, A.P.N_int), T, 0, s>>>(A);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "verlet2");
}

int launch_quick_load(pd_ctx* c, double load, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_quick_load<<<grid_for(c, 6 * (int64_t)A.P.nx), T, 0, s>>>(A, load);
    c->launches++;
    c->pos_valid = false;
    return cuda_err(c, cudaGetLastError(), "quick_load");
}

int launch_load_tensile(pd_ctx* c, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_load_tensile<<<grid_for(c, A.P.ny), T, 0, s>>>(A);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "load_plate_tensile");
}

int launch_damage(pd_ctx* c, cudaStream_t s) {
    const KParams P = kparams(c->p);
    const Sell& S = c->sell;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (P.N_int + T - 1) / T);
    if (c->bits_current && S.bits) {
        // the step loop's flags as they stand (no conversion to the CSR flags)
        k_damage<true><<<grid, T, 0, s>>>(P, c->rowptr, nullptr, S.fbase, S.bits, c->fac, c->nf[PD_F_DMG]);
    } else {
        int rc = sync_fail_to_csr(c, s);
        if (rc) return rc;
        k_damage<false><<<grid, T, 0, s>>>(P, c->rowptr, c->fail, nullptr, nullptr, c->fac, c->nf[PD_F_DMG]);
    }
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "damage");
}

int reduce_sum(pd_ctx* c, const double* x, int64_t n, double* out_dev, cudaStream_t s) {
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + T - 1) / T, 1024));
    k_sum_partials<<<g, T, 0, s>>>(x, n, c->partials);
    k_sum_final<<<1, T, 0, s>>>(c->partials, (int)g, out_dev);
    c->launches += 2;
    return cuda_err(c, cudaGetLastError(), "reduce_sum");
}

// u += du on the free nodes (du: x components then y components, N_int each).
__global__ void k_add_increment(NodeArgs A, const double* __restrict__ du) {
    const KParams& P = A.P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N_int;
         i += (int64_t)gridDim.x * blockDim.x) {
        A.ux[i] += du[i];
        A.uy[i] += du[P.N_int + i];
    }
}

int add_increment(pd_ctx* c, const double* du, cudaStream_t s) {
    NodeArgs A = node_args(c);
    k_add_increment<<<grid_for(c, A.P.N_int), T, 0, s>>>(A, du);
    c->launches++;
    c->pos_valid = false;
    return cuda_err(c, cudaGetLastError(), "add_increment");
}

int residual_sq(pd_ctx* c, double* out_dev, cudaStream_t s) {
    NodeArgs A = node_args(c);
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((A.P.N_int + T - 1) / T, 1024));
    k_residual_partials<<<g, T, 0, s>>>(A, c->partials);
    k_sum_final<<<1, T, 0, s>>>(c->partials, (int)g, out_dev);
    c->launches += 2;
    return cuda_err(c, cudaGetLastError(), "residual");
}

int check_finite(pd_ctx* c, cudaStream_t s, int* bad_host) {
    int* d = reinterpret_cast<int*>(c->ticket) + 1;  // spare word after the ticket
    cudaMemsetAsync(d, 0, sizeof(int), s);
    NodeArgs A = node_args(c);
    k_finite<<<grid_for(c, A.P.N), T, 0, s>>>(A, d);
    c->launches++;
    cudaError_t e = cudaMemcpyAsync(bad_host, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_err(c, e, "check_finite");
}

}  // namespace pdg
