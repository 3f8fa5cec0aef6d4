// Batches of specimens: many 2-D bond-based plates of uneven size, each with
// its own modulus, critical stretch, pre-crack and loading rate, solved
// together by ADR.  The reference has no batching; each specimen follows the
// quasi-static pipeline of solve_plate_tensile (Solve_Plate_Tensile.cu:94-131:
// family, surface correction, force + kernel_cnn/cal_cn + kernel_integrate per
// step) with the moving boundary rows of kernel_quick_load
// (Solve_Plate_Crack_Grow.cu:8-19).
//
// Packing.  Every specimen keeps its own coordinate frame (centred on its
// plate, exactly as a standalone run lays it out), so positions, stretches and
// forces round exactly as they would alone.  Specimen k's interior rows come
// first, padded to a whole number of 32-row slices with padding rows that
// have no bonds, so a SELL slice never mixes specimens; all boundary rows (3
// rows up, 3 rows down per specimen) follow all interiors.  The family build
// keys its cell grid by specimen (a node only meets nodes of its own
// specimen), and whatever a specimen does not share lives in per-node arrays
// (bc, surface energy density, s0, ADR mass, boundary speed factor) or in
// per-slice / per-specimen arrays (damping sums, damping coefficient).  One
// launch per phase covers all specimens:
//   k_bond_force<2, EPI_ADR>  forces + damping sums per slice
//   k_batch_cn                damping coefficient per specimen (cal_cn)
//   k_batch_update            ADR update with the specimen's coefficient and
//                             each node's mass, next step's boundary motion,
//                             current positions
// and the step loop is captured in CUDA graphs like the single-specimen one.
#include <algorithm>
#include <cmath>

#include "pd_internal.cuh"

namespace pdg {
namespace {

constexpr int T = 256;

// cal_cn (Integrate.cu:108-129) per specimen: one warp sums the specimen's
// per-slice damping sums in a fixed order.  It also forms the update's
// 2 - cn dt and 2 + cn dt (kernel_integrate's expressions) and the IEEE
// reciprocal of the latter, once per specimen.
__global__ void k_batch_cn(int count, const int64_t* __restrict__ inst_slices, const double* __restrict__ part,
                           double dt, double* __restrict__ inst_cn, double* __restrict__ inst_nd) {
    const int k = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= count) return;
    double a = 0.0, b = 0.0;
    for (int64_t s = inst_slices[k] + lane; s < inst_slices[k + 1]; s += 32) {
        a += part[2 * s];
        b += part[2 * s + 1];
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if (lane == 0) {
        double cn = 0.0;
        if (b != 0.0) {
            if (a / b > 0.0) cn = 2.0 * sqrt(a / b);
        }
        if (cn > 2.0) cn = 1.9;
        inst_cn[k] = cn;
        const double num = 2.0 - cn * dt, den = 2.0 + cn * dt;
        inst_nd[3 * k] = num;
        inst_nd[3 * k + 1] = den;
        inst_nd[3 * k + 2] = 1.0 / den;
    }
}

struct BatchArgs {
    KParams P;
    double *x, *y, *ux, *uy, *vx, *vy, *fx, *fy, *bx, *by, *vhx, *vhy, *fox, *foy;
    double2* pxy;  // current positions, x and y interleaved
    const double* mass;
    const double* c1;  // 2 dt / mass per node
    const double* sign;
    const int* slice_inst;
    const double* inst_cn;
    const double* inst_nd;  // per specimen: 2 - cn dt, 2 + cn dt, 1 / (2 + cn dt)
};

// kernel_quick_load with the row's signed speed factor: +1 / -1 times the
// specimen's load scale (for a scale of one, (s * load) * dt rounds exactly
// like the reference's +- load * dt).
__device__ __forceinline__ void move_boundary(const BatchArgs& A, int64_t i, double load) {
    const double sg = A.sign[i];
    if (sg != 0.0) A.uy[i] += (sg * load) * A.P.dt;
}

// kernel_integrate (Integrate.cu:54-106) with each node's mass and its
// specimen's damping coefficient, same operand order.
__global__ void k_batch_update(BatchArgs A, int ct, int do_next, double load) {
    const KParams& P = A.P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < P.N_int) {
            const int k = A.slice_inst[i >> 5];
            // 2 dt / mass comes precomputed (the same IEEE operations, on the
            // host): two FP64 divides per node fewer on a pipe this GPU runs
            // at 1/64 rate; dt / mass is formed only for the first step.  The
            // division by 2 + cn dt goes through the specimen's reciprocal
            // (div_recip: bit for bit the quotient).  A padding row (k < 0)
            // takes cn = 0, the values k_batch_cn forms for cn = 0.
            const double c1 = A.c1[i];
            const double c0 = ct == 0 ? 1.0 * P.dt / A.mass[i] : 0.0;
            const double num = k >= 0 ? A.inst_nd[3 * k] : 2.0, den = k >= 0 ? A.inst_nd[3 * k + 1] : 2.0;
            const double rden = k >= 0 ? A.inst_nd[3 * k + 2] : 0.5;
            double* vh[2] = {A.vhx, A.vhy};
            double* v[2] = {A.vx, A.vy};
            double* u[2] = {A.ux, A.uy};
            double* fo[2] = {A.fox, A.foy};
            const double* f[2] = {A.fx, A.fy};
            const double* b[2] = {A.bx, A.by};
            for (int a = 0; a < 2; a++) {
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
            move_boundary(A, i, load);
        }
        A.pxy[i] = make_double2(A.x[i] + A.ux[i], A.y[i] + A.uy[i]);
    }
}

// First step of a run: boundary motion and current positions.
__global__ void k_batch_prologue(BatchArgs A, double load) {
    const KParams& P = A.P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.N; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= P.N_int && load != 0.0) move_boundary(A, i, load);
        A.pxy[i] = make_double2(A.x[i] + A.ux[i], A.y[i] + A.uy[i]);
    }
}

BatchArgs batch_args(pd_ctx* c) {
    BatchArgs a;
    a.P = kparams(c->p);
    double** f = c->nf;
    a.x = f[PD_F_X], a.y = f[PD_F_Y], a.ux = f[PD_F_UX], a.uy = f[PD_F_UY], a.vx = f[PD_F_VX], a.vy = f[PD_F_VY];
    a.fx = f[PD_F_FX], a.fy = f[PD_F_FY], a.bx = f[PD_F_BX], a.by = f[PD_F_BY];
    a.vhx = f[PD_F_VHX], a.vhy = f[PD_F_VHY], a.fox = f[PD_F_FOX], a.foy = f[PD_F_FOY];
    a.pxy = c->posxy[c->parity];
    a.mass = c->batch.node_mass;
    a.c1 = c->batch.node_c1;
    a.sign = c->batch.load_sign;
    a.slice_inst = c->batch.slice_inst;
    a.inst_cn = c->batch.inst_cn;
    a.inst_nd = c->batch.inst_nd;
    return a;
}

inline unsigned node_grid(pd_ctx* c, int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + T - 1) / T, (int64_t)c->num_sms * 16));
}

template <typename V>
cudaError_t upload(V*& dst, const std::vector<V>& src) {
    cudaError_t e = cudaMalloc(&dst, std::max<size_t>(src.size(), 1) * sizeof(V));
    if (e == cudaSuccess && !src.empty())
        e = cudaMemcpy(dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice);
    return e;
}

}  // namespace

void release_batch(pd_ctx* c) {
    BatchInfo& b = c->batch;
    void* ptrs[] = {b.node_group, b.node_bc,    b.node_sed,    b.node_s0,    b.node_mass, b.node_c1,
                    b.node_rmass, b.load_sign,  b.slice_inst,  b.inst_slices, b.slice_part, b.inst_cn,
                    b.inst_nd};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    b = BatchInfo{};
}

int batch_prologue(pd_ctx* c, double load, cudaStream_t s) {
    BatchArgs A = batch_args(c);
    k_batch_prologue<<<node_grid(c, A.P.N), T, 0, s>>>(A, load);
    c->launches++;
    c->pos_valid = true;
    return cuda_err(c, cudaGetLastError(), "batch prologue");
}

int batch_force(pd_ctx* c, cudaStream_t s) {
    StepFlags f;
    f.epi = EPI_ADR;
    f.residual = 0;  // a batch has no convergence check
    return launch_force(c, f, s);
}

int batch_finish(pd_ctx* c, int ct, int last, double load, cudaStream_t s) {
    const BatchInfo& B = c->batch;
    k_batch_cn<<<(unsigned)(((int64_t)B.count * 32 + T - 1) / T), T, 0, s>>>(B.count, B.inst_slices, B.slice_part,
                                                                              c->p.dt, B.inst_cn, B.inst_nd);
    BatchArgs A = batch_args(c);
    k_batch_update<<<node_grid(c, A.P.N), T, 0, s>>>(A, ct, last ? 0 : 1, load);
    c->launches += 2;
    c->pos_valid = true;
    return cuda_err(c, cudaGetLastError(), "batch step");
}

int batch_step(pd_ctx* c, int ct, int last, double load, cudaStream_t s) {
    int rc = batch_force(c, s);
    return rc ? rc : batch_finish(c, ct, last, load, s);
}

}  // namespace pdg

using namespace pdg;

extern "C" {

pd_ctx* pd_batch_create(const pd_params* base, const pd_specimen* spec, int count, int* status) {
    auto fail = [&](int st) -> pd_ctx* {
        if (status) *status = st;
        return nullptr;
    };
    if (!base || !spec || count <= 0 || base->dim != 2 || base->model != PD_MODEL_BOND || !(base->dx > 0.0))
        return fail(PD_ERR_ARG);
    const double dx = base->dx;
    // ---- per-specimen parameters, derived exactly as a standalone run's ----
    std::vector<pd_params> q((size_t)count);
    std::vector<int64_t> int_off(count + 1), bnd_off(count + 1);
    int64_t nint = 0, nbnd = 0;
    int maxnx = 0, maxny = 0;
    for (int k = 0; k < count; k++) {
        const pd_specimen& sp = spec[k];
        if (sp.nx < 4 || sp.ny < 4 || !(sp.emod > 0.0) || !(sp.critical_s > 0.0) || !(sp.crack_len >= 0.0) ||
            !std::isfinite(sp.load_scale))
            return fail(PD_ERR_ARG);
        int rc = pd_params_derive(&q[k], 2, PD_MODEL_BOND, base->mode, base->dt, base->nt, dx, base->load,
                                  base->thick, sp.nx * dx, sp.ny * dx, 0.0, sp.emod, base->pratio, base->dens,
                                  sp.critical_s, 0);
        if (rc) return fail(rc);
        int_off[k] = nint;
        nint += ((int64_t)sp.nx * sp.ny + 31) / 32 * 32;
        bnd_off[k] = nbnd;
        nbnd += 6 * (int64_t)sp.nx;
        maxnx = std::max(maxnx, sp.nx);
        maxny = std::max(maxny, sp.ny);
    }
    int_off[count] = nint;
    bnd_off[count] = nbnd;
    const int64_t N = nint + nbnd;
    if (N > INT32_MAX / 2) return fail(PD_ERR_ARG);
    pd_params p = *base;
    p.N = (int32_t)N;
    p.N_int = (int32_t)nint;
    p.nx = maxnx;  // widest specimen (the per-specimen layouts are in the offset tables)
    p.ny = maxny;
    p.nz = 1;
    // ---- node arrays --------------------------------------------------------
    std::vector<double> x((size_t)N, 0.0), y((size_t)N, 0.0), mass((size_t)N, 1.0), sign((size_t)N, 0.0);
    std::vector<double> nbc((size_t)N, 0.0), nsed((size_t)N, 0.0), ns0((size_t)N, 0.0);
    std::vector<int> grp((size_t)N, -1);
    for (int k = 0; k < count; k++) {
        const pd_specimen& sp = spec[k];
        const pd_params& qk = q[k];
        const int nx = sp.nx, ny = sp.ny;
        // surface-correction energy density of Surf_Corr.cu:246 (2-D)
        const double sed = 0.5 * qk.emod / (1.0 - qk.pratio * qk.pratio) * 1.0e-6;
        auto node = [&](int64_t r, double xr, double yr, double sg) {
            x[r] = xr;
            y[r] = yr;
            grp[r] = k;
            nbc[r] = qk.bc;
            nsed[r] = sed;
            ns0[r] = qk.critical_s;
            mass[r] = qk.mass;
            sign[r] = sg;
        };
        // kernel_coord_plate_crack layout (Coord.cu:34-45) of this specimen
        for (int64_t idx = 0; idx < (int64_t)nx * (ny + 3); idx++) {
            const double xr = (-nx / 2.0 + 0.5 + (double)(idx % nx)) * dx;
            const double yr = (-ny / 2.0 + 0.5 + (double)(idx / nx)) * dx;
            if (idx < (int64_t)nx * ny)
                node(int_off[k] + idx, xr, yr, 0.0);
            else
                node(nint + bnd_off[k] + (idx - (int64_t)nx * ny), xr, yr, sp.load_scale);
        }
        for (int64_t idx = 0; idx < 3 * (int64_t)nx; idx++) {
            const double xr = (-nx / 2.0 + 0.5 + (double)(idx % nx)) * dx;
            const double yr = (-ny / 2.0 - 0.5 - (double)(idx / nx)) * dx;
            node(nint + bnd_off[k] + 3 * (int64_t)nx + idx, xr, yr, -sp.load_scale);
        }
        // padding rows: the specimen's material, no family (group -1), at rest
        for (int64_t r = int_off[k] + (int64_t)nx * ny; r < int_off[k + 1]; r++) {
            node(r, 0.0, 0.0, 0.0);
            grp[r] = -1;
        }
    }
    int st = 0;
    pd_ctx* c = pd_create(&p, &st);
    if (!c) return fail(st);
    BatchInfo& B = c->batch;
    B.count = count;
    B.h_inst_nodes = int_off;
    B.h_inst_bnd = bnd_off;
    const int64_t nslices = (N + 31) / 32;
    std::vector<int> slice_inst((size_t)nslices, -1);
    std::vector<int64_t> inst_slices(count + 1);
    for (int k = 0; k < count; k++) {
        inst_slices[k] = int_off[k] / 32;
        for (int64_t s2 = int_off[k] / 32; s2 < int_off[k + 1] / 32; s2++) slice_inst[s2] = k;
    }
    inst_slices[count] = nint / 32;
    cudaError_t e = cudaSuccess;
    auto up = [&](auto*& dst, const auto& src) {
        if (e == cudaSuccess) e = upload(dst, src);
    };
    up(B.node_group, grp);
    up(B.node_bc, nbc);
    up(B.node_sed, nsed);
    up(B.node_s0, ns0);
    up(B.node_mass, mass);
    {
        std::vector<double> c1((size_t)N);
        for (int64_t r = 0; r < N; r++) c1[r] = 2.0 * p.dt / mass[r];  // kernel_integrate's 2 dt / mass
        up(B.node_c1, c1);
        for (int64_t r = 0; r < N; r++) c1[r] = 1.0 / mass[r];  // the ADR epilogue's divisor reciprocal
        up(B.node_rmass, c1);
    }
    up(B.load_sign, sign);
    up(B.slice_inst, slice_inst);
    up(B.inst_slices, inst_slices);
    up(B.slice_part, std::vector<double>(2 * (size_t)nslices, 0.0));
    up(B.inst_cn, std::vector<double>((size_t)count, 0.0));
    up(B.inst_nd, std::vector<double>(3 * (size_t)count, 0.0));
    if (e != cudaSuccess) {
        pd_destroy(c);
        return fail(e == cudaErrorMemoryAllocation ? PD_ERR_NOMEM : PD_ERR_CUDA);
    }
    // ---- family, surface correction, pre-cracks, bond arrays ------------------
    int rc;
    if ((rc = pd_set_field(c, PD_F_X, x.data(), N, nullptr)) || (rc = pd_set_field(c, PD_F_Y, y.data(), N, nullptr)) ||
        (rc = pd_find_neighbor(c, nullptr)) || (rc = pd_surface_correct(c, nullptr)) ||
        (rc = pd_initial_state(c, nullptr))) {
        pd_destroy(c);
        return fail(rc);
    }
    for (int k = 0; k < count && !rc; k++)
        if (spec[k].crack_len > 0.0)
            rc = set_crack_2d_rows(c, int_off[k], int_off[k] + (int64_t)spec[k].nx * spec[k].ny, spec[k].crack_len,
                                   0.0, 0.0, spec[k].crack_theta, nullptr);
    if (rc || (rc = pd_prepare(c, nullptr)) || (rc = cuda_err(c, cudaDeviceSynchronize(), "pd_batch_create"))) {
        pd_destroy(c);
        return fail(rc);
    }
    if (status) *status = PD_OK;
    return c;
}

int pd_batch_info(const pd_ctx* c, int* count, int64_t* interior_offsets, int64_t* boundary_offsets) {
    if (!c || !count) return PD_ERR_ARG;
    const BatchInfo& B = c->batch;
    *count = B.count;
    if (interior_offsets) std::copy(B.h_inst_nodes.begin(), B.h_inst_nodes.end(), interior_offsets);
    if (boundary_offsets) std::copy(B.h_inst_bnd.begin(), B.h_inst_bnd.end(), boundary_offsets);
    return PD_OK;
}

int pd_batch_get_cn(pd_ctx* c, double* cn, void* stream) {
    if (!c || !cn) return PD_ERR_ARG;
    if (c->batch.count == 0) return set_err(c, PD_ERR_STATE, "not a batch context");
    cudaError_t e = cudaMemcpyAsync(cn, c->batch.inst_cn, c->batch.count * sizeof(double), cudaMemcpyDeviceToHost,
                                    st(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(st(stream));
    return cuda_err(c, e, "pd_batch_get_cn");
}

}  // extern "C"
