// C ABI of the engine (include/pd.h): context management, field I/O, the
// per-operator entry points that replace the reference's host launchers, the
// graph-captured step loops and the three drivers.
//
// Host arithmetic that must match the reference (parameter derivation,
// coordinates) is written with the reference's operand order and this file's
// host code is compiled with -ffp-contract=off.
#include <atomic>
#include <cmath>
#include <cstring>

#include "pd_internal.cuh"

namespace pdg {

int set_err(pd_ctx* c, int status, const std::string& msg) {
    if (c) c->err = msg;
    return status;
}

int cuda_err(pd_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PD_OK;
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PD_ERR_NOMEM : PD_ERR_CUDA;
}

void release_sell(pd_ctx* c);

// Every cached graph bakes in device pointers (SELL arrays, node fields,
// position buffers) and kernel parameters by value; any reallocation or
// parameter change must drop them before the next replay.
void drop_graphs(pd_ctx* c) {
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

namespace {

__global__ void k_fill_int(int* a, int64_t n, int v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

// The extension of each slot (a float pair) into the CSR-ordered double array.
__global__ void k_sell_to_csr(int64_t S, const int* __restrict__ csr, const float2* __restrict__ src,
                              double* __restrict__ dst) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < S; t += (int64_t)gridDim.x * blockDim.x) {
        const int q = csr[t];
        if (q >= 0) dst[q] = (double)src[t].x + (double)src[t].y;
    }
}

__global__ void k_cyl_half(KParams P, CylDev* cy, int half) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int a = 0; a < 3; a++) {
        if (half == 1) {  // kernel_cy_integrate_1
            cy->vel[a] = fma(P.dt / 2.0, cy->acc[a], cy->vel[a]);
            cy->disp[a] = fma(cy->vel[a], P.dt, cy->disp[a]);
        } else {  // kernel_cy_integrate_2
            cy->acc[a] = cy->force[a] / cy->mass;
            cy->vel[a] = fma(P.dt / 2.0, cy->acc[a], cy->vel[a]);
            cy->force[a] = 0.0;
        }
    }
}

constexpr int kNodeDoubleFields = PD_F_NN;  // node fields stored as double arrays

int field_info(const pd_ctx* c, int f, size_t* count, size_t* esize) {
    if (f < 0 || f >= PD_F_COUNT) return PD_ERR_ARG;
    const int64_t N = c->p.N;
    if (f < kNodeDoubleFields) {
        *count = (size_t)N;
        *esize = 8;
    } else if (f == PD_F_NN) {
        *count = (size_t)N;
        *esize = 4;
    } else if (f == PD_F_ROWPTR) {
        *count = (size_t)N + 1;
        *esize = 8;
    } else {
        if (!c->family) return PD_ERR_STATE;
        *count = (size_t)c->B;
        *esize = (f == PD_F_NL || f == PD_F_FAIL) ? 4 : 8;
    }
    return PD_OK;
}

void* field_dev(pd_ctx* c, int f) {
    if (f < kNodeDoubleFields) return c->nf[f];
    switch (f) {
        case PD_F_NN: return c->NN;
        case PD_F_ROWPTR: return c->rowptr;
        case PD_F_NL: return c->NL;
        case PD_F_IDIST: return c->idist;
        case PD_F_FAC: return c->fac;
        case PD_F_SCR: return c->scr;
        case PD_F_W: return c->w;
        case PD_F_E: return c->e;
        case PD_F_FAIL: return c->fail;
        default: return nullptr;
    }
}

bool is_pos_field(int f) {
    return f == PD_F_X || f == PD_F_Y || f == PD_F_Z || f == PD_F_UX || f == PD_F_UY || f == PD_F_UZ;
}

// Make the bond coefficients, intact bits and position buffer current.
int ensure_ready(pd_ctx* c, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "no bond family: call pd_find_neighbor");
    int rc;
    if (!c->prepared && (rc = prepare(c, s))) return rc;
    if ((rc = sync_fail_to_bits(c, s))) return rc;
    if (!c->pos_valid && (rc = refresh_pos(c, s))) return rc;
    return PD_OK;
}

// Runs `body` either directly or as a cached CUDA graph keyed by `key`.
struct Key {
    int kind, nsteps, parity, flags;
    double load;
    int dmg_every;
};

bool graph_match(const GraphEntry& g, const Key& k) {
    return g.kind == k.kind && g.nsteps == k.nsteps && g.parity == k.parity && (g.flags & 0xffff) == k.flags &&
           g.load == k.load && g.dmg_every == k.dmg_every;
}

// Stream used for capture: the caller's, or the context's own when the caller
// passes the legacy default stream (which cannot be captured).
struct StreamScope {
    pd_ctx* c;
    cudaStream_t user, s;
    cudaStream_t own = nullptr;
    cudaEvent_t ev = nullptr;
    StreamScope(pd_ctx* ctx, void* stream) : c(ctx), user(st(stream)), s(st(stream)) {
        if (user == nullptr) {
            cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            cudaEventRecord(ev, 0);
            cudaStreamWaitEvent(own, ev, 0);
            s = own;
        }
    }
    ~StreamScope() {
        if (own) {
            cudaEventRecord(ev, own);
            cudaStreamWaitEvent(0, ev, 0);
            cudaStreamSynchronize(own);
            cudaStreamDestroy(own);
            cudaEventDestroy(ev);
        }
    }
};

}  // namespace

int make_ready(pd_ctx* c, cudaStream_t s) { return ensure_ready(c, s); }

// Look-up helper shared by the run loops: finds a cached graph whose low flag
// bits match, or captures one.
template <typename F>
static int graph_chunk(pd_ctx* c, const Key& k, cudaStream_t s, F body) {
    for (auto& g : c->graphs) {
        if (graph_match(g, k)) {
            cudaError_t e = cudaGraphLaunch(g.exec, s);
            if (e != cudaSuccess) return cuda_err(c, e, "graph launch");
            c->launches += g.kernels;
            c->parity = (g.flags >> 16) & 1;
            c->pos_valid = true;
            c->csr_fail_current = false;
            return PD_OK;
        }
    }
    cudaGraph_t graph;
    const int64_t l0 = c->launches;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(c, e, "begin capture");
    int rc = body();
    e = cudaStreamEndCapture(s, &graph);
    if (rc) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_err(c, e, "end capture");
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(c, e, "graph instantiate");
    GraphEntry g{k.kind, k.nsteps, k.parity, k.flags | ((c->parity & 1) << 16), k.load, k.dmg_every, exec,
                 c->launches - l0};
    c->graphs.push_back(g);
    e = cudaGraphLaunch(exec, s);
    if (e != cudaSuccess) return cuda_err(c, e, "graph launch");
    return PD_OK;
}

}  // namespace pdg

using namespace pdg;

// ---------------------------------------------------------------------------
// Test hook (pd_debug_fail_allocation): device allocations of pd_create
// still to go before one is refused as if the device were out of memory; -1:
// none is refused.
static std::atomic<int> g_alloc_countdown{-1};

template <class T>
static bool ctx_alloc(T** ptr, size_t bytes) {
    const int k = g_alloc_countdown.load();
    if (k >= 0) {
        g_alloc_countdown.store(k - 1);
        if (k == 0) return false;
    }
    return cudaMalloc(ptr, bytes) == cudaSuccess;
}

extern "C" {

const char* pd_status_string(int status) {
    switch (status) {
        case PD_OK: return "PD_OK";
        case PD_ERR_ARG: return "PD_ERR_ARG";
        case PD_ERR_CUDA: return "PD_ERR_CUDA";
        case PD_ERR_STATE: return "PD_ERR_STATE";
        case PD_ERR_FAMILY: return "PD_ERR_FAMILY";
        case PD_ERR_NONFINITE: return "PD_ERR_NONFINITE";
        case PD_ERR_NOMEM: return "PD_ERR_NOMEM";
        case PD_ERR_TIMEOUT: return "PD_ERR_TIMEOUT";
        case PD_ERR_UNSUPPORTED: return "PD_ERR_UNSUPPORTED";
        default: return "PD_ERR_UNKNOWN";
    }
}

const char* pd_last_error(const pd_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

int pd_params_derive(pd_params* p, int dim, int model, int mode, double dt, double nt, double dx, double load,
                     double thick, double length, double height, double width, double emod, double pratio,
                     double dens, double critical_s, int fix_k3d) {
    if (!p || (dim != 2 && dim != 3) || (model != PD_MODEL_BOND && model != PD_MODEL_STATE) || !(dx > 0.0))
        return PD_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    const double pi = std::acos(-1.0);  // Base.cuh:31
    p->pi = pi;
    p->dim = dim;
    p->model = model;
    p->mode = mode;
    p->dt = dt;
    p->nt = (int32_t)nt;
    p->dx = dx;
    p->load = load;
    p->length = length;
    p->height = height;
    p->width = width;
    p->emod = emod;
    p->pratio = pratio;
    p->dens = dens;
    p->critical_s = critical_s;
    // BaseModel_Parameter::cal_parameter (Base.cuh:114-183)
    p->delta = 3.015 * dx;
    p->nx = (int32_t)((length - dx / 2.0) / dx + 1);
    p->ny = (int32_t)((height - dx / 2.0) / dx + 1);
    p->nz = dim == 3 ? (int32_t)((width - dx / 2.0) / dx + 1) : 0;
    p->MN = dim == 2 ? 32 : 128;
    p->N = p->N_int = dim == 2 ? p->nx * p->ny : p->nx * p->ny * p->nz;
    p->break_ymin = dim == 3 ? -0.04 : -1e300;
    p->sedload = dim == 3 ? 0.6 * emod * 1.0e-6 : 0.5 * emod / (1.0 - pratio * pratio) * 1.0e-6;
    const double delta = p->delta;
    if (model == PD_MODEL_BOND) {
        p->thick = thick;
        if (dim == 2) {
            p->vol = dx * dx * thick;
            p->bc = 6.0 * emod / (pi * thick * (delta * delta * delta) * (1.0 - pratio));
        } else {
            p->vol = dx * dx * dx;
            p->bc = 6.0 * emod / (pi * delta * (delta * delta * delta) * (1.0 - 2.0 * pratio));
        }
        p->mass = 0.25 * dt * dt * (pi * delta * delta * thick) * (p->bc) / dx * 5.0;
    } else {
        p->G = 0.5 * emod / (1 + pratio);
        if (dim == 2) {
            p->thick = dx;  // Base.cuh:166
            p->vol = dx * dx * p->thick;
            p->K = 0.5 * emod / (1 - pratio);
        } else {
            p->thick = thick;
            p->K = fix_k3d ? emod / (3.0 * (1.0 - 2.0 * pratio)) : emod / 3.0 / (1 - 2.0 * p->G);
            p->vol = dx * dx * dx;
        }
    }
    return PD_OK;
}

int pd_debug_fail_allocation(int n) {
    if (n < -1) return PD_ERR_ARG;
    g_alloc_countdown.store(n);
    return PD_OK;
}

pd_ctx* pd_create(const pd_params* p, int* status) {
    auto fail = [&](int st) -> pd_ctx* {
        if (status) *status = st;
        return nullptr;
    };
    if (!p || p->N <= 0 || p->N_int < 0 || p->N_int > p->N || (p->dim != 2 && p->dim != 3) ||
        (p->model != PD_MODEL_BOND && p->model != PD_MODEL_STATE))
        return fail(PD_ERR_ARG);
    if (p->critical_s < 0.0) return fail(PD_ERR_ARG);
    pd_ctx* c = new pd_ctx();
    c->p = *p;
    cudaGetDevice(&c->device);
    if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) {
        delete c;
        return fail(PD_ERR_CUDA);
    }
    const size_t nb = (size_t)p->N * 8;
    bool ok = true;
    for (int f = 0; f < kNodeDoubleFields && ok; f++) ok = ctx_alloc(&c->nf[f], nb);
    for (int b = 0; b < 2 && ok; b++)
        ok = ctx_alloc(&c->posxy[b], 2 * nb) && ctx_alloc(&c->posz[b], nb);
    ok = ok && ctx_alloc(&c->NN, (size_t)p->N * 4);
    ok = ok && ctx_alloc(&c->rowptr, ((size_t)p->N + 1) * 8);
    ok = ok && ctx_alloc(&c->node_a, 2 * nb) && ctx_alloc(&c->node_b, nb);
    ok = ok && ctx_alloc(&c->partials, (size_t)kMaxPartials * 4 * 8);
    ok = ok && ctx_alloc(&c->ticket, 4 * sizeof(unsigned));
    ok = ok && ctx_alloc(&c->cn, 8) && ctx_alloc(&c->red_out, 8);
    ok = ok && ctx_alloc(&c->res, 8);
    ok = ok && ctx_alloc(&c->cyl, sizeof(CylDev));
    if (!ok) {
        pd_destroy(c);
        cudaGetLastError();
        return fail(PD_ERR_NOMEM);
    }
    for (int f = 0; f < kNodeDoubleFields; f++) cudaMemset(c->nf[f], 0, nb);
    for (int b = 0; b < 2; b++)
        cudaMemset(c->posxy[b], 0, 2 * nb), cudaMemset(c->posz[b], 0, nb);
    cudaMemset(c->NN, 0, (size_t)p->N * 4);
    cudaMemset(c->rowptr, 0, ((size_t)p->N + 1) * 8);
    cudaMemset(c->node_a, 0, 2 * nb);
    cudaMemset(c->node_b, 0, nb);
    cudaMemset(c->ticket, 0, 4 * sizeof(unsigned));
    cudaMemset(c->cn, 0, 8);
    cudaMemset(c->res, 0, 8);
    cudaMemset(c->cyl, 0, sizeof(CylDev));
    c->pos_valid = true;
    if (cudaDeviceSynchronize() != cudaSuccess) {
        pd_destroy(c);
        return fail(PD_ERR_CUDA);
    }
    if (status) *status = PD_OK;
    return c;
}

int pd_destroy(pd_ctx* c) {
    if (!c) return PD_ERR_ARG;
    drop_graphs(c);
    for (int f = 0; f < kNodeDoubleFields; f++)
        if (c->nf[f]) cudaFree(c->nf[f]);
    for (int b = 0; b < 2; b++) {
        if (c->posxy[b]) cudaFree(c->posxy[b]);
        if (c->posz[b]) cudaFree(c->posz[b]);
    }
    void* ptrs[] = {c->NN,  c->rowptr, c->node_a, c->node_b, c->partials, c->ticket, c->cn,
                    c->red_out, c->res, c->cyl, c->NL, c->idist, c->fac, c->scr, c->w, c->e, c->fail,
                    c->warm_hist};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    release_sell(c);
    release_batch(c);
    delete c;
    return PD_OK;
}

int pd_get_params(const pd_ctx* c, pd_params* out) {
    if (!c || !out) return PD_ERR_ARG;
    *out = c->p;
    return PD_OK;
}

int pd_set_params(pd_ctx* c, const pd_params* p) {
    if (!c || !p) return PD_ERR_ARG;
    if (p->N != c->p.N || p->dim != c->p.dim || p->model != c->p.model || p->N_int > p->N || p->critical_s < 0.0)
        return set_err(c, PD_ERR_ARG, "pd_set_params cannot change N, dim or model");
    if (c->batch.count && p->dt != c->p.dt)  // the per-node ADR coefficients were formed at pd_batch_create
        return set_err(c, PD_ERR_ARG, "pd_set_params cannot change dt of a batch");
    c->p = *p;
    c->prepared = false;  // coefficients depend on the parameters
    drop_graphs(c);
    return PD_OK;
}

int pd_get_field(pd_ctx* c, int field, void* host, size_t count, void* stream) {
    if (!c || !host) return PD_ERR_ARG;
    size_t n, es;
    int rc = field_info(c, field, &n, &es);
    if (rc) return set_err(c, rc, "bad field id or bond field before pd_find_neighbor");
    if (count > n) return set_err(c, PD_ERR_ARG, "count exceeds the field size");
    cudaStream_t s = st(stream);
    if (field == PD_F_FAIL && (rc = sync_fail_to_csr(c, s))) return rc;
    if (field == PD_F_E && c->p.model == PD_MODEL_STATE && c->prepared) {
        const int64_t S = c->sell.S;
        k_sell_to_csr<<<(unsigned)std::min<int64_t>((S + 255) / 256 + 1, 65535), 256, 0, s>>>(S, c->sell.csr,
                                                                                              c->sell.e, c->e);
        c->launches++;
    }
    cudaError_t e = cudaMemcpyAsync(host, field_dev(c, field), count * es, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_err(c, e, "pd_get_field");
}

int pd_set_field(pd_ctx* c, int field, const void* host, size_t count, void* stream) {
    if (!c || !host) return PD_ERR_ARG;
    size_t n, es;
    int rc = field_info(c, field, &n, &es);
    if (rc) return set_err(c, rc, "bad field id or bond field before pd_find_neighbor");
    if (count > n) return set_err(c, PD_ERR_ARG, "count exceeds the field size");
    if (field == PD_F_NN || field == PD_F_ROWPTR || field == PD_F_NL)
        return set_err(c, PD_ERR_ARG, "the bond family is built by pd_find_neighbor");
    cudaStream_t s = st(stream);
    if (field == PD_F_FAIL && (rc = sync_fail_to_csr(c, s))) return rc;
    cudaError_t e = cudaMemcpyAsync(field_dev(c, field), host, count * es, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_set_field");
    if (is_pos_field(field)) c->pos_valid = false;
    if (field == PD_F_X || field == PD_F_Y || field == PD_F_Z) {
        c->family = false;
        c->prepared = false;
    }
    if (field == PD_F_IDIST || field == PD_F_FAC || field == PD_F_SCR || field == PD_F_W || field == PD_F_M)
        c->prepared = false;
    if (field == PD_F_FAIL) c->bits_current = false;
    return PD_OK;
}

int pd_field_ptr(pd_ctx* c, int field, void** dev, size_t* count) {
    if (!c || !dev) return PD_ERR_ARG;
    size_t n, es;
    int rc = field_info(c, field, &n, &es);
    if (rc) return set_err(c, rc, "bad field id or bond field before pd_find_neighbor");
    *dev = field_dev(c, field);
    if (count) *count = n;
    if (is_pos_field(field)) c->pos_valid = false;  // the caller may write through it
    return PD_OK;
}

int64_t pd_num_bonds(const pd_ctx* c) { return c ? c->B : -1; }

int pd_sync(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    return cuda_err(c, cudaStreamSynchronize(st(stream)), "pd_sync");
}

// ---- geometry --------------------------------------------------------------
static int put_coords(pd_ctx* c, const std::vector<double>& x, const std::vector<double>& y, void* stream) {
    cudaStream_t s = st(stream);
    cudaMemcpyAsync(c->nf[PD_F_X], x.data(), x.size() * 8, cudaMemcpyHostToDevice, s);
    cudaError_t e = cudaMemcpyAsync(c->nf[PD_F_Y], y.data(), y.size() * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    c->family = false;
    c->prepared = false;
    c->pos_valid = false;
    return cuda_err(c, e, "coordinates");
}

int pd_coord_plate(pd_ctx* c, void* stream) {
    if (!c || c->p.dim != 2) return PD_ERR_ARG;
    const pd_params& p = c->p;
    if ((int64_t)p.nx * p.ny > p.N) return set_err(c, PD_ERR_ARG, "nx*ny exceeds N");
    std::vector<double> x((size_t)p.N, 0.0), y((size_t)p.N, 0.0);
    for (int i = 0; i < p.ny; i++)  // Initial_coord_plate_cpu (Coord.cu:19-28)
        for (int j = 0; j < p.nx; j++) {
            x[(size_t)i * p.nx + j] = (-p.nx / 2.0 + 0.5 + j) * p.dx;
            y[(size_t)i * p.nx + j] = (-p.ny / 2.0 + 0.5 + i) * p.dx;
        }
    return put_coords(c, x, y, stream);
}

int pd_coord_plate_crack(pd_ctx* c, void* stream) {
    if (!c || c->p.dim != 2) return PD_ERR_ARG;
    const pd_params& p = c->p;
    if ((int64_t)p.N_int + 6 * (int64_t)p.nx != p.N) return set_err(c, PD_ERR_ARG, "N must be N_int + 6 nx");
    std::vector<double> x((size_t)p.N), y((size_t)p.N);
    const int64_t top = (int64_t)p.N_int + 3 * (int64_t)p.nx;
    for (int64_t idx = 0; idx < p.N; idx++) {  // kernel_coord_plate_crack (Coord.cu:34-45)
        x[idx] = (-p.nx / 2.0 + 0.5 + (double)(idx % p.nx)) * p.dx;
        if (idx < top)
            y[idx] = (-p.ny / 2.0 + 0.5 + (double)(idx / p.nx)) * p.dx;
        else
            y[idx] = (-p.ny / 2.0 - 0.5 - (double)((idx - p.N_int - 3 * (int64_t)p.nx) / p.nx)) * p.dx;
    }
    return put_coords(c, x, y, stream);
}

int pd_coord_kw(const pd_params* p, double rad, double* x, double* y, double* z, int64_t cap, int64_t* n) {
    if (!p || !n || cap < 0 || p->dim != 3) return PD_ERR_ARG;
    int64_t num = 0;
    for (int k = 0; k < p->nz; k++)  // coord_KW (Coord.cu:77-129)
        for (int j = 0; j < p->ny; j++)
            for (int i = 0; i < p->nx; i++) {
                const double tx = (-(p->nx - 1) / 2.0 + i) * p->dx;
                const double ty = (-(p->ny - 1) / 2.0 + j) * p->dx;
                const double tz = (-p->nz / 2.0 + 0.5 + k) * p->dx;
                bool keep;
                if (tx > (-rad - 1.1 * p->dx) && tx < (-rad + 0.1 * p->dx))
                    keep = ty < -1.0e-10;
                else if (tx > (rad - 0.1 * p->dx) && tx < (rad + 1.1 * p->dx))
                    keep = ty < -1.0e-10;
                else
                    keep = true;
                if (keep) {
                    if (num < cap && x && y && z) {
                        x[num] = tx;
                        y[num] = ty;
                        z[num] = tz;
                    }
                    num++;
                }
            }
    *n = num;
    return num <= cap ? PD_OK : PD_ERR_ARG;
}

// ---- family and setup -------------------------------------------------------
int pd_find_neighbor(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    drop_graphs(c);
    release_sell(c);
    return build_family(c, st(stream));
}

int pd_vol_corr(pd_ctx* c, void* stream) { return c ? vol_corr(c, st(stream)) : PD_ERR_ARG; }
int pd_surface_correct(pd_ctx* c, void* stream) { return c ? surface_correct(c, st(stream)) : PD_ERR_ARG; }
int pd_initial_weight(pd_ctx* c, void* stream) { return c ? initial_weight(c, st(stream)) : PD_ERR_ARG; }
int pd_set_crack_2d(pd_ctx* c, double clength, double lx, double ly, double theta, void* stream) {
    return c ? set_crack_2d(c, clength, lx, ly, theta, st(stream)) : PD_ERR_ARG;
}
int pd_set_crack_kw(pd_ctx* c, double rad, void* stream) { return c ? set_crack_kw(c, rad, st(stream)) : PD_ERR_ARG; }
int pd_prepare(pd_ctx* c, void* stream) { return c ? prepare(c, st(stream)) : PD_ERR_ARG; }

int pd_initial_state(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    const int ids[] = {PD_F_UX, PD_F_UY, PD_F_UZ, PD_F_VX, PD_F_VY, PD_F_VZ, PD_F_AX, PD_F_AY, PD_F_AZ,
                       PD_F_FX, PD_F_FY, PD_F_FZ, PD_F_BX, PD_F_BY, PD_F_BZ, PD_F_VHX, PD_F_VHY, PD_F_VHZ,
                       PD_F_FOX, PD_F_FOY, PD_F_FOZ, PD_F_DMG};
    for (int f : ids) cudaMemsetAsync(c->nf[f], 0, (size_t)c->p.N * 8, s);
    cudaMemsetAsync(c->cn, 0, 8, s);
    if (c->family) {
        k_fill_int<<<(unsigned)std::min<int64_t>((c->B + 255) / 256 + 1, 65535), 256, 0, s>>>(c->fail, c->B, 1);
        c->launches++;
        c->csr_fail_current = true;
        c->bits_current = false;
    }
    c->pos_valid = false;
    return cuda_err(c, cudaGetLastError(), "initial_state");
}

// ---- forces -------------------------------------------------------------------
int pd_bond_force(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    if (c->p.model != PD_MODEL_BOND) return set_err(c, PD_ERR_STATE, "the context is state-based");
    cudaStream_t s = st(stream);
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    StepFlags f;
    return launch_force(c, f, s);
}

int pd_state_force(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    if (c->p.model != PD_MODEL_STATE) return set_err(c, PD_ERR_STATE, "the context is bond-based");
    cudaStream_t s = st(stream);
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    if ((rc = launch_theta(c, s))) return rc;
    StepFlags f;
    return launch_force(c, f, s);
}

// ---- integration --------------------------------------------------------------
int pd_integrate_adr(pd_ctx* c, int ct, void* stream) {
    if (!c) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens steps with pd_batch_run_adr");
    cudaStream_t s = st(stream);
    int rc = launch_adr_cnn(c, s);
    if (rc) return rc;
    return launch_adr_update(c, ct, 0, 0.0, s);
}

int pd_get_adr_cn(pd_ctx* c, double* cn, void* stream) {
    if (!c || !cn) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens has one cn per specimen");
    cudaError_t e = cudaMemcpyAsync(cn, c->cn, 8, cudaMemcpyDeviceToHost, st(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(st(stream));
    return cuda_err(c, e, "pd_get_adr_cn");
}

int pd_integrate_verlet1(pd_ctx* c, void* stream) { return c ? launch_verlet1(c, st(stream)) : PD_ERR_ARG; }
int pd_integrate_verlet2(pd_ctx* c, void* stream) { return c ? launch_verlet2(c, st(stream)) : PD_ERR_ARG; }

int pd_reduce_sum(pd_ctx* c, const double* dev_x, int64_t n, double* result, void* stream) {
    if (!c || !dev_x || !result || n < 0) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    int rc = reduce_sum(c, dev_x, n, c->red_out, s);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(result, c->red_out, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_err(c, e, "pd_reduce_sum");
}

int pd_damage(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    if (!c->family) return set_err(c, PD_ERR_STATE, "damage needs the bond family");
    if (!c->volcorr) {
        int rc = vol_corr(c, st(stream));
        if (rc) return rc;
    }
    return launch_damage(c, st(stream));
}

int pd_quick_load(pd_ctx* c, double load, void* stream) {
    if (!c) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "batch boundary rows move inside pd_batch_run_adr");
    return launch_quick_load(c, load, st(stream));
}

int pd_load_plate_tensile(pd_ctx* c, void* stream) {
    if (!c || c->p.dim != 2) return PD_ERR_ARG;
    return pdg::launch_load_tensile(c, st(stream));
}

int pd_cylinder_init(pd_ctx* c, const pd_cylinder* cyl, void* stream) {
    if (!c || !cyl) return PD_ERR_ARG;
    CylDev d{};
    d.rad = cyl->rad;
    d.mass = cyl->mass;
    d.height = cyl->height;
    d.v = cyl->v;
    d.x = cyl->x;
    d.y = cyl->y;
    d.z = cyl->z;
    for (int a = 0; a < 3; a++) {
        d.vel[a] = cyl->vel[a];
        d.disp[a] = cyl->disp[a];
        d.acc[a] = cyl->acc[a];
        d.force[a] = cyl->force[a];
    }
    cudaError_t e = cudaMemcpyAsync(c->cyl, &d, sizeof(d), cudaMemcpyHostToDevice, st(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(st(stream));
    if (e == cudaSuccess) {
        if (!c->has_cyl) drop_graphs(c);  // captured steps without the contact epilogue
        c->has_cyl = true;
    }
    return cuda_err(c, e, "pd_cylinder_init");
}

int pd_cylinder_get(pd_ctx* c, pd_cylinder* cyl, void* stream) {
    if (!c || !cyl) return PD_ERR_ARG;
    CylDev d;
    cudaError_t e = cudaMemcpyAsync(&d, c->cyl, sizeof(d), cudaMemcpyDeviceToHost, st(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(st(stream));
    if (e != cudaSuccess) return cuda_err(c, e, "pd_cylinder_get");
    cyl->rad = d.rad;
    cyl->mass = d.mass;
    cyl->height = d.height;
    cyl->v = d.v;
    cyl->x = d.x;
    cyl->y = d.y;
    cyl->z = d.z;
    for (int a = 0; a < 3; a++) {
        cyl->vel[a] = d.vel[a];
        cyl->disp[a] = d.disp[a];
        cyl->acc[a] = d.acc[a];
        cyl->force[a] = d.force[a];
    }
    return PD_OK;
}

int pd_cylinder_integrate1(pd_ctx* c, void* stream) {
    if (!c || !c->has_cyl) return PD_ERR_ARG;
    k_cyl_half<<<1, 32, 0, st(stream)>>>(kparams(c->p), c->cyl, 1);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "cy_integrate_1");
}

int pd_cylinder_integrate2(pd_ctx* c, void* stream) {
    if (!c || !c->has_cyl) return PD_ERR_ARG;
    k_cyl_half<<<1, 32, 0, st(stream)>>>(kparams(c->p), c->cyl, 2);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "cy_integrate_2");
}

int pd_contact(pd_ctx* c, void* stream) { return c ? launch_contact(c, st(stream)) : PD_ERR_ARG; }

// ---- fused step loops ------------------------------------------------------
static const int kChunk = 50;

int pd_run_adr(pd_ctx* c, int ct0, int nsteps, double load, void* stream) {
    if (!c || nsteps < 0 || ct0 < 0) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens steps with pd_batch_run_adr");
    if (nsteps == 0) return PD_OK;
    if (c->p.mass == 0.0) return set_err(c, PD_ERR_ARG, "ADR needs the fictitious mass (bond-based parameters)");
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    if ((rc = launch_prologue(c, load, 0, 0, s))) return rc;
    int done = 0;
    auto step = [&](int ct, int last) -> int {
        StepFlags f;
        f.epi = EPI_ADR;
        f.residual = last;  // read after the call (pd_adr_solve); not formed on the other steps
        int r = launch_force(c, f, s);
        if (r) return r;
        return launch_adr_update(c, ct, last ? 0 : 1, load, s);
    };
    if (ct0 == 0) {
        if ((rc = step(0, nsteps == 1))) return rc;
        done = 1;
    }
    while (done < nsteps) {
        const int len = std::min(kChunk, nsteps - done);
        const int final_chunk = done + len == nsteps;
        Key k{1, len, c->parity, final_chunk, load, 0};
        rc = graph_chunk(c, k, s, [&]() -> int {
            for (int t = 0; t < len; t++) {
                int r = step(ct0 + done + t, final_chunk && t == len - 1);
                if (r) return r;
            }
            return PD_OK;
        });
        if (rc) return rc;
        done += len;
    }
    return cuda_err(c, cudaGetLastError(), "pd_run_adr");
}

int pd_run_explicit(pd_ctx* c, int nsteps, double load, int dmg_every, void* stream) {
    if (!c || nsteps < 0 || dmg_every < 0) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens is solved by ADR only");
    if (nsteps == 0) return PD_OK;
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    const bool state = c->p.model == PD_MODEL_STATE;
    const int contact = c->has_cyl ? 1 : 0;
    if (contact && c->p.dim != 3) return set_err(c, PD_ERR_UNSUPPORTED, "contact is 3-D only");
    if ((rc = launch_prologue(c, load, 1, contact, s))) return rc;
    int done = 0;
    const int chunk = dmg_every > 0 ? dmg_every : kChunk;
    while (done < nsteps) {
        const int len = std::min(chunk, nsteps - done);
        const int final_chunk = done + len == nsteps;
        const int dmg_at_end = dmg_every > 0 && ((done + len) % dmg_every == 0);
        Key k{2, len, c->parity, final_chunk | (dmg_at_end << 1), load, dmg_every};
        rc = graph_chunk(c, k, s, [&]() -> int {
            for (int t = 0; t < len; t++) {
                const int last = final_chunk && t == len - 1;
                int r;
                if (state && (r = launch_theta(c, s))) return r;
                StepFlags f;
                f.epi = EPI_VERLET;
                f.do_next = last ? 0 : 1;
                f.load = load;
                f.contact = contact;
                if ((r = launch_force(c, f, s))) return r;
            }
            if (dmg_at_end) return launch_damage(c, s);
            return PD_OK;
        });
        if (rc) return rc;
        done += len;
    }
    return cuda_err(c, cudaGetLastError(), "pd_run_explicit");
}

// ---- quasi-static load stepping ------------------------------------------------
static int residual_now(pd_ctx* c, cudaStream_t s, double* norm) {
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    StepFlags f;
    f.nobreak = 1;
    if (c->p.model == PD_MODEL_STATE && (rc = launch_theta(c, s))) return rc;
    if ((rc = launch_force(c, f, s))) return rc;
    if ((rc = residual_sq(c, c->red_out, s))) return rc;
    double v = 0.0;
    cudaError_t e = cudaMemcpyAsync(&v, c->red_out, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "residual");
    *norm = std::sqrt(v);
    return PD_OK;
}

int pd_residual(pd_ctx* c, double* norm, void* stream) {
    if (!c || !norm) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "residual of a batch: not provided");
    StreamScope sc(c, stream);
    return residual_now(c, sc.s, norm);
}

int pd_adr_solve(pd_ctx* c, int ct0, int max_iters, int check_every, double tol, int* iters, double* norm,
                 void* stream) {
    if (!c || ct0 < 0 || max_iters < 1 || check_every < 1 || !(tol >= 0.0) || !iters || !norm) return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens steps with pd_batch_run_adr");
    int done = 0;
    double r = HUGE_VAL;
    while (done < max_iters) {
        const int len = std::min(check_every, max_iters - done);
        int rc = pd_run_adr(c, ct0 + done, len, 0.0, stream);
        if (rc) return rc;
        done += len;
        double v = 0.0;
        cudaError_t e = cudaMemcpyAsync(&v, c->res, sizeof(double), cudaMemcpyDeviceToHost, st(stream));
        if (e == cudaSuccess) e = cudaStreamSynchronize(st(stream));
        if (e != cudaSuccess) return cuda_err(c, e, "pd_adr_solve");
        r = std::sqrt(v);
        if (!(r > tol)) break;  // also stops on NaN
    }
    *iters = done;
    *norm = r;
    if (!std::isfinite(r)) return set_err(c, PD_ERR_NONFINITE, "ADR residual is not finite");
    return PD_OK;
}

int pd_load_step(pd_ctx* c, double delta, const double* dev_du, int ncand, int probe_iters, double tol_rel,
                 int max_iters, int check_every, pd_load_step_stats* out, void* stream) {
    if (!c || !out || !(tol_rel > 0.0) || max_iters < 1 || check_every < 1 || ncand < 0 || ncand > 8 ||
        (ncand > 0 && !dev_du) || probe_iters < 0 || probe_iters >= max_iters)
        return PD_ERR_ARG;
    if (c->batch.count) return set_err(c, PD_ERR_UNSUPPORTED, "load stepping of a batch: not provided");
    if (c->p.mass == 0.0) return set_err(c, PD_ERR_ARG, "ADR needs the fictitious mass (bond-based parameters)");
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    pd_load_step_stats st{};
    int rc = ensure_ready(c, s);
    const int64_t ni = c->p.N_int;
    double* saved = nullptr;  // [0, 2 ni): previous solution; [2 ni, 8 ni): best probed state
    // the increment: boundary rows move by +-delta (kernel_quick_load), ADR restarts
    if (!rc) rc = launch_quick_load(c, delta / c->p.dt, s);
    const int zero[] = {PD_F_VHX, PD_F_VHY, PD_F_VHZ, PD_F_FOX, PD_F_FOY, PD_F_FOZ};
    auto restart = [&]() -> int {
        for (int k = 0; k < 6; k++) {
            cudaError_t e = cudaMemsetAsync(c->nf[zero[k]], 0, c->p.N * sizeof(double), s);
            if (e != cudaSuccess) return cuda_err(c, e, "ADR restart");
        }
        return PD_OK;
    };
    if (!rc) rc = restart();
    c->pos_valid = false;
    if (!rc) rc = residual_now(c, s, &st.r_plain);
    st.r_start = st.r_plain;
    int ct0 = 0;
    if (!rc && ncand > 0) {
        cudaError_t e = cudaMallocAsync(&saved, 8 * ni * sizeof(double), s);
        rc = cuda_err(c, e, "warm start scratch");
        const int state[] = {PD_F_UX, PD_F_UY, PD_F_VHX, PD_F_VHY, PD_F_FOX, PD_F_FOY};
        auto copy_state = [&](int nfields, double* dst, bool to_ctx) -> int {
            for (int k = 0; k < nfields; k++) {
                double* f = c->nf[state[k]];
                cudaError_t r = to_ctx ? cudaMemcpyAsync(f, dst + k * ni, ni * 8, cudaMemcpyDeviceToDevice, s)
                                       : cudaMemcpyAsync(dst + k * ni, f, ni * 8, cudaMemcpyDeviceToDevice, s);
                if (r != cudaSuccess) return cuda_err(c, r, "warm start state copy");
            }
            c->pos_valid = false;
            return PD_OK;
        };
        if (!rc) rc = copy_state(2, saved, false);
        // rule 1: a candidate is admissible when its start's residual is not
        // larger than the plain start's
        std::vector<int> ok;
        std::vector<double> rw(ncand, HUGE_VAL);
        for (int k = 0; k < ncand && !rc; k++) {
            if (k > 0) rc = copy_state(2, saved, true);
            if (!rc) rc = add_increment(c, dev_du + (int64_t)k * 2 * ni, s);
            if (!rc) rc = residual_now(c, s, &rw[k]);
            if (!rc && rw[k] <= st.r_plain) ok.push_back(k);
        }
        if (!rc && ok.size() == 1) {
            st.warm_used = ok[0] + 1;
        } else if (!rc && ok.size() > 1 && probe_iters == 0) {
            int best = ok[0];
            for (int k : ok)
                if (rw[k] < rw[best]) best = k;
            st.warm_used = best + 1;
        } else if (!rc && ok.size() > 1) {
            // rule 2: among several admissible starts, the one whose residual is
            // lowest after probe_iters ADR steps; its state after the probe is kept
            double best_r = HUGE_VAL;
            for (int k : ok) {
                if ((rc = copy_state(2, saved, true)) || (rc = add_increment(c, dev_du + (int64_t)k * 2 * ni, s)) ||
                    (rc = restart()))
                    break;
                int it = 0;
                double r = 0.0;
                if ((rc = pd_adr_solve(c, 0, probe_iters, probe_iters, 0.0, &it, &r, s))) break;
                st.iters += it;
                st.probes++;
                if (r < best_r) {
                    best_r = r;
                    st.warm_used = k + 1;
                    if ((rc = copy_state(6, saved + 2 * ni, false))) break;
                }
            }
            if (!rc) rc = copy_state(6, saved + 2 * ni, true);
            ct0 = probe_iters;
        }
        if (!rc && st.warm_used > 0) st.r_start = rw[st.warm_used - 1];
        if (!rc && st.probes == 0) {  // bring back the chosen start (or the plain one)
            rc = copy_state(2, saved, true);
            if (!rc && st.warm_used > 0) rc = add_increment(c, dev_du + (int64_t)(st.warm_used - 1) * 2 * ni, s);
        }
    }
    if (saved) cudaFreeAsync(saved, s);
    if (!rc) {
        int it = 0;
        rc = pd_adr_solve(c, ct0, std::max(1, max_iters - st.iters), check_every, tol_rel * st.r_plain, &it,
                          &st.r_final, s);
        st.iters += it;
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    st.ms = ms;
    *out = st;
    return rc;
}

// Batched ADR: the loop of pd_run_adr over every specimen of a batch context,
// three launches per step (force + per-slice damping sums, per-specimen cn,
// update), captured in CUDA graphs of kChunk steps.
int pd_batch_run_adr(pd_ctx* c, int ct0, int nsteps, double load, void* stream) {
    if (!c || nsteps < 0 || ct0 < 0) return PD_ERR_ARG;
    if (!c->batch.count) return set_err(c, PD_ERR_STATE, "not a batch context (pd_batch_create)");
    if (nsteps == 0) return PD_OK;
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    if ((rc = batch_prologue(c, load, s))) return rc;
    int done = 0;
    if (ct0 == 0) {
        if ((rc = batch_step(c, 0, nsteps == 1, load, s))) return rc;
        done = 1;
    }
    while (done < nsteps) {
        const int len = std::min(kChunk, nsteps - done);
        const int final_chunk = done + len == nsteps;
        Key k{3, len, c->parity, final_chunk, load, 0};
        rc = graph_chunk(c, k, s, [&]() -> int {
            for (int t = 0; t < len; t++) {
                int r = batch_step(c, ct0 + done + t, final_chunk && t == len - 1, load, s);
                if (r) return r;
            }
            return PD_OK;
        });
        if (rc) return rc;
        done += len;
    }
    return cuda_err(c, cudaGetLastError(), "pd_batch_run_adr");
}

// The step loops of pd_run_adr / pd_batch_run_adr (kind 0) or pd_run_explicit
// (kind 1) for nsteps steps, launched directly instead of from graphs, with
// CUDA events around every step's force launch(es) and around the whole step.
// The state advances exactly as in those loops.
int pd_profile_steps(pd_ctx* c, int kind, int ct0, int nsteps, double load, double* force_ms, double* step_ms,
                     void* stream) {
    if (!c || (kind != 0 && kind != 1) || nsteps < 1 || nsteps > 10000 || ct0 < 0 || !force_ms || !step_ms)
        return PD_ERR_ARG;
    const bool batch = c->batch.count > 0;
    if (kind == 1 && batch) return set_err(c, PD_ERR_UNSUPPORTED, "a batch of specimens is solved by ADR only");
    if (kind == 0 && !batch && c->p.mass == 0.0) return set_err(c, PD_ERR_ARG, "ADR needs the fictitious mass");
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    const bool state = c->p.model == PD_MODEL_STATE;
    const int contact = c->has_cyl ? 1 : 0;
    if (kind == 1 && contact && c->p.dim != 3) return set_err(c, PD_ERR_UNSUPPORTED, "contact is 3-D only");
    std::vector<cudaEvent_t> ev(3 * (size_t)nsteps, nullptr);
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            for (auto& q : ev)
                if (q) cudaEventDestroy(q);
            return cuda_err(c, cudaGetLastError(), "profile events");
        }
    if (kind == 0)
        rc = batch ? batch_prologue(c, load, s) : launch_prologue(c, load, 0, 0, s);
    else
        rc = launch_prologue(c, load, 1, contact, s);
    for (int t = 0; t < nsteps && !rc; t++) {
        const int last = t == nsteps - 1;
        cudaEventRecord(ev[3 * t], s);
        StepFlags f;
        if (kind == 0) {
            f.epi = EPI_ADR;
            f.residual = last;
            rc = launch_force(c, f, s);
            cudaEventRecord(ev[3 * t + 1], s);
            if (!rc) rc = batch ? batch_finish(c, ct0 + t, last, load, s)
                                : launch_adr_update(c, ct0 + t, last ? 0 : 1, load, s);
        } else {
            if (state) rc = launch_theta(c, s);
            f.epi = EPI_VERLET;
            f.do_next = last ? 0 : 1;
            f.load = load;
            f.contact = contact;
            if (!rc) rc = launch_force(c, f, s);
            cudaEventRecord(ev[3 * t + 1], s);
        }
        cudaEventRecord(ev[3 * t + 2], s);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    double fsum = 0.0, ssum = 0.0;
    for (int t = 0; t < nsteps && !rc && e == cudaSuccess; t++) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, ev[3 * t], ev[3 * t + 1]);
        cudaEventElapsedTime(&b, ev[3 * t], ev[3 * t + 2]);
        fsum += a;
        ssum += b;
    }
    for (auto& q : ev) cudaEventDestroy(q);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(c, e, "pd_profile_steps");
    if (kind == 1) c->csr_fail_current = false;
    *force_ms = fsum / nsteps;
    *step_ms = ssum / nsteps;
    return PD_OK;
}

int pd_set_launch(pd_ctx* c, int block, int chunked, int waves, int split) {
    if (!c || (block != 128 && block != 256 && block != 512) || (chunked != 0 && chunked != 1) || waves < 1 ||
        waves > 8 || (split != 1 && split != 2 && split != 4 && split != 8))
        return PD_ERR_ARG;
    if (split > 1 && (chunked || block / 32 < split || c->p.model != PD_MODEL_BOND))
        return set_err(c, PD_ERR_ARG, "a split slice needs the bond kernel, strided order and block >= 32 split");
    if (block != c->tune_block || chunked != c->tune_chunked || waves != c->tune_waves || split != c->tune_split) {
        drop_graphs(c);  // captured launches carry the old shape
        c->tune_block = block;
        c->tune_chunked = chunked;
        c->tune_waves = waves;
        c->tune_split = split;
    }
    return PD_OK;
}

int pd_set_force_layout(pd_ctx* c, int layout) {
    if (!c || layout < PD_LAYOUT_AUTO || layout > PD_LAYOUT_COMPACT) return PD_ERR_ARG;
    if (layout != c->layout_pref) {
        c->layout_pref = layout;
        if (c->prepared) {
            // the intact flags back to the CSR array, then the SELL arrays go;
            // the next prepare rebuilds them in the requested layout
            int rc = sync_fail_to_csr(c, nullptr);
            if (rc) return rc;
            release_sell(c);
            c->prepared = false;
            c->bits_current = false;
        }
    }
    return PD_OK;
}

int pd_get_force_layout(const pd_ctx* c, int* layout) {
    if (!c || !layout) return PD_ERR_ARG;
    const pdg::Sell& S = c->sell;
    *layout = (S.rec16 || S.srec || S.sk) ? PD_LAYOUT_COMPACT : (S.rec || S.sgeo) ? PD_LAYOUT_RECORDS : PD_LAYOUT_AUTO;
    return PD_OK;
}

int pd_get_launch(const pd_ctx* c, int* block, int* chunked, int* waves, int* split) {
    if (!c || !block || !chunked || !waves || !split) return PD_ERR_ARG;
    *block = c->tune_block;
    *chunked = c->tune_chunked;
    *waves = c->tune_waves;
    *split = c->tune_split;
    return PD_OK;
}

// Times the bond-force kernel at the current displacements for every launch
// shape (block 128/256/512 x strided/chunked slice order x 1/2/4/8 waves of
// resident blocks, and 2 or 4 warps per slice) and keeps the fastest.  The intact flags and forces are
// restored afterwards, so a run continues exactly as it would have.
int pd_autotune(pd_ctx* c, int reps, double* best_ms, void* stream) {
    if (!c || reps < 1) return PD_ERR_ARG;
    if (c->p.model != PD_MODEL_BOND) return set_err(c, PD_ERR_UNSUPPORTED, "the launch shape applies to bond kernels");
    StreamScope sc(c, stream);
    cudaStream_t s = sc.s;
    int rc = ensure_ready(c, s);
    if (rc) return rc;
    const Sell& S = c->sell;
    const int64_t N = c->p.N;
    const size_t nbits = (size_t)std::max<int64_t>(S.F, 1) * 4;
    uint32_t* saved_bits = nullptr;
    double* saved_f = nullptr;
    cudaError_t e;
    if ((e = cudaMallocAsync(&saved_bits, nbits, s)) != cudaSuccess) return cuda_err(c, e, "autotune scratch");
    const int nf = c->p.dim;  // force components saved and restored
    const int fid[3] = {PD_F_FX, PD_F_FY, PD_F_FZ};
    if ((e = cudaMallocAsync(&saved_f, nf * N * sizeof(double), s)) != cudaSuccess) {
        cudaFreeAsync(saved_bits, s);
        return cuda_err(c, e, "autotune scratch");
    }
    cudaMemcpyAsync(saved_bits, S.bits, nbits, cudaMemcpyDeviceToDevice, s);
    for (int a = 0; a < nf; a++)
        cudaMemcpyAsync(saved_f + a * N, c->nf[fid[a]], N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    const bool csr_current = c->csr_fail_current, pos_valid = c->pos_valid;
    const int b0 = c->tune_block, k0 = c->tune_chunked, w0 = c->tune_waves, p0 = c->tune_split;
    StepFlags f;
    f.epi = c->batch.count ? EPI_ADR : EPI_NONE;  // a batch's ADR epilogue writes only per-slice scratch
    // between timed launches a 256 MB write evicts the node arrays from L2, as
    // the update kernel does between the force launches of a real step loop
    const size_t flush_bytes = (size_t)256 << 20;
    void* flush = nullptr;
    if (cudaMallocAsync(&flush, flush_bytes, s) != cudaSuccess) {
        cudaGetLastError();
        flush = nullptr;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 1e300;
    int bb = b0, bk = k0, bw = w0, bp = p0;
    // shapes: block x order x waves with one warp per slice, and block x
    // {2, 4} warps per slice x waves {1, 2}
    struct Shape {
        int block, chunked, waves, split;
    };
    std::vector<Shape> shapes;
    for (int blk : {128, 256, 512})
        for (int ck : {0, 1})
            for (int wv : {1, 2, 4, 8}) shapes.push_back({blk, ck, wv, 1});
    for (int blk : {128, 256, 512})
        for (int sp : {2, 4})
            for (int wv : {1, 2}) shapes.push_back({blk, 0, wv, sp});
    if (c->p.dim == 3 && S.rec16) {
        // the 3-D compact kernel has its own unit order (quarter slices): only
        // block size and waves apply
        std::vector<Shape> kept;
        for (const Shape& sh : shapes)
            if (sh.chunked == 0 && sh.split == 1) kept.push_back(sh);
        shapes.swap(kept);
    }
    for (size_t ish = 0; ish < shapes.size() && !rc; ish++) {
                c->tune_block = shapes[ish].block;
                c->tune_chunked = shapes[ish].chunked;
                c->tune_waves = shapes[ish].waves;
                c->tune_split = shapes[ish].split;
                if ((rc = launch_force(c, f, s))) break;  // warm-up
                double tot = 0.0;
                for (int r = 0; r < reps && !rc; r++) {
                    if (flush) cudaMemsetAsync(flush, r & 0xff, flush_bytes, s);
                    cudaEventRecord(e0, s);
                    rc = launch_force(c, f, s);
                    cudaEventRecord(e1, s);
                    if (rc || (e = cudaEventSynchronize(e1)) != cudaSuccess) {
                        if (!rc) rc = cuda_err(c, e, "autotune timing");
                        break;
                    }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    tot += ms;
                }
                if (rc) break;
                if (tot / reps < best) {
                    best = tot / reps;
                    bb = shapes[ish].block, bk = shapes[ish].chunked, bw = shapes[ish].waves, bp = shapes[ish].split;
                }
            }
    cudaMemcpyAsync(S.bits, saved_bits, nbits, cudaMemcpyDeviceToDevice, s);
    for (int a = 0; a < nf; a++)
        cudaMemcpyAsync(c->nf[fid[a]], saved_f + a * N, N * sizeof(double), cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(saved_bits, s);
    cudaFreeAsync(saved_f, s);
    if (flush) cudaFreeAsync(flush, s);
    e = cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->csr_fail_current = csr_current;
    c->pos_valid = pos_valid;
    c->tune_block = b0, c->tune_chunked = k0, c->tune_waves = w0, c->tune_split = p0;
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(c, e, "pd_autotune");
    if (best_ms) *best_ms = best;
    return pd_set_launch(c, bb, bk, bw, bp);
}

// ---- drivers ----------------------------------------------------------------
static int finish_driver(pd_ctx* c, int64_t n, double* a, double* b, double* cz, double* dmg, pd_result* res,
                         double setup_ms, double loop_ms, int64_t steps) {
    int rc = pd_damage(c, nullptr);
    if (!rc && a) rc = pd_get_field(c, PD_F_UX, a, (size_t)n, nullptr);
    if (!rc && b) rc = pd_get_field(c, PD_F_UY, b, (size_t)n, nullptr);
    if (!rc && cz) rc = pd_get_field(c, PD_F_UZ, cz, (size_t)n, nullptr);
    if (!rc && dmg) rc = pd_get_field(c, PD_F_DMG, dmg, (size_t)n, nullptr);
    if (res) {
        res->N = c->p.N;
        res->N_int = c->p.N_int;
        res->B = c->B;
        res->setup_ms = setup_ms;
        res->loop_ms = loop_ms;
        res->bond_updates_per_s = loop_ms > 0 ? (double)c->B * (double)steps / (loop_ms * 1e-3) : 0.0;
    }
    return rc;
}

struct Timer {
    cudaEvent_t a, b;
    Timer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, 0);
    }
    double stop() {
        cudaEventRecord(b, 0);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        cudaEventRecord(a, 0);
        return ms;
    }
    ~Timer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

#define PD_TRY(x)                  \
    do {                           \
        int _r = (x);              \
        if (_r) {                  \
            pd_destroy(c);         \
            return _r;             \
        }                          \
    } while (0)

int pd_solve_plate_tensile(double dx, int nt, double* ux, double* uy, double* dmg, pd_result* res) {
    // Solve_Plate_Tensile.cu:30-138
    pd_params p;
    const double f_dx = dx > 1.0e-8 ? dx : 0.01;
    int rc = pd_params_derive(&p, 2, PD_MODEL_BOND, PD_MODE_STATIC, 1.0, nt, f_dx, 1.0, 0.01, 1.0, 0.5, 0.0, 200.e9,
                              1. / 3., 7850, 1.0, 0);
    if (rc) return rc;
    pd_ctx* c = pd_create(&p, &rc);
    if (!c) return rc;
    Timer t;
    PD_TRY(pd_coord_plate(c, nullptr));
    PD_TRY(pd_find_neighbor(c, nullptr));
    PD_TRY(pd_surface_correct(c, nullptr));
    PD_TRY(pd_initial_state(c, nullptr));
    PD_TRY(pd_load_plate_tensile(c, nullptr));
    PD_TRY(pd_prepare(c, nullptr));
    const double setup_ms = t.stop();
    PD_TRY(pd_run_adr(c, 0, nt, 0.0, nullptr));
    const double loop_ms = t.stop();
    rc = finish_driver(c, p.N_int, ux, uy, nullptr, dmg, res, setup_ms, loop_ms, nt);
    pd_destroy(c);
    return rc;
}

int pd_solve_plate_crack_grow(double dx, int nt, double* ux, double* uy, double* dmg, pd_result* res) {
    // Solve_Plate_Crack_Grow.cu:167-308
    pd_params p;
    const double f_dx = dx > 1.0e-8 ? dx : 0.0001;
    int rc = pd_params_derive(&p, 2, PD_MODEL_STATE, PD_MODE_DYNAMIC, 1.3367e-8, nt, f_dx, 1.0, 0.0001, 0.05, 0.05,
                              0.0, 192.e9, 0.3, 7850, 0.04472, 0);
    if (rc) return rc;
    p.N += 6 * p.nx;
    pd_ctx* c = pd_create(&p, &rc);
    if (!c) return rc;
    Timer t;
    PD_TRY(pd_coord_plate_crack(c, nullptr));
    PD_TRY(pd_find_neighbor(c, nullptr));
    PD_TRY(pd_initial_state(c, nullptr));
    PD_TRY(pd_set_crack_2d(c, 0.01, 0.0, 0.0, 0.0, nullptr));
    PD_TRY(pd_initial_weight(c, nullptr));  // with vol_Corr in one family pass
    PD_TRY(pd_prepare(c, nullptr));
    const double setup_ms = t.stop();
    PD_TRY(pd_run_explicit(c, nt, 20.0, 0, nullptr));
    const double loop_ms = t.stop();
    rc = finish_driver(c, p.N_int, ux, uy, nullptr, dmg, res, setup_ms, loop_ms, nt);
    pd_destroy(c);
    return rc;
}

int pd_solve_kalthoff_winkler(double dx, int nt, double* ux, double* uy, double* uz, double* dmg, int64_t cap,
                              pd_result* res) {
    // Solve_Kalthoff_Winkler.cu:268-441
    pd_params p;
    const double f_dx = dx > 1.0e-8 ? dx : 0.001;
    int rc = pd_params_derive(&p, 3, PD_MODEL_BOND, PD_MODE_DYNAMIC, 8.7e-8, nt, f_dx, 1.0, 0.001, 0.2, 0.1, 0.009,
                              191.0e9, 0.25, 8000, 0.01, 0);
    if (rc) return rc;
    p.nx++;
    p.ny++;
    p.N = p.nx * p.ny * p.nz;
    pd_cylinder cy{};
    cy.rad = 0.025;
    cy.mass = 1.57;
    cy.v = -32.0;
    cy.height = 0.05;
    cy.x = 0.0;
    cy.y = p.height / 2.0 + cy.height / 2.0 + 0.1 * p.dx;
    cy.z = 0.0;
    cy.vel[1] = cy.v;  // kernel_initial_cylinder
    std::vector<double> x((size_t)p.N), y((size_t)p.N), z((size_t)p.N);
    int64_t n = 0;
    if ((rc = pd_coord_kw(&p, cy.rad, x.data(), y.data(), z.data(), p.N, &n))) return rc;
    p.N = p.N_int = (int32_t)n;
    pd_ctx* c = pd_create(&p, &rc);
    if (!c) return rc;
    Timer t;
    PD_TRY(pd_set_field(c, PD_F_X, x.data(), n, nullptr));
    PD_TRY(pd_set_field(c, PD_F_Y, y.data(), n, nullptr));
    PD_TRY(pd_set_field(c, PD_F_Z, z.data(), n, nullptr));
    PD_TRY(pd_find_neighbor(c, nullptr));
    PD_TRY(pd_surface_correct(c, nullptr));
    PD_TRY(pd_initial_state(c, nullptr));
    PD_TRY(pd_set_crack_kw(c, cy.rad, nullptr));
    PD_TRY(pd_cylinder_init(c, &cy, nullptr));
    PD_TRY(pd_prepare(c, nullptr));
    const double setup_ms = t.stop();
    PD_TRY(pd_run_explicit(c, nt, 0.0, 0, nullptr));
    const double loop_ms = t.stop();
    if (cap < n) {
        pd_destroy(c);
        return PD_ERR_ARG;
    }
    rc = finish_driver(c, n, ux, uy, uz, dmg, res, setup_ms, loop_ms, nt);
    pd_destroy(c);
    return rc;
}

int pd_check_finite(pd_ctx* c, void* stream) {
    if (!c) return PD_ERR_ARG;
    int bad = 0;
    int rc = check_finite(c, st(stream), &bad);
    if (rc) return rc;
    return bad ? set_err(c, PD_ERR_NONFINITE, "NaN or Inf in displacement or force") : PD_OK;
}

int64_t pd_kernel_launches(const pd_ctx* c) { return c ? c->launches : -1; }

int pd_probe_fp64(double* gfma_per_s) { return gfma_per_s ? fp64_probe(gfma_per_s) : PD_ERR_ARG; }

int pd_check_division(const double* dev_n, const double* dev_d, int64_t count, unsigned long long* dev_mismatches,
                      void* stream) {
    return div_check(dev_n, dev_d, count, dev_mismatches, st(stream));
}

}  // extern "C"
