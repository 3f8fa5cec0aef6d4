// Output: the reference's text writers, binary snapshots of the simulation
// state (checkpoint / resume), and the crack-tip position.
//
//   pd_write_disp_txt / pd_save_disp   save_disp_gpu / save_disp_cpu (Save.cu:6-60)
//   pd_write_kw_txt / pd_save_kw       save_kw_gpu / save_kw_cpu (Save.cu:62-140)
//   pd_snapshot_save / _load           no reference counterpart (text only there)
//   pd_crack_tip                       the tracker the crack-plate driver carries
//                                      commented out (Solve_Plate_Crack_Grow.cu:150-162)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pd_internal.cuh"

namespace pdg {
namespace {

// Broken bonds from the SELL intact bits: slots of the family (csr >= 0)
// whose bit is clear; one warp per slice, one atomic per warp.
__global__ void k_count_broken_bits(int64_t nslices, const int* __restrict__ width, const int64_t* __restrict__ base,
                                    const int64_t* __restrict__ fbase, const int* __restrict__ csr,
                                    const uint32_t* __restrict__ bits, unsigned long long* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < nslices;
         s += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        unsigned cnt = 0;
        const int W = width[s];
        for (int k = 0; k < W; k++) {
            const bool valid = csr[base[s] + (int64_t)k * 32 + lane] >= 0;
            const bool alive = (bits[fbase[s] + k] >> lane) & 1u;
            cnt += __popc(__ballot_sync(0xffffffffu, valid && !alive));
        }
        if (lane == 0 && cnt) atomicAdd(out, (unsigned long long)cnt);
    }
}

// Broken bonds from the CSR flags (fail == 0).
__global__ void k_count_broken_csr(int64_t B, const int* __restrict__ fail, unsigned long long* __restrict__ out) {
    unsigned cnt = 0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < B; q += (int64_t)gridDim.x * blockDim.x)
        cnt += fail[q] == 0;
    for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, (unsigned long long)cnt);
}

// std::ostream << double with the default format: %g with precision 6.
void put(FILE* f, double v) { std::fprintf(f, "%g", v); }

struct File {
    FILE* f;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

constexpr char kMagic[8] = {'P', 'D', 'G', 'B', '3', '0', '0', 'S'};
constexpr uint32_t kVersion = 1;

struct SnapHeader {
    char magic[8];
    uint32_t version;
    int32_t dim, model, has_cyl;
    int64_t N, N_int, B;
    double cn;
    CylDev cyl;
};

// Node fields a snapshot carries, in file order (the state of both loops;
// coordinates, family and coefficients come from the set-up).
const int kSnapFields[] = {PD_F_UX,  PD_F_UY,  PD_F_UZ,  PD_F_VX,  PD_F_VY,  PD_F_VZ,  PD_F_AX,  PD_F_AY,
                           PD_F_AZ,  PD_F_FX,  PD_F_FY,  PD_F_FZ,  PD_F_BX,  PD_F_BY,  PD_F_BZ,  PD_F_VHX,
                           PD_F_VHY, PD_F_VHZ, PD_F_FOX, PD_F_FOY, PD_F_FOZ, PD_F_DMG, PD_F_THETA};

// Order-preserving map of a double onto an unsigned 64-bit key.
__device__ __forceinline__ unsigned long long ordered(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Pass 1: the largest x among interior nodes with dmg > threshold.
__global__ void k_tip_max(const double* __restrict__ x, const double* __restrict__ dmg, int64_t n, double thr,
                          unsigned long long* key) {
    unsigned long long best = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (dmg[i] > thr) {
            const unsigned long long k = ordered(x[i]);
            best = k > best ? k : best;
        }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, best, off);
        best = o > best ? o : best;
    }
    if ((threadIdx.x & 31) == 0 && best) atomicMax(key, best);
}

// Pass 2: the lowest node index at that x (a deterministic choice among ties).
__global__ void k_tip_index(const double* __restrict__ x, const double* __restrict__ dmg, int64_t n, double thr,
                            const unsigned long long* key, unsigned long long* idx) {
    const unsigned long long k = *key;
    if (!k) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (dmg[i] > thr && ordered(x[i]) == k) atomicMin(idx, (unsigned long long)i);
}

}  // namespace
}  // namespace pdg

using namespace pdg;

extern "C" {

int pd_write_disp_txt(const char* path, int64_t n, const double* ux, const double* uy, const double* uz,
                      const double* dmg) {
    if (!path || n < 0 || !ux || !uy || !dmg) return PD_ERR_ARG;
    File f(path, "w");
    if (!f.f) return PD_ERR_ARG;
    for (int64_t i = 0; i < n; i++) {
        put(f.f, ux[i]);
        std::fputc(' ', f.f);
        put(f.f, uy[i]);
        std::fputc(' ', f.f);
        if (uz) {
            put(f.f, uz[i]);
            std::fputc(' ', f.f);
        }
        put(f.f, dmg[i]);
        std::fputc('\n', f.f);
    }
    return std::ferror(f.f) ? PD_ERR_ARG : PD_OK;
}

int pd_write_kw_txt(const char* path, const pd_params* p, double rad, int64_t n, const double* ux, const double* uy,
                    const double* uz, const double* dmg) {
    if (!path || !p || !ux || !uy || !uz || !dmg || n < 0) return PD_ERR_ARG;
    File f(path, "w");
    if (!f.f) return PD_ERR_ARG;
    int64_t num = 0;  // the first z layer: save_kw starts at z_num = 0
    for (int j = 0; j < p->ny; j++)
        for (int i = 0; i < p->nx; i++) {
            const double tx = (-(p->nx - 1) / 2.0 + i) * p->dx;
            const double ty = (-(p->ny - 1) / 2.0 + j) * p->dx;
            const bool notch = (tx > (-rad - 1.1 * p->dx) && tx < (-rad + 0.1 * p->dx)) ||
                               (tx > (rad - 0.1 * p->dx) && tx < (rad + 1.1 * p->dx));
            if (notch && ty >= -1.0e-10) {
                std::fputs("nan nan 0 nan\n", f.f);
                continue;
            }
            if (num >= n) return PD_ERR_ARG;
            put(f.f, ux[num]);
            std::fputc(' ', f.f);
            put(f.f, uy[num]);
            std::fputc(' ', f.f);
            put(f.f, uz[num]);
            std::fputc(' ', f.f);
            put(f.f, dmg[num]);
            std::fputc('\n', f.f);
            num++;
        }
    return std::ferror(f.f) ? PD_ERR_ARG : PD_OK;
}

int pd_save_disp(pd_ctx* c, const char* path, void* stream) {
    if (!c || !path) return PD_ERR_ARG;
    const int64_t n = c->p.N_int;
    std::vector<double> ux(n), uy(n), uz(c->p.dim == 3 ? n : 0), dmg(n);
    int rc;
    if ((rc = pd_get_field(c, PD_F_UX, ux.data(), n, stream)) || (rc = pd_get_field(c, PD_F_UY, uy.data(), n, stream)) ||
        (c->p.dim == 3 && (rc = pd_get_field(c, PD_F_UZ, uz.data(), n, stream))) ||
        (rc = pd_get_field(c, PD_F_DMG, dmg.data(), n, stream)))
        return rc;
    rc = pd_write_disp_txt(path, n, ux.data(), uy.data(), c->p.dim == 3 ? uz.data() : nullptr, dmg.data());
    return rc ? set_err(c, rc, std::string("cannot write ") + path) : PD_OK;
}

int pd_save_kw(pd_ctx* c, double rad, const char* path, void* stream) {
    if (!c || !path || c->p.dim != 3) return PD_ERR_ARG;
    const int64_t n = c->p.N_int;
    std::vector<double> ux(n), uy(n), uz(n), dmg(n);
    int rc;
    if ((rc = pd_get_field(c, PD_F_UX, ux.data(), n, stream)) || (rc = pd_get_field(c, PD_F_UY, uy.data(), n, stream)) ||
        (rc = pd_get_field(c, PD_F_UZ, uz.data(), n, stream)) || (rc = pd_get_field(c, PD_F_DMG, dmg.data(), n, stream)))
        return rc;
    rc = pd_write_kw_txt(path, &c->p, rad, n, ux.data(), uy.data(), uz.data(), dmg.data());
    return rc ? set_err(c, rc, std::string("cannot write ") + path) : PD_OK;
}

int pd_snapshot_save(pd_ctx* c, const char* path, void* stream) {
    if (!c || !path) return PD_ERR_ARG;
    if (!c->family) return set_err(c, PD_ERR_STATE, "snapshot needs the bond family");
    SnapHeader h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.dim = c->p.dim;
    h.model = c->p.model;
    h.has_cyl = c->has_cyl;
    h.N = c->p.N;
    h.N_int = c->p.N_int;
    h.B = c->B;
    cudaStream_t s = st(stream);
    cudaError_t e = cudaMemcpyAsync(&h.cn, c->cn, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h.cyl, c->cyl, sizeof(CylDev), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_snapshot_save");
    File f(path, "wb");
    if (!f.f) return set_err(c, PD_ERR_ARG, std::string("cannot open ") + path);
    std::fwrite(&h, sizeof(h), 1, f.f);
    std::vector<double> buf((size_t)h.N);
    int rc;
    for (int fld : kSnapFields) {
        if ((rc = pd_get_field(c, fld, buf.data(), h.N, stream))) return rc;
        std::fwrite(buf.data(), sizeof(double), h.N, f.f);
    }
    std::vector<int32_t> fail((size_t)std::max<int64_t>(h.B, 1));
    if ((rc = pd_get_field(c, PD_F_FAIL, fail.data(), h.B, stream))) return rc;
    std::fwrite(fail.data(), sizeof(int32_t), h.B, f.f);
    return std::ferror(f.f) ? set_err(c, PD_ERR_ARG, std::string("cannot write ") + path) : PD_OK;
}

int pd_snapshot_load(pd_ctx* c, const char* path, void* stream) {
    if (!c || !path) return PD_ERR_ARG;
    if (!c->family) return set_err(c, PD_ERR_STATE, "load the snapshot after the same set-up (family)");
    File f(path, "rb");
    if (!f.f) return set_err(c, PD_ERR_ARG, std::string("cannot open ") + path);
    SnapHeader h{};
    if (std::fread(&h, sizeof(h), 1, f.f) != 1 || std::memcmp(h.magic, kMagic, 8) || h.version != kVersion)
        return set_err(c, PD_ERR_ARG, "not a snapshot of this format");
    if (h.N != c->p.N || h.N_int != c->p.N_int || h.B != c->B || h.dim != c->p.dim || h.model != c->p.model)
        return set_err(c, PD_ERR_ARG, "snapshot of a different problem (N, N_int, B, dim or model)");
    std::vector<double> buf((size_t)h.N);
    int rc;
    for (int fld : kSnapFields) {
        if (std::fread(buf.data(), sizeof(double), h.N, f.f) != (size_t)h.N)
            return set_err(c, PD_ERR_ARG, "truncated snapshot");
        if ((rc = pd_set_field(c, fld, buf.data(), h.N, stream))) return rc;
    }
    std::vector<int32_t> fail((size_t)std::max<int64_t>(h.B, 1));
    if (std::fread(fail.data(), sizeof(int32_t), h.B, f.f) != (size_t)h.B)
        return set_err(c, PD_ERR_ARG, "truncated snapshot");
    if ((rc = pd_set_field(c, PD_F_FAIL, fail.data(), h.B, stream))) return rc;
    cudaStream_t s = st(stream);
    cudaError_t e = cudaMemcpyAsync(c->cn, &h.cn, sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && h.has_cyl) {
        e = cudaMemcpyAsync(c->cyl, &h.cyl, sizeof(CylDev), cudaMemcpyHostToDevice, s);
        if (!c->has_cyl) drop_graphs(c);  // captured loops without the impactor
        c->has_cyl = true;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    c->pos_valid = false;
    return cuda_err(c, e, "pd_snapshot_load");
}

int pd_count_broken(pd_ctx* c, int64_t* count, void* stream) {
    if (!c || !count) return PD_ERR_ARG;
    *count = 0;
    if (!c->family || c->B == 0) return PD_OK;
    cudaStream_t s = st(stream);
    unsigned long long* w = reinterpret_cast<unsigned long long*>(c->partials);
    cudaError_t e = cudaMemsetAsync(w, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_count_broken");
    const Sell& S = c->sell;
    if (c->bits_current && S.bits) {
        const unsigned g = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((S.nslices * 32 + 255) / 256, (int64_t)c->num_sms * 16));
        k_count_broken_bits<<<g, 256, 0, s>>>(S.nslices, S.width, S.base, S.fbase, S.csr, S.bits, w);
    } else {
        const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((c->B + 255) / 256, (int64_t)c->num_sms * 16));
        k_count_broken_csr<<<g, 256, 0, s>>>(c->B, c->fail, w);
    }
    c->launches++;
    unsigned long long out = 0;
    e = cudaMemcpyAsync(&out, w, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_count_broken");
    *count = (int64_t)out;
    return PD_OK;
}

int pd_crack_tip(pd_ctx* c, double threshold, double* tip_xy, void* stream) {
    if (!c || !tip_xy) return PD_ERR_ARG;
    cudaStream_t s = st(stream);
    unsigned long long* w = reinterpret_cast<unsigned long long*>(c->partials);
    const unsigned long long init[2] = {0ull, ~0ull};
    cudaError_t e = cudaMemcpyAsync(w, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_crack_tip");
    const int64_t n = c->p.N_int;
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)c->num_sms * 8));
    k_tip_max<<<g, 256, 0, s>>>(c->nf[PD_F_X], c->nf[PD_F_DMG], n, threshold, w);
    k_tip_index<<<g, 256, 0, s>>>(c->nf[PD_F_X], c->nf[PD_F_DMG], n, threshold, w, w + 1);
    c->launches += 2;
    unsigned long long out[2];
    e = cudaMemcpyAsync(out, w, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "pd_crack_tip");
    if (!out[0]) {  // no damaged node
        tip_xy[0] = tip_xy[1] = NAN;
        return PD_OK;
    }
    const int64_t i = (int64_t)out[1];
    e = cudaMemcpyAsync(&tip_xy[0], c->nf[PD_F_X] + i, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tip_xy[1], c->nf[PD_F_Y] + i, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_err(c, e, "pd_crack_tip");
}

}  // extern "C"
