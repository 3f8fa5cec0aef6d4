// Internal declarations of the GB300 peridynamics engine (not part of the C ABI).
//
// Layout in HBM
//   node fields   SoA double arrays of N entries (the reference's BAtom,
//                 Base.cuh:186-225), plus two ping-pong copies of the current
//                 position P = x + u that the force kernels gather.
//   bond family   CSR: rowptr (int64, N+1), NL (int32, B) with ascending rows,
//                 and the reference's per-bond arrays idist, fac, scr, w, e
//                 (double, B) and fail (int32, B) in CSR order.
//   force layout  SELL-32: node rows are grouped into slices of 32 consecutive
//                 rows; slot k of row 32s+l lives at sbase[s] + 32k + l, padded
//                 to the slice's widest row.  One warp owns a slice, so every
//                 per-bond load is a coalesced 32-wide access and the intact
//                 flags of a slot are one 32-bit word (bit l = lane l).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "bondtpl.h"
#include "pd.h"

namespace pdg {

constexpr int kWarp = 32;
constexpr int kForceBlock = 256;       // threads per block in the slice kernels
constexpr int kMaxPartials = 8192;     // block partial sums of one reduction

// Parameters the kernels read, passed by value (graph-capture friendly).
struct KParams {
    int64_t N, N_int;
    int nx, ny, nz, dim, model;
    double dx, emod, dens, pratio, bc, delta, critical_s, vol, dt, mass, K, G, pi, break_ymin;
    double rdens, rmass;  // 1 / dens and 1 / mass, IEEE-rounded (the divisors' reciprocals for div_recip)
};

// n / d rounded to nearest, given y = RN(1/d) (an IEEE division done once per
// divisor).  q1 = RN(n y) corrected once by its residual is a faithful
// quotient; one more correction, q2 = RN(q1 + (n - d q1) y) with the
// residual exact under FMA, is RN(n / d) by Markstein's theorem (P. Markstein,
// IBM J. Res. Develop. 34(1), 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, Newton-Raphson-based division with an FMA): a faithful q and a
// y within 2^-53 relative of 1/d give the correctly rounded quotient.  Five
// FP64 instructions against a full division's sequence, on GB300's slow FP64
// pipe.  Outside the range where the theorem's no-underflow conditions hold
// for certain (|n|, |y| or |q| outside [2^-900, 2^900], zeros, infinities,
// NaNs, or y = 0 for "no reciprocal") the IEEE division is taken, so the
// result is always bit for bit n / d.
__device__ __forceinline__ double div_recip(double n, double d, double y) {
    const double q0 = n * y;
    const unsigned en = ((unsigned)__double2hiint(n) >> 20) & 0x7ffu;
    const unsigned ey = ((unsigned)__double2hiint(y) >> 20) & 0x7ffu;
    const unsigned eq = ((unsigned)__double2hiint(q0) >> 20) & 0x7ffu;
    if ((en - 123u > 1800u) | (ey - 123u > 1800u) | (eq - 123u > 1800u)) return n / d;  // biased 123..1923
    const double q1 = fma(fma(-q0, d, n), y, q0);
    return fma(fma(-q1, d, n), y, q1);
}

// Rigid impactor state kept in device memory (Cylinder, Base.cuh:237-242).
struct CylDev {
    double rad, mass, height, v, x, y, z;
    double vel[3], disp[3], acc[3], force[3];
};

// Per-bond coefficient arrays of the SELL layout.
// Per-slot data of the bond-based kernels, one 48-byte record per slot (three
// 16-byte words, read with three 128-bit loads; the 32 records of a slot row
// are one contiguous 1,536-byte run).
struct alignas(16) BondRec {
    int col;       // neighbour id (self for padding)
    float xf[3];   // reference vector x_c - x_i rounded to float per component (z = 0 in 2-D)
    float2 c0;     // |xf|^2 - l0^2 as a float pair (computed exactly)
    float2 l0;     // l0 as a float pair
    float2 k2;     // 2 vol fac bc scr / l0 times 2^-kexp as a float pair
    double ecrit;  // break threshold on e = L - l0 (s0 l0; +inf: never)
};
static_assert(sizeof(BondRec) == 48, "BondRec is three 16-byte words");

// Per-slot data of the state-based kernels: three 32-byte records per slot in
// three arrays, so that each pass streams only what it reads (the dilatation
// pass StateGeo + StateTheta, the force pass StateGeo + StateForce; one
// 96-byte record read in part was measured to pull whole lines, ~99 B per
// bond for the 64 the pass used).
struct alignas(16) StateGeo {
    int col;      // neighbour id (self for padding)
    float xf[3];  // xi rounded to float per component (z = 0 in 2-D)
    float2 c0;    // |xf|^2 - l0^2 as a float pair (computed exactly)
    float2 l0;    // l0 as a float pair
};
struct alignas(16) StateTheta {
    double xi[3];  // reference vector x_c - x_i (FP64, the dilatation pass's operand; z = 0 in 2-D)
    float2 cth;    // dilatation weight of e times 2^sth_exp, as a float pair
};
struct alignas(16) StateForce {
    float2 c1;     // dilatation coefficient of t times 2^(sn_exp - st_exp), as a float pair
    float2 c2;     // extension coefficient of t times 2^(sn_exp - st_exp), as a float pair
    double ecrit;  // break threshold on e = L - l0 (s0 l0; +inf: never)
    double xiz;    // xi[2] again (the 3-D length's z term in the dilatation order)
};
static_assert(sizeof(StateGeo) == 32 && sizeof(StateTheta) == 32 && sizeof(StateForce) == 32,
              "state records are two 16-byte words each");

// Coefficients of the 2-D state-based bonds of one offset class, at the
// class's reference length l0t, as float pairs carrying the context's
// power-of-two scales: c1 and c2 of the force pass (T = c1 (theta_i/m_i +
// theta_j/m_j) + c2 e (1/m_i + 1/m_j)), cth of the dilatation pass.  They
// depend on the bond length only: c2 on the weight exp(-l0^2/delta^2) and the
// partial-volume factor, c1 and cth on those times l0.  The bond lengths of a
// class differ from l0t by dl, a few ulps, so a bond's coefficient is the
// class's times 1 + g dl, g the logarithmic derivative at l0t (g1 for c1 and
// cth, g2 for c2; checked per slot at set-up to 2^-45).
struct alignas(16) StateTpl {
    float c1h, c1l, c2h, c2l;
    float cth_h, cth_l, g1, g2;
};

struct Sell {
    int64_t nslices = 0;     // ceil(N / 32)
    int64_t S = 0;           // total slots (sum of 32 * width)
    int64_t F = 0;           // total flag words (sum of width)
    int wmax = 0;            // widest slice
    int* width = nullptr;    // [nslices]
    int64_t* base = nullptr; // [nslices] slot offset
    int64_t* fbase = nullptr;// [nslices] flag-word offset
    int* csr = nullptr;      // [S] CSR index of the slot (-1 for padding)
    BondRec* rec = nullptr;  // [S] bond-based: the force kernels' per-slot record
    int kexp = 0;            // power-of-two scale that brings k2 near one
    double kscale = 1.0;     // 2^kexp
    double kscale_inv = 1.0; // 2^-kexp
    StateGeo* sgeo = nullptr;     // [S] state-based: geometry record (both passes)
    StateTheta* sth = nullptr;    // [S] state-based: dilatation-pass record
    StateForce* sfo = nullptr;    // [S] state-based: force-pass record
    float2* e = nullptr;     // [S] state-based: extension (dilatation-pass operand order) as a float pair
    // state-based power-of-two scales that keep the pair arithmetic of the two
    // passes in float range whatever the lattice spacing: theta/m and 1/m are
    // carried times 2^-sn_exp, the dilatation weights times 2^sth_exp, the force
    // pair sums times 2^-st_exp (exact scalings, undone in FP64 per node)
    int sn_exp = 0, sth_exp = 0, st_exp = 0;
    uint32_t* bits = nullptr;// [F] intact flags
    // 2-D bond-based compact layout: a 16-byte record per slot (column, dl and
    // class id, k2 / 2) and one template per lattice offset class; when set,
    // rec is not allocated
    bt::Rec* rec16 = nullptr;  // [S]
    bt::Tpl* tpl = nullptr;    // [ntpl] templates of all specimens
    int ntpl = 0;
    int* inst_tbase = nullptr; // batch: first template of each specimen (null: one specimen)
    // 2-D state-based compact layout: per slot a 16-byte record for the
    // dilatation pass (column, dl and class id, the reference vector's
    // distance from its class's float vector in doubles, per component) and an
    // 8-byte record for the force pass (column, dl and class id); the bond
    // coefficients (functions of the bond length only) live in one StateTpl
    // per class; the extension e of the dilatation pass stays in e;
    // sgeo/sth/sfo are not allocated
    int4* srec = nullptr;       // [S]
    int2* srec8 = nullptr;      // [S]
    StateTpl* stpl = nullptr;   // [ntpl]
    // 3-D state-based compact layout: srec8 and stpl as in 2-D, 3-D class
    // templates, and per slot {kx, ky, kz, flags} for the dilatation pass and
    // {kz, flags} for the force pass (flags bit 0: the bond may break; the 3-D
    // kernels spare bonds with an end below y = -0.04)
    bt::Tpl3* tpl3 = nullptr;   // [ntpl]
    int4* sk = nullptr;         // [S]
    int2* skz = nullptr;        // [S]
    // 3-D state-based compact layout: per slot the dilatation pass's
    // extension and the exact offset of its z component (the length's z term
    // of the force pass, Force_State.cu:272), both as float pairs; per
    // (slice, slot) a word of "may break" bits
    float4* e4 = nullptr;       // [S]
    uint32_t* bbits = nullptr;  // [F]
};

// Layout of the bond-based force path (pd_set_force_layout).
enum ForceLayout { LAYOUT_AUTO = 0, LAYOUT_RECORDS = 1, LAYOUT_COMPACT = 2 };

}  // namespace pdg

// A batch of specimens packed into one context (see batch.cu).
struct BatchInfo {
    int count = 0;                     // number of specimens (0: not a batch)
    int* node_group = nullptr;         // [N] specimen of each node (-1: padding row, no family)
    double* node_bc = nullptr;         // [N] micro-modulus constant of the node's specimen
    double* node_sed = nullptr;        // [N] surface-correction energy density of the node's specimen
    double* node_s0 = nullptr;         // [N] critical stretch of the node's specimen
    double* node_mass = nullptr;       // [N] ADR fictitious mass per node
    double* node_c1 = nullptr;         // [N] 2 dt / mass per node (the update's coefficient, host-computed)
    double* node_rmass = nullptr;      // [N] 1 / mass per node (host-computed, IEEE-rounded)
    double* load_sign = nullptr;       // [N] signed load factor of moving boundary rows, 0 elsewhere
    int* slice_inst = nullptr;         // [nslices] specimen of each slice (-1: none)
    int64_t* inst_slices = nullptr;    // [count + 1] first slice of each specimen's interior
    double* slice_part = nullptr;      // [2 * nslices] per-slice damping sums
    double* inst_cn = nullptr;         // [count] damping coefficient per specimen
    double* inst_nd = nullptr;         // [3 count] 2 - cn dt, 2 + cn dt and 1 / (2 + cn dt) per specimen
    std::vector<int64_t> h_inst_nodes; // host: interior node offset of each specimen (+ total)
    std::vector<int64_t> h_inst_bnd;   // host: boundary node offset of each specimen (+ total)
};

struct GraphEntry {
    int kind, nsteps, parity, flags;
    double load;
    int dmg_every;
    cudaGraphExec_t exec;
    int64_t kernels;
};

struct pd_ctx {
    pd_params p{};
    std::string err;
    int64_t launches = 0;
    int device = 0;
    int num_sms = 0;

    // node fields, indexed by pd_field for ids < PD_F_NN (N doubles each)
    double* nf[PD_F_NN] = {};
    // ping-pong current position P = x + u: x and y interleaved (one 16-byte
    // gather per neighbour), z apart
    double2* posxy[2] = {};
    double* posz[2] = {};
    int parity = 0;          // pos[parity] is current
    bool pos_valid = false;  // pos[parity] == x + u
    int* NN = nullptr;
    float4* node_a = nullptr;  // state-based: {theta/m, 1/m} times 2^-sn_exp, as float pairs
    double* node_b = nullptr;  // state-based: 1/m (IEEE-rounded)

    // CSR bond family
    int64_t B = 0;
    int64_t* rowptr = nullptr;
    int* NL = nullptr;
    double *idist = nullptr, *fac = nullptr, *scr = nullptr, *w = nullptr, *e = nullptr;
    int* fail = nullptr;

    pdg::Sell sell;

    // scratch
    double* partials = nullptr;  // [kMaxPartials * 4]
    unsigned int* ticket = nullptr;
    double* cn = nullptr;        // ADR damping coefficient (device scalar)
    double* red_out = nullptr;   // reduction result (device scalar)
    double* res = nullptr;       // ADR: |F + b|^2 over the free nodes at the last step (device scalar)
    pdg::CylDev* cyl = nullptr;
    bool has_cyl = false;

    // stage flags
    bool family = false, volcorr = false, surfcorr = false, weights = false;
    bool prepared = false;        // SELL arrays match the CSR coefficients
    bool bits_current = false;    // SELL bits are the authoritative fail flags
    bool csr_fail_current = true; // CSR fail array is current

    std::vector<GraphEntry> graphs;
    BatchInfo batch;
    // launch shape of the bond-force kernel (pd_autotune may change it)
    int tune_block = 256;   // threads per block: 128, 256 or 512
    int tune_waves = 1;     // grid = resident blocks x waves
    int tune_chunked = 0;   // 1: contiguous slice runs per warp
    int tune_split = 1;     // warps sharing one slice's slots (2-D bond kernels)
    int layout_pref = pdg::LAYOUT_AUTO;  // bond-based SELL layout requested (pd_set_force_layout)
    double* warm_hist = nullptr;  // [3 N_int] learned warm start: the previous increment's history (pd_warm_record)
};

namespace pdg {

inline KParams kparams(const pd_params& p) {
    KParams k;
    k.N = p.N;
    k.N_int = p.N_int;
    k.nx = p.nx;
    k.ny = p.ny;
    k.nz = p.nz;
    k.dim = p.dim;
    k.model = p.model;
    k.dx = p.dx;
    k.emod = p.emod;
    k.dens = p.dens;
    k.pratio = p.pratio;
    k.bc = p.bc;
    k.delta = p.delta;
    k.critical_s = p.critical_s;
    k.vol = p.vol;
    k.dt = p.dt;
    k.mass = p.mass;
    k.K = p.K;
    k.G = p.G;
    k.pi = p.pi;
    k.break_ymin = p.break_ymin;
    k.rdens = 1.0 / p.dens;
    k.rmass = 1.0 / p.mass;
    return k;
}

int set_err(pd_ctx* c, int status, const std::string& msg);
int cuda_err(pd_ctx* c, cudaError_t e, const char* what);
inline cudaStream_t st(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// neighbour.cu
int build_family(pd_ctx* c, cudaStream_t s);
// setup.cu
int vol_corr(pd_ctx* c, cudaStream_t s);
int surface_correct(pd_ctx* c, cudaStream_t s);
int initial_weight(pd_ctx* c, cudaStream_t s);
int set_crack_2d(pd_ctx* c, double clength, double lx, double ly, double theta, cudaStream_t s);
// the same segment test on rows [r0, r1) only
int set_crack_2d_rows(pd_ctx* c, int64_t r0, int64_t r1, double clength, double lx, double ly, double theta,
                      cudaStream_t s);
int set_crack_kw(pd_ctx* c, double rad, cudaStream_t s);
int prepare(pd_ctx* c, cudaStream_t s);
int sync_fail_to_csr(pd_ctx* c, cudaStream_t s);
int sync_fail_to_bits(pd_ctx* c, cudaStream_t s);
// force.cu
enum Epi { EPI_NONE = 0, EPI_VERLET = 1, EPI_ADR = 2 };
struct StepFlags {
    int epi = EPI_NONE;
    int do_next = 0;      // apply the next step's loading + first Verlet half
    double load = 0.0;    // boundary-row speed of the next step (quick_load)
    int contact = 0;      // rigid impactor contact in the epilogue
    int nobreak = 0;      // leave the intact flags unchanged (residual evaluations)
    int residual = 1;     // ADR: also reduce |F + b|^2 (the convergence checks read the last step's)
};
int launch_force(pd_ctx* c, const StepFlags& f, cudaStream_t s);
int launch_theta(pd_ctx* c, cudaStream_t s);
// integrate.cu
int refresh_pos(pd_ctx* c, cudaStream_t s);
int launch_prologue(pd_ctx* c, double load, int first_verlet, int cyl_step, cudaStream_t s);
int launch_adr_update(pd_ctx* c, int ct, int do_next, double load, cudaStream_t s);
int launch_adr_cnn(pd_ctx* c, cudaStream_t s);
int launch_verlet1(pd_ctx* c, cudaStream_t s);
int launch_verlet2(pd_ctx* c, cudaStream_t s);
int launch_damage(pd_ctx* c, cudaStream_t s);
int launch_quick_load(pd_ctx* c, double load, cudaStream_t s);
int launch_load_tensile(pd_ctx* c, cudaStream_t s);
void release_sell(pd_ctx* c);
// Destroy the cached step graphs (they hold device pointers and parameters).
void drop_graphs(pd_ctx* c);
int launch_contact(pd_ctx* c, cudaStream_t s);
int launch_cyl_integrate(pd_ctx* c, int half, cudaStream_t s);
int reduce_sum(pd_ctx* c, const double* x, int64_t n, double* out_dev, cudaStream_t s);
int check_finite(pd_ctx* c, cudaStream_t s, int* bad_host);
// |F + b|^2 summed over the free nodes [0, N_int) into *out_dev (current forces)
int residual_sq(pd_ctx* c, double* out_dev, cudaStream_t s);
// u += du on the free nodes (du on the device: N_int x components, then N_int y)
int add_increment(pd_ctx* c, const double* du, cudaStream_t s);
// Bond coefficients, intact bits and positions current (the run loops' entry check).
int make_ready(pd_ctx* c, cudaStream_t s);
int fp64_probe(double* gfma_per_s);
int div_check(const double* n, const double* d, int64_t count, unsigned long long* mismatches, cudaStream_t s);
// batch.cu
void release_batch(pd_ctx* c);
int batch_prologue(pd_ctx* c, double load, cudaStream_t s);
int batch_step(pd_ctx* c, int ct, int last, double load, cudaStream_t s);
int batch_force(pd_ctx* c, cudaStream_t s);  // first phase of batch_step
int batch_finish(pd_ctx* c, int ct, int last, double load, cudaStream_t s);  // the rest

}  // namespace pdg
