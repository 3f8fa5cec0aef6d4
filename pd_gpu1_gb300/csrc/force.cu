// Force kernels: bond-based PMB and ordinary state-based, 2-D and 3-D.
//
// Replaces kernel_particle_force_2D / kernel_bond_force_2D / kernel_bond_force_3D
// (Force_Bond.cu:6-141) and kernel_cal_theta_2D/3D + kernel_state_force_2D/3D
// (Force_State.cu:56-306).
//
// Mapping: one warp per SELL slice (32 consecutive node rows), lane l owns row
// 32s+l and walks its bond slots k = 0..width-1 (k_bond_force, k_state_force);
// for small or 3-D problems several warps share a slice (k_bond_split,
// k_bond_split3) and the first adds their parts in the one-warp order.  Slot
// loads are 32-wide coalesced: a bond-based slot is one 48-byte BondRec
// (three 128-bit loads), and the 32 records of a slot row are contiguous.  On
// the regular lattices of the reference's drivers slot k of every interior
// row points at the same lattice offset, so the neighbour gathers are
// coalesced as well.  The intact flags of a slot are one 32-bit word, read
// once per warp and rewritten with a ballot when bonds break.  Forces are
// summed per lane in registers (no shuffles).
//
// GB300's FP64 pipe issues about 1/64 of the FP32 rate, so each bond costs as
// few FP64 instructions as parity allows.  Bond-based (bond3): the bond vector
// d = (P_c - x_i) - u_i with the reference's roundings (P = x + u kept per
// node, so d rounds exactly as x_c + u_c - x_i - u_i), 2 FP64 instructions
// per component; its offset eta = d - xf from the per-slot float reference
// vector exactly on the integer pipe; L^2 - l0^2 = c0 + 2 xf.eta + eta.eta,
// 1/L, e = L - l0 and the force t (xf + eta) in pair-of-floats arithmetic
// (ff.cuh); the break test e > s0 l0 decided on the pair, the double sum only
// near the threshold.  State-based (k_theta, k_state_force): the same
// stretch arithmetic on three 32-byte records per slot, with the bond vector in
// the dilatation pass's operand order ((x_c - x_i) + u_c) - u_i for theta and
// the force pass's (P_c - x_i) - u_i for the force, as the reference rounds
// them; e, the theta sum and t_i + t_j in pairs (the node quantities theta/m
// and 1/m as power-of-two-scaled pairs).
//
// Epilogues fused into the same launch (one launch per explicit step):
//   EPI_VERLET  a = (F+b)/rho; v += dt/2 a (kernel_integrate_2D_2, Integrate.cu:218-249),
//               optional rigid-impactor contact (kernel_contact,
//               Solve_Kalthoff_Winkler.cu:112-175) and, when do_next is set, the
//               next step's boundary loading (kernel_quick_load,
//               Solve_Plate_Crack_Grow.cu:8-19) and first Verlet half
//               (kernel_integrate_2D_1, Integrate.cu:174-185) into the other
//               position buffer.
//   EPI_ADR     per-node damping numerator/denominator (kernel_cnn,
//               Integrate.cu:7-49) reduced across the grid; the last block to
//               finish forms the damping coefficient (cal_cn, :108-129) on the
//               device, so ADR needs no host round trip.
#include "exact_sub.h"
#include "ff.cuh"
#include "pd_internal.cuh"

namespace pdg {

struct ForceArgs {
    KParams P;
    int64_t nslices;  // slices processed (covering [0, N) for boundary epilogues)
    int64_t nforce;   // rows [0, nforce) get forces
    const int* width;
    const int64_t* base;
    const int64_t* fbase;
    const BondRec* rec;  // bond-based: per-slot record (column, float reference vector, c0, l0, k2, ecrit)
    int kexp;           // sums of bond forces carry 2^-kexp (undone in the conversion to FP64)
    const StateGeo* sgeo;    // state-based: per-slot geometry (column, float reference vector, c0, l0)
    const StateTheta* sth;   // state-based: dilatation-pass record (xi, cth)
    const StateForce* sfo;   // state-based: force-pass record (c1, c2, ecrit, xi_z)
    float2* e;                // state: extension per slot as a float pair
    double sn_scale;          // state: 2^-sn_exp (theta/m and 1/m pairs)
    int sth_exp;              // state: the dilatation sums carry 2^sth_exp
    int st_exp;               // state: the force pair sums carry 2^-st_exp
    uint32_t* bits;
    int64_t S;
    const int* NN;
    const double *x, *y, *z;
    double *ux, *uy, *uz;
    const double2* pc;  // current positions, x and y interleaved
    const double* pcz;
    double2* pn;        // next positions (the other ping-pong buffer)
    double* pnz;
    double *fx, *fy, *fz;
    double *vx, *vy, *vz;
    double *ax, *ay, *az;
    const double *bx, *by, *bz;
    const double *fox, *foy, *foz;
    const double *vhx, *vhy, *vhz;
    // state: per node {theta/m, 1/m} times 2^-sn_exp as float pairs (one
    // 16-byte gather per bond in the force pass); the dilatation pass writes
    // the first pair, the set-up the second
    float4* nab;
    const double* nb;   // state: 1/m (IEEE-rounded)
    const double* m;
    double* theta;
    const double* dmg;
    int epi, do_next, contact, first_step;
    double load;
    CylDev* cyl;
    double* partials;
    unsigned int* ticket;
    double* cn_out;
    int chunked;              // contiguous slice runs per warp instead of a grid stride
    int split;                // warps sharing one slice (k_bond_split)
    int wmax;                 // widest slice
    int nobreak;              // evaluate forces without updating the intact flags
    double* res_out;          // ADR: sum over force rows of |F + b|^2 (device scalar)
    // batch of specimens (null for a single one)
    const double* node_mass;  // ADR fictitious mass per node
    const double* node_rmass; // 1 / node_mass (IEEE-rounded)
    double* slice_part;       // per-slice damping sums (2 per slice) instead of a grid reduction
    // 2-D bond-based compact layout (null: the 48-byte records)
    const bt::Rec* rec16;     // per-slot record: column, dl and class id, k2 / 2
    const bt::Tpl* tpl;       // offset-class templates
    int ntpl;
    const int* inst_tbase;    // batch: first template of each specimen (null: one specimen)
    const int* slice_inst;    // batch: specimen of each slice
    const double* node_s0;    // batch: critical stretch per node (null: P.critical_s)
    // 2-D state-based compact layout (null: the three 32-byte records)
    const int4* srec;         // dilatation pass: column, dl and class id, kx, ky
    const int2* srec8;        // force pass: column, dl and class id
    const StateTpl* stpl;     // per class: c1, c2, cth as pairs
    // 3-D state-based compact layout (srec8 and stpl as above)
    const bt::Tpl3* tpl3;     // 3-D class templates
    const int4* sk;           // dilatation pass: kx, ky, kz, flags
    float4* e4;               // per slot: e and the exact z offset of the dilatation-order bond vector
    const uint32_t* bbits;    // per (slice, slot): "may break" bits
};

namespace {

constexpr int kWarpsPerBlock = kForceBlock / 32;
constexpr int kMaxBondBlock = 512;  // the bond kernels take any block size up to this
// The bond kernels are compiled for two resident 512-thread blocks per SM (64
// registers a thread, 32 warps an SM).  Left alone the compiler takes 111
// registers for the fused 3-D Verlet + contact epilogue and the SM holds 18
// warps, too few to cover the neighbour gathers (measured on the 180,873-node
// impact slab: 0.90 ms per step uncapped, 0.70 ms capped, a few spilled bytes
// outside the slot loop); the 2-D kernels fit 64 without spilling.
constexpr int kBondMinBlocks = 2;
// The state-force kernel likewise at four resident 256-thread blocks (64
// registers): the 3-D instance drops from 70 registers, +6 % on the
// Kalthoff-Winkler slab (1.52 -> 1.44 ms per step); the 2-D one is unchanged.
constexpr int kStateMinBlocks = 4;
constexpr int kMaxWarpsPerBlock = kMaxBondBlock / 32;
// P_c - x_i by integer operations (exact_sub.h) instead of an FP64 subtraction.
// Measured slower on the 1.6M-node plate (1.01 ms against 0.85 ms per step):
// the normalisation of the difference costs more issue slots than the FP64
// instruction it replaces.
constexpr bool kIntExactA = false;

// diff * 2^(e - 1075) as a normalized pair; exact for |diff| < 2^48 and a
// scale within the float range (the caller checks both).  h is zero or a
// multiple of 2^24 sc and 0 <= l < 2^24 sc, so |h| >= |l| whenever h != 0 and
// the fast two-sum gives the exact pair (the same one as the full two-sum).
__device__ __forceinline__ ff ff_from_scaled(int64_t diff, int e) {
    const float sc = __int_as_float((e - 1075 + 127) << 23);
    const float h = __int2float_rn((int)(diff >> 24)) * (sc * 16777216.0f);
    const float l = __int2float_rn((int)(diff & 0xffffff)) * sc;
    return ff_fast(h, l);
}

__device__ __forceinline__ uint64_t dbits(double v) { return (uint64_t)__double_as_longlong(v); }

// eta = d - xf exactly, as a pair, for a rounded bond-vector component d and
// its per-slot float reference xf (d - xf is exact by Sterbenz's lemma; it is
// formed on the integer pipe and falls back to FP64 outside the usual range).
// bond_offset (below) forms d = (P_c - x_i) - u_i with the reference's
// roundings first, the rounding subtraction in FP64.
__device__ __forceinline__ ff exact_offset(double d, float xf) {
    if (xf == 0.0f) return ff_split(d);
    const double x = f64_of_f32s(xf);
    // usual case: d and x of the same sign and binade (eta is the small
    // displacement-induced offset), where the difference of the bit patterns is
    // the difference of the mantissas -- the value sub_exact_scaled forms, with
    // two integer instructions instead of the exponent alignment
    {
        const long long bd = __double_as_longlong(d), bx = __double_as_longlong(x);
        const int hd = (int)(bd >> 32), hx = (int)(bx >> 32);
        const int eb = (hd >> 20) & 0x7ff;
        long long df = bd - bx;
        if (hd < 0) df = -df;
        if (((hd ^ hx) & (int)0xfff00000) == 0 && eb >= 949 && eb <= 1170 && df < (1ll << 48) && df > -(1ll << 48))
            return ff_from_scaled(df, eb);
    }
    int64_t diff;
    int e;
    if (sub_exact_scaled(dbits(d), dbits(x), diff, e) && e >= 949 && e <= 1170 && diff < (1ll << 48) &&
        diff > -(1ll << 48))
        return ff_from_scaled(diff, e);
    return ff_split(d - x);
}

__device__ __forceinline__ ff bond_offset(double pc, double xi, double ui, float xf) {
    double a;
    if (kIntExactA) {
        uint64_t ua;
        if (sub_exact(dbits(pc), dbits(xi), ua))
            a = __longlong_as_double((long long)ua);
        else
            a = pc - xi;
    } else {
        a = pc - xi;
    }
    return exact_offset(a - ui, xf);
}

// e > ecrit for ecrit > 0: ordered like the IEEE bit patterns read as signed
// integers (a negative e has its sign bit set and compares below).  Integer
// compare keeps the test off the FP64 pipe.
__device__ __forceinline__ bool exceeds(double e, double ecrit) {
    return __double_as_longlong(e) > __double_as_longlong(ecrit);
}

// fl(h + l) > ecrit for a pair e = h + l (h = fl(h + l)) and a double ecrit >
// 0, without the FP64 addition where the float h alone decides: with t =
// ecrit truncated to float (t <= ecrit < next(t)), h at or above the second
// float after t gives h + l >= next(t) > ecrit, and h below t gives
// h + l <= t <= ecrit (|l| <= ulp(h) / 2; positive floats order like their
// bit patterns, negative ones lie below).  Otherwise, and for thresholds
// outside the float range, the double test decides as before.
__device__ __forceinline__ bool pair_exceeds(ff e, double ecrit) {
    const unsigned hi = (unsigned)__double2hiint(ecrit), lo = (unsigned)__double2loint(ecrit);
    const unsigned E = hi >> 20;  // biased exponent (ecrit > 0)
    if (E >= 1151u) return false;  // ecrit >= 2^128 (+inf: never breaks) exceeds every pair
    if (E >= 897u) {
        const int tb = (int)((((hi - (896u << 20)) << 3) | (lo >> 29)));
        const int hb = __float_as_int(e.h);
        if (hb >= tb + 2) return true;
        if (hb < tb) return false;
    }
    return exceeds(f64_of_f32s(e.h) + f64_of_f32s(e.l), ecrit);
}

__device__ __forceinline__ double block_sum(double v, double* sm) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sm[k];
    return r;  // valid in thread 0
}

// Per-node contact with the rigid cylinder (Solve_Kalthoff_Winkler.cu:112-175).
// Returns the node's reaction-force contribution in rf.
__device__ __forceinline__ void contact_node(const KParams& P, const CylDev& cy, double xi, double yi, double zi,
                                             double& ux, double& uy, double& uz, double& vx, double& vy, double& vz,
                                             double rf[3]) {
    const double dpenx = xi + ux - cy.x - cy.disp[0];
    const double dpeny = yi + uy - cy.y - cy.disp[1];
    const double dpenz = zi + uz - cy.z - cy.disp[2];
    const double dpend = sqrt(dpenx * dpenx + dpenz * dpenz);
    if (dpend <= cy.rad && fabs(dpeny) <= (cy.height / 2.0)) {
        double dprx, dpry, dprz;
        if (cy.rad - dpend <= cy.height / 2.0 - fabs(dpeny)) {
            dprx = dpenx / dpend * cy.rad;
            dpry = dpeny;
            dprz = dpenz / dpend * cy.rad;
        } else if (dpeny >= 0.0) {
            dprx = dpenx;
            dpry = cy.height / 2.0;
            dprz = dpenz;
        } else {
            dprx = dpenx;
            dpry = -cy.height / 2.0;
            dprz = dpenz;
        }
        const double oux = ux, ouy = uy, ouz = uz, ovx = vx, ovy = vy, ovz = vz;
        ux = cy.x + cy.disp[0] + dprx - xi;
        uy = cy.y + cy.disp[1] + dpry - yi;
        uz = cy.z + cy.disp[2] + dprz - zi;
        vx = (ux - oux) / P.dt;
        vy = (uy - ouy) / P.dt;
        vz = (uz - ouz) / P.dt;
        rf[0] += -P.dens * (vx - ovx) / P.dt * P.vol;
        rf[1] += -P.dens * (vy - ovy) / P.dt * P.vol;
        rf[2] += -P.dens * (vz - ovz) / P.dt * P.vol;
    }
}

// The ADR damping terms (kernel_cnn) through reciprocals: bt::damping_term
// (bondtpl.h, checked on the host against quadruple precision).
using bt::damping_term;

// v != 0.0 on the integer pipe (+0 and -0 compare equal to zero, NaN does not).
__device__ __forceinline__ bool nonzero(double v) { return (__double_as_longlong(v) << 1) != 0; }

// Epilogue of one force-computed row r (r < nforce).
template <int DIM, int EPI>
__device__ __forceinline__ void row_epilogue(const ForceArgs& A, int64_t r, double fxr, double fyr, double fzr,
                                             double xi, double yi, double zi, double uxi, double uyi, double uzi,
                                             double red[3]) {
    const KParams& P = A.P;
    A.fx[r] = fxr;
    A.fy[r] = fyr;
    if (DIM == 3) A.fz[r] = fzr;
    if (EPI == EPI_ADR) {
        // kernel_cnn (Integrate.cu:17-33) through damping_term; a batch of
        // specimens carries its fictitious mass per node.
        const double rmass = A.node_mass ? A.node_rmass[r] : P.rmass;
        const double vhx = A.vhx[r], vhy = A.vhy[r];
        double cn = 0.0, disp;
        if (nonzero(vhx)) cn = damping_term(uxi, fxr, A.fox[r], rmass, P.dt, vhx);
        disp = uxi * uxi;
        if (nonzero(vhy)) cn += damping_term(uyi, fyr, A.foy[r], rmass, P.dt, vhy);
        disp += uyi * uyi;
        if (DIM == 3) {
            const double vhz = A.vhz[r];
            if (nonzero(vhz)) cn += damping_term(uzi, fzr, A.foz[r], rmass, P.dt, vhz);
            disp += uzi * uzi;
        }
        red[0] += cn;
        red[1] += disp;
        if (A.res_out) {
            // residual of the iterate: |F + b|^2 over the force rows (free nodes)
            const double rx = fxr + A.bx[r], ry = fyr + A.by[r];
            double rr = rx * rx + ry * ry;
            if (DIM == 3) {
                const double rz = fzr + A.bz[r];
                rr += rz * rz;
            }
            red[2] += rr;
        }
        return;
    }
    if (EPI == EPI_VERLET) {
        double vx = A.vx[r], vy = A.vy[r], vz = DIM == 3 ? A.vz[r] : 0.0;
        double ux = uxi, uy = uyi, uz = uzi;
        if (DIM == 3 && A.contact && A.dmg[r] < 1.0) contact_node(P, *A.cyl, xi, yi, zi, ux, uy, uz, vx, vy, vz, red);
        const double hdt = P.dt / 2.0;
        // a = (F + b) / rho through rho's reciprocal (div_recip: bit for bit the quotient)
        const double ax = div_recip(fxr + A.bx[r], P.dens, P.rdens);
        const double ay = div_recip(fyr + A.by[r], P.dens, P.rdens);
        vx = fma(hdt, ax, vx);
        vy = fma(hdt, ay, vy);
        A.ax[r] = ax;
        A.ay[r] = ay;
        double az = 0.0;
        if (DIM == 3) {
            az = div_recip(fzr + A.bz[r], P.dens, P.rdens);
            vz = fma(hdt, az, vz);
            A.az[r] = az;
        }
        if (A.do_next) {
            vx = fma(hdt, ax, vx);
            vy = fma(hdt, ay, vy);
            ux = fma(vx, P.dt, ux);
            uy = fma(vy, P.dt, uy);
            if (DIM == 3) {
                vz = fma(hdt, az, vz);
                uz = fma(vz, P.dt, uz);
            }
        }
        A.vx[r] = vx;
        A.vy[r] = vy;
        if (DIM == 3) A.vz[r] = vz;
        if (A.do_next || A.contact) {
            A.ux[r] = ux;
            A.uy[r] = uy;
            if (DIM == 3) A.uz[r] = uz;
        }
        if (A.do_next) {
            A.pn[r] = make_double2(xi + ux, yi + uy);
            if (DIM == 3) A.pnz[r] = zi + uz;
        }
    }
}

// Batch of specimens: the damping sums of one slice (one specimen's rows)
// reduced over the warp in a fixed order and stored per slice.
__device__ __forceinline__ void slice_partials(const ForceArgs& A, int64_t s, double red[3]) {
    double a = red[0], b = red[1];
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        A.slice_part[2 * s] = a;
        A.slice_part[2 * s + 1] = b;
    }
    red[0] = red[1] = red[2] = 0.0;
}

// Boundary rows [N_int, N): the next step's prescribed motion
// (kernel_quick_load: the first 3 nx rows move up, the next 3 nx down).
template <int DIM>
__device__ __forceinline__ void boundary_row(const ForceArgs& A, int64_t r) {
    const KParams& P = A.P;
    double uy = A.uy[r];
    if (A.load != 0.0) {
        const int64_t k = r - P.N_int;
        if (k < 3 * (int64_t)P.nx)
            uy += A.load * P.dt;
        else if (k < 6 * (int64_t)P.nx)
            uy -= A.load * P.dt;
        A.uy[r] = uy;
    }
    A.pn[r] = make_double2(A.pc[r].x, A.y[r] + uy);
    if (DIM == 3) A.pnz[r] = A.pcz[r];
}

// Grid-level reduction of red[0..nred) into partials; the last block to finish
// forms the result (ADR damping or contact reaction + cylinder update).
// mode: EPI_ADR -> damping coefficient; EPI_VERLET -> contact reaction and
// impactor update; EPI_NONE -> contact reaction accumulated only.
template <int EPI>
__device__ void finish_reduction(const ForceArgs& A, double red[3], int nred) {
    __shared__ double sm[kMaxWarpsPerBlock];
    __shared__ bool last;
    for (int k = 0; k < nred; k++) {
        const double v = block_sum(red[k], sm);
        if (threadIdx.x == 0) A.partials[(int64_t)blockIdx.x * 4 + k] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(A.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    double tot[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < nred; k++) {
        double v = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(A.partials + (int64_t)b * 4 + k);
        tot[k] = block_sum(v, sm);
    }
    if (threadIdx.x != 0) return;
    *A.ticket = 0u;
    const KParams& P = A.P;
    if (EPI == EPI_ADR) {
        // cal_cn (Integrate.cu:108-129)
        const double cn1 = tot[0], cn2 = tot[1];
        double cn = 0.0;
        if (cn2 != 0.0) cn = (cn1 / cn2 > 0.0) ? 2.0 * sqrt(cn1 / cn2) : 0.0;
        if (cn > 2.0) cn = 1.9;
        *A.cn_out = cn;
        if (A.res_out) *A.res_out = tot[2];
    } else if (EPI == EPI_NONE) {
        for (int a = 0; a < 3; a++) A.cyl->force[a] += tot[a];
    } else {
        // kernel_cy_integrate_2 (Solve_Kalthoff_Winkler.cu:242-253), then the
        // next step's kernel_cy_integrate_1 (:89-99)
        CylDev& cy = *A.cyl;
        for (int a = 0; a < 3; a++) {
            cy.force[a] = tot[a];
            cy.acc[a] = cy.force[a] / cy.mass;
            cy.vel[a] = fma(P.dt / 2.0, cy.acc[a], cy.vel[a]);
            cy.force[a] = 0.0;
            if (A.do_next) {
                cy.vel[a] = fma(P.dt / 2.0, cy.acc[a], cy.vel[a]);
                cy.disp[a] = fma(cy.vel[a], P.dt, cy.disp[a]);
            }
        }
    }
}

// The three 16-byte words of a slot's BondRec: q0 = {col, xf[0..2]},
// q1 = {c0, l0}, q2 = {k2, ecrit}.
__device__ __forceinline__ int4 rec_q0(const BondRec* r, int64_t slot) {
    return __ldg(reinterpret_cast<const int4*>(r + slot));
}
__device__ __forceinline__ float4 rec_q1(const BondRec* r, int64_t slot) {
    return __ldg(reinterpret_cast<const float4*>(r + slot) + 1);
}
__device__ __forceinline__ float4 rec_q2(const BondRec* r, int64_t slot) {
    return __ldg(reinterpret_cast<const float4*>(r + slot) + 2);
}

// From the exact offsets eta of a bond vector from its float reference xf
// (per component) and the slot's c0 = |xf|^2 - l0^2 and l0 (pairs): the bond
// vector xf + eta (dp), 1/L (y) and e = L - l0 (e2), all as pairs.
//   L^2 - l0^2 = c0 + 2 xf.eta + eta.eta has no cancellation;
//   e = (L^2 - l0^2) / (L + l0).
template <int DIM>
__device__ __forceinline__ void pair_stretch(const ff eta[3], const float xf[3], float2 c0, float2 l0, ff dp[3],
                                             ff& y, ff& e2) {
    ff D, Q;
#pragma unroll
    for (int a = 0; a < DIM; a++) {
        // the first terms are taken as they are: ff_add of a zero pair and a
        // pair that ff_fast produced returns that pair unchanged
        D = a == 0 ? ff_mul_f(eta[a], xf[a]) : ff_add(D, ff_mul_f(eta[a], xf[a]));
        Q = a == 0 ? ff_sq(eta[a]) : ff_add(Q, ff_sq(eta[a]));
        dp[a] = ff_add_f(xf[a], eta[a]);
    }
    D = ff_add(ff_add(ff{c0.x, c0.y}, ff{2.0f * D.h, 2.0f * D.l}), Q);  // L^2 - l0^2
    const ff L0p{l0.x, l0.y};
    const ff L2p = ff_add(ff_sq(L0p), D);
    y = ff_rsqrt(L2p);                                     // 1/L
    e2 = ff_mul(D, ff_rcp(ff_add(ff_mul(L2p, y), L0p)));  // L - l0
}

// One bond: its force contribution t (xf + eta) per component as pairs (cf)
// and whether it breaks.
//   d = (P_c - x_i) - u_i with the reference's roundings (FP64),
//   eta = d - xf exactly (integer pipe), then everything in pairs.
// q0..q2: the slot's record words (the neighbour id is q0.x).
template <int DIM>
__device__ __forceinline__ bool bond3(const ForceArgs& A, int4 q0, float4 q1, float4 q2, double xi, double yi,
                                      double zi, double uxi, double uyi, double uzi, ff cf[3]) {
    const int c = q0.x;
    const double2 pxy = __ldg(A.pc + c);
    const double pc[3] = {pxy.x, pxy.y, DIM == 3 ? __ldg(A.pcz + c) : 0.0};
    const double xr[3] = {xi, yi, zi}, ur[3] = {uxi, uyi, uzi};
    const float xfs[3] = {__int_as_float(q0.y), __int_as_float(q0.z), __int_as_float(q0.w)};
    ff eta[3], dp[3], y, e2;
#pragma unroll
    for (int a = 0; a < DIM; a++) eta[a] = bond_offset(pc[a], xr[a], ur[a], xfs[a]);
    pair_stretch<DIM>(eta, xfs, make_float2(q1.x, q1.y), make_float2(q1.z, q1.w), dp, y, e2);
    const ff t = ff_mul(ff_mul(ff{q2.x, q2.y}, e2), ff{0.5f * y.h, 0.5f * y.l});
#pragma unroll
    for (int a = 0; a < DIM; a++) cf[a] = ff_mul(t, dp[a]);
    // the break test in double against the double s0 l0: a threshold held as a
    // pair (48 bits) moves near-threshold breaks by a step and, over a long
    // fracture run, the crack path with them
    return pair_exceeds(e2, __hiloint2double(__float_as_int(q2.w), __float_as_int(q2.z)));
}

// Record words of the 32-byte state records (16 bytes each).
template <typename R>
__device__ __forceinline__ float4 srec_w(const R* r, int64_t slot, int w) {
    return __ldg(reinterpret_cast<const float4*>(r + slot) + w);
}
__device__ __forceinline__ double lo_f64(float4 v) { return __hiloint2double(__float_as_int(v.y), __float_as_int(v.x)); }
__device__ __forceinline__ double hi_f64(float4 v) { return __hiloint2double(__float_as_int(v.w), __float_as_int(v.z)); }

template <int DIM, int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kBondMinBlocks) k_bond_force(const ForceArgs A) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    // warp -> slice mapping: strided over the grid, or one contiguous run of
    // slices per warp (the autotuner chooses; the per-lane sums are the same)
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    int64_t s_begin = w, s_end = A.nslices, s_step = nwarps;
    if (A.chunked) {
        const int64_t per = (A.nslices + nwarps - 1) / nwarps;
        s_begin = w * per;
        s_end = s_begin + per < A.nslices ? s_begin + per : A.nslices;
        s_step = 1;
    }
    for (int64_t s = s_begin; s < s_end; s += s_step) {
        const int64_t r = s * 32 + lane;
        const bool force_row = r < A.nforce;
        if (s * 32 < A.nforce) {
            const int64_t rr = force_row ? r : A.nforce - 1;
            const double xi = A.x[rr], yi = A.y[rr], zi = DIM == 3 ? A.z[rr] : 0.0;
            const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = DIM == 3 ? A.uz[rr] : 0.0;
            double fxr = 0.0, fyr = 0.0, fzr = 0.0;
            ff fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
            ff bxa{0.0f, 0.0f}, bya{0.0f, 0.0f}, bza{0.0f, 0.0f};  // 3-D: sums of the current 32-slot block
            const int W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            // the first record word of the next slot (neighbour id and float
            // reference vector) loaded one iteration ahead, so the gather of
            // slot k starts at the top of iteration k
            // (prefetching the whole next record as well was measured slower: the
            // twelve registers spill under the 64-register cap)
            int4 q0_next = W > 0 ? rec_q0(A.rec, b + lane) : make_int4(0, 0, 0, 0);
            for (int k = 0; k < W; k++) {
                const int64_t slot = b + (int64_t)k * 32 + lane;
                const int4 q0 = q0_next;
                if (k + 1 < W) q0_next = rec_q0(A.rec, slot + 32);
                const float4 q1 = rec_q1(A.rec, slot), q2 = rec_q2(A.rec, slot);
                const uint32_t word = wbits[k];
                const bool alive = force_row && ((word >> lane) & 1u);
                bool brk = false;
                if (alive) {
                    ff cf[3];
                    brk = bond3<DIM>(A, q0, q1, q2, xi, yi, zi, uxi, uyi, uzi, cf);
                    if (DIM == 3) {
                        bxa = ff_add(bxa, cf[0]);
                        bya = ff_add(bya, cf[1]);
                        bza = ff_add(bza, cf[2]);
                    } else {
                        fxa = ff_add(fxa, cf[0]);
                        fya = ff_add(fya, cf[1]);
                    }
                }
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
                if (DIM == 3 && ((k & 31) == 31 || k + 1 == W)) {
                    // a 3-D row is summed in blocks of 32 slots, each from zero, the
                    // block sums in block order: the order k_bond_split3 keeps
                    fxa = ff_add(fxa, bxa);
                    fya = ff_add(fya, bya);
                    fza = ff_add(fza, bza);
                    bxa = bya = bza = ff{0.0f, 0.0f};
                }
            }
            // undo the power-of-two scaling of the bond coefficient (exact)
            fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
            fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
            if (DIM == 3) fzr = f64_of_pair_scaled(fza.h, fza.l, A.kexp);
            if (force_row) row_epilogue<DIM, EPI>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
            if (EPI == EPI_ADR && A.slice_part) slice_partials(A, s, red);
        }
        if (EPI == EPI_VERLET && A.do_next && !force_row && r < P.N) boundary_row<DIM>(A, r);
    }
    if (EPI == EPI_ADR && !A.slice_part) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// 2-D bond force with several warps per slice (A.split of them): warp `sub`
// of a slice group computes the slots k = sub, sub + split, ... and leaves
// each contribution in shared memory; the group's first warp then adds them
// in slot order, so every row's sums are the same, bit for bit, as with one
// warp per slice.  For small problems (fewer slices than the GPU has warp
// slots) the split multiplies the bonds in flight.  Shared memory per group:
// wmax slots x 2 components x 32 lanes pairs + one alive word per slot.
template <int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kBondMinBlocks) k_bond_split(const ForceArgs A) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int split = A.split, G = (int)(blockDim.x >> 5) / split;
    const int g = wib / split, sub = wib % split;
    const int Wm = A.wmax;
    float2* contrib = reinterpret_cast<float2*>(sm_raw) + (size_t)g * Wm * 64;
    uint32_t* alive_w = reinterpret_cast<uint32_t*>(reinterpret_cast<float2*>(sm_raw) + (size_t)G * Wm * 64) + g * Wm;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const int64_t groups = (int64_t)gridDim.x * G;
    const int64_t rounds = (A.nslices + groups - 1) / groups;
    for (int64_t it = 0; it < rounds; it++) {
        const int64_t s = it * groups + (int64_t)blockIdx.x * G + g;
        const int64_t r = s * 32 + lane;
        const bool in = s < A.nslices;
        const bool force_row = in && r < A.nforce;
        const bool work = in && s * 32 < A.nforce;
        const int64_t rr = force_row ? r : (A.nforce > 0 ? A.nforce - 1 : 0);
        double xi = 0.0, yi = 0.0, uxi = 0.0, uyi = 0.0;
        int W = 0;
        if (work) {
            xi = A.x[rr], yi = A.y[rr], uxi = A.ux[rr], uyi = A.uy[rr];
            W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            for (int k = sub; k < W; k += split) {
                const int64_t slot = b + (int64_t)k * 32 + lane;
                const uint32_t word = wbits[k];
                const bool alive = force_row && ((word >> lane) & 1u);
                bool brk = false;
                ff cf[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
                if (alive)
                    brk = bond3<2>(A, rec_q0(A.rec, slot), rec_q1(A.rec, slot), rec_q2(A.rec, slot), xi, yi, 0.0, uxi,
                                   uyi, 0.0, cf);
                contrib[(k * 2 + 0) * 32 + lane] = make_float2(cf[0].h, cf[0].l);
                contrib[(k * 2 + 1) * 32 + lane] = make_float2(cf[1].h, cf[1].l);
                const uint32_t am = __ballot_sync(0xffffffffu, alive);
                if (lane == 0) alive_w[k] = am;
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
            }
        }
        __syncthreads();
        if (sub == 0 && work) {
            ff fxa{0.0f, 0.0f}, fya{0.0f, 0.0f};
            for (int k = 0; k < W; k++) {
                if (!((alive_w[k] >> lane) & 1u)) continue;
                const float2 cx = contrib[(k * 2 + 0) * 32 + lane], cy = contrib[(k * 2 + 1) * 32 + lane];
                fxa = ff_add(fxa, ff{cx.x, cx.y});
                fya = ff_add(fya, ff{cy.x, cy.y});
            }
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
            if (force_row) row_epilogue<2, EPI>(A, r, fxr, fyr, 0.0, xi, yi, 0.0, uxi, uyi, 0.0, red);
            if (EPI == EPI_ADR && A.slice_part) slice_partials(A, s, red);
        }
        if (sub == 0 && EPI == EPI_VERLET && A.do_next && in && !force_row && r < P.N) boundary_row<2>(A, r);
        __syncthreads();
    }
    if (EPI == EPI_ADR && !A.slice_part) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// ---- 2-D bond force on the compact layout ----------------------------------
//
// Per slot one 16-byte record (column; dl = l0 - l0t with the offset class id
// in its low byte; k2 / 2 as a pair) and the class's template (bondtpl.h: the
// float reference vector, |xf|^2, c0, l0t), read through the read-only cache:
// a specimen has a few dozen classes, and on a regular lattice the 32 lanes
// of a slot read the same one.  The bond arithmetic is bt::bond2; the break
// test bt::exceeds decides on floats away from the threshold and on the double
// test near it.

// The templates of slice s's specimen.
__device__ __forceinline__ const bt::Tpl* slice_templates(const ForceArgs& A, int64_t s) {
    return A.inst_tbase ? A.tpl + A.inst_tbase[A.slice_inst[s]] : A.tpl;
}

// One bond of the compact layout: its force contribution (pairs, times
// 2^-kexp) and whether it breaks.
__device__ __forceinline__ bool bond_compact_p(const bt::Tpl* __restrict__ tpls, int4 rq, double pcx, double pcy,
                                               double xi, double yi, double uxi, double uyi, double s0, float s0f,
                                               bt::f2 cf[2]) {
    const uint32_t dlb = (uint32_t)rq.y;
    const bt::Tpl& T = tpls[dlb & 0xffu];
    const float dl = __uint_as_float(dlb & ~0xffu);
    const double pc[2] = {pcx, pcy};
    const double xr[2] = {xi, yi}, ur[2] = {uxi, uyi};
    bt::f2 eta[2];
#pragma unroll
    for (int a = 0; a < 2; a++) {
        // d = (P_c - x_i) - u_i with the reference's roundings, then its exact
        // offset from the class's float reference vector
        const double d = (pc[a] - xr[a]) - ur[a];
        const uint64_t xb = T.xd[a];
        if (xb == 0)
            eta[a] = bt::split_bits(d);
        else if (!bt::offset_pair(d, xb, eta[a]))
            eta[a] = bt::split_bits(d - bt::dfrom(xb));  // exact by Sterbenz's lemma
    }
    const bt::BondOut o = bt::bond2(eta, T, dl, bt::f2{__int_as_float(rq.z), __int_as_float(rq.w)});
    cf[0] = o.f[0];
    cf[1] = o.f[1];
    return bt::exceeds(o.e, s0, s0f, T, dl);
}
__device__ __forceinline__ bool bond_compact(const ForceArgs& A, const bt::Tpl* __restrict__ tpls, int4 rq, double xi,
                                             double yi, double uxi, double uyi, double s0, float s0f, bt::f2 cf[2]) {
    const double2 pxy = __ldg(A.pc + rq.x);
    return bond_compact_p(tpls, rq, pxy.x, pxy.y, xi, yi, uxi, uyi, s0, s0f, cf);
}

// The compact kernel's software pipeline: records two slots ahead and the
// neighbour positions one slot ahead (true), or records one slot ahead and
// the positions gathered in the slot's own iteration (false).
constexpr bool kGatherAhead = false;

// The templates are read through the read-only cache: staged in shared memory
// instead (one specimen, a few dozen classes) the kernel was measured twice as
// slow on the 1.6M-node plate (1.00 against 0.49 ms per launch).
// Resident 512-thread blocks per SM the compact kernel is compiled for (the
// register cap: 2 -> 64 registers a thread).
constexpr int kCompactMinBlocks = 2;
template <int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kCompactMinBlocks) k_bond_compact(const ForceArgs A) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    int64_t s_begin = w, s_end = A.nslices, s_step = nwarps;
    if (A.chunked) {
        const int64_t per = (A.nslices + nwarps - 1) / nwarps;
        s_begin = w * per;
        s_end = s_begin + per < A.nslices ? s_begin + per : A.nslices;
        s_step = 1;
    }
    for (int64_t s = s_begin; s < s_end; s += s_step) {
        const int64_t r = s * 32 + lane;
        const bool force_row = r < A.nforce;
        if (s * 32 < A.nforce) {
            const int64_t rr = force_row ? r : A.nforce - 1;
            const double xi = A.x[rr], yi = A.y[rr];
            const double uxi = A.ux[rr], uyi = A.uy[rr];
            const double s0 = A.node_s0 ? A.node_s0[rr] : P.critical_s;
            const float s0f = __double2float_rn(s0);
            const bt::Tpl* tpls = slice_templates(A, s);
            bt::f2 fxa{0.0f, 0.0f}, fya{0.0f, 0.0f};
            const int W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            // the next slot's record loaded one iteration ahead, so that its
            // neighbour gathers can start as soon as the iteration does
            const int4* rp = reinterpret_cast<const int4*>(A.rec16 + b) + lane;
            if (kGatherAhead) {
                const int4 z4 = make_int4(0, 0, 0, 0);
                int4 rq_a = W > 0 ? __ldg(rp) : z4, rq_b = W > 1 ? __ldg(rp + 32) : z4;
                const double2 g0 = W > 0 ? __ldg(A.pc + rq_a.x) : make_double2(0.0, 0.0);
                double gx = g0.x, gy = g0.y;
                for (int k = 0; k < W; k++) {
                    const int4 rq = rq_a;
                    const double pcx = gx, pcy = gy;
                    rq_a = rq_b;
                    if (k + 2 < W) rq_b = __ldg(rp + (int64_t)(k + 2) * 32);
                    if (k + 1 < W) {
                        const double2 g1 = __ldg(A.pc + rq_a.x);
                        gx = g1.x;
                        gy = g1.y;
                    }
                    const uint32_t word = wbits[k];
                    const bool alive = force_row && ((word >> lane) & 1u);
                    bool brk = false;
                    if (alive) {
                        bt::f2 cf[2];
                        brk = bond_compact_p(tpls, rq, pcx, pcy, xi, yi, uxi, uyi, s0, s0f, cf);
                        bt::acc_add(fxa, cf[0]);
                        bt::acc_add(fya, cf[1]);
                    }
                    const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                    if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
                }
            } else {
                int4 rq_next = W > 0 ? __ldg(rp) : make_int4(0, 0, 0, 0);
                for (int k = 0; k < W; k++) {
                    const int4 rq = rq_next;
                    if (k + 1 < W) rq_next = __ldg(rp + (int64_t)(k + 1) * 32);
                    const uint32_t word = wbits[k];
                    const bool alive = force_row && ((word >> lane) & 1u);
                    bool brk = false;
                    if (alive) {
                        bt::f2 cf[2];
                        brk = bond_compact(A, tpls, rq, xi, yi, uxi, uyi, s0, s0f, cf);
                        bt::acc_add(fxa, cf[0]);
                        bt::acc_add(fya, cf[1]);
                    }
                    const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                    if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
                }
            }
            // undo the power-of-two scaling of the bond coefficient (exact)
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
            if (force_row) row_epilogue<2, EPI>(A, r, fxr, fyr, 0.0, xi, yi, 0.0, uxi, uyi, 0.0, red);
            if (EPI == EPI_ADR && A.slice_part) slice_partials(A, s, red);
        }
        if (EPI == EPI_VERLET && A.do_next && !force_row && r < P.N) boundary_row<2>(A, r);
    }
    if (EPI == EPI_ADR && !A.slice_part) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// Pair sums of a row spread over Q lane groups (lane j + R p, R = 32 / Q),
// added as a lane tree: pair addition is commutative, so every lane of the
// row gets the same sum.
template <int Q>
__device__ __forceinline__ bt::f2 phase_sum(bt::f2 v) {
#pragma unroll
    for (int off = 32 / Q; off < 32; off <<= 1)
        v = bt::add(v, bt::f2{__shfl_xor_sync(0xffffffffu, v.h, off), __shfl_xor_sync(0xffffffffu, v.l, off)});
    return v;
}

// d - x exactly as a pair, x the double value of a float (bit pattern xb).
__device__ __forceinline__ bt::f2 offset1(double d, uint64_t xb) {
    bt::f2 eta;
    if (xb == 0)
        eta = bt::split_bits(d);
    else if (!bt::offset_pair(d, xb, eta))
        eta = bt::split_bits(d - bt::dfrom(xb));  // exact by Sterbenz's lemma
    return eta;
}
// One bond's exact offsets from its class's float reference vector.
template <int N, class TT>
__device__ __forceinline__ void offsets_n(const TT& T, const double* d, bt::f2* eta) {
#pragma unroll
    for (int a = 0; a < N; a++) eta[a] = offset1(d[a], T.xd[a]);
}

// The 3-D bond force (kernel_bond_force_3D, Force_Bond.cu:87-141) on the
// compact layout: one 16-byte record per slot (k2 / 2 negated where the
// bond may not break, the y >= -0.04 guard of Force_Bond.cu:117) and 80-byte
// class templates; the bond vector with the reference's roundings (6 FP64
// instructions), the stretch in pairs (bt::stretch3).  Work units of 32 / Q
// rows with Q slot phases, as k_state_compact3; the sum order depends on Q
// only (not on block size, waves or slice order).  Measured on the impact
// slab (ms per step, the autotuner's shape): Q = 1: 0.361, 2: 0.379, 4: 0.440,
// 8: 0.552; the 48-byte records: 0.385.  So one warp per slice here.
constexpr int kBondPhases3 = 1;
template <int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kCompactMinBlocks) k_bond_compact3(const ForceArgs A) {
    constexpr int Q = kBondPhases3, R = 32 / Q;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int j = lane % R, ph = lane / R;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const double s0 = P.critical_s;
    const float s0f = __double2float_rn(s0);
    const int64_t units = A.nslices * Q;
    for (int64_t u = (int64_t)blockIdx.x * wpb + wib; u < units; u += (int64_t)gridDim.x * wpb) {
        const int64_t s = u / Q;
        const int h = (int)(u - s * Q);
        const int rl = h * R + j;
        const int64_t r = s * 32 + rl;
        const bool force_row = r < A.nforce;
        if (s * 32 + h * R < A.nforce) {  // warp-uniform: the unit holds a force row
            const int64_t rr = force_row ? r : A.nforce - 1;
            const double xi = A.x[rr], yi = A.y[rr], zi = A.z[rr];
            const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = A.uz[rr];
            bt::f2 fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
            const int W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            const int4* rp = reinterpret_cast<const int4*>(A.rec16 + b) + rl;
            const int iters = (W + Q - 1) / Q;
            // the lane's next slot's record loaded one iteration ahead
            int4 rq_next = ph < W ? __ldg(rp + (int64_t)ph * 32) : make_int4(0, 0, 0, 0);
            for (int i = 0; i < iters; i++) {
                const int k = i * Q + ph;
                const int4 rq = rq_next;
                if (k + Q < W) rq_next = __ldg(rp + (int64_t)(k + Q) * 32);
                const uint32_t word = k < W ? wbits[k] : 0u;
                const bool alive = force_row && ((word >> rl) & 1u);
                bool brk = false;
                if (alive) {
                    const int c = rq.x;
                    const uint32_t dlb = (uint32_t)rq.y;
                    const bt::Tpl3& T = A.tpl3[dlb & 0xffu];
                    const float dl = __uint_as_float(dlb & ~0xffu);
                    // d = (P_c - x_i) - u_i with the reference's roundings
                    const double2 pxy = __ldg(A.pc + c);
                    const double d[3] = {(pxy.x - xi) - uxi, (pxy.y - yi) - uyi, (__ldg(A.pcz + c) - zi) - uzi};
                    bt::f2 eta[3], w[3], y, e;
                    offsets_n<3>(T, d, eta);
                    bt::stretch3(eta, T, dl, w, y, e);
                    const bool spared = __int_as_float(rq.z) < 0.0f;
                    const bt::f2 k2half = spared ? bt::f2{-__int_as_float(rq.z), -__int_as_float(rq.w)}
                                                 : bt::f2{__int_as_float(rq.z), __int_as_float(rq.w)};
                    // t = (k2 / 2) e / L, f = t W
                    const bt::f2 t = bt::mul(bt::mul(k2half, e), y);
                    bt::acc_add(fxa, bt::mul(t, w[0]));
                    bt::acc_add(fya, bt::mul(t, w[1]));
                    bt::acc_add(fza, bt::mul(t, w[2]));
                    brk = !spared && bt::exceeds(e, s0, s0f, T, dl);
                }
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (broke && j == 0 && !A.nobreak) {
                    constexpr uint32_t kRows = R >= 32 ? 0xffffffffu : ((1u << (R % 32)) - 1u);
                    const uint32_t mine = (broke >> (ph * R)) & kRows;
                    if (mine) atomicAnd(wbits + k, ~(mine << ((h * R) % 32)));
                }
            }
            fxa = phase_sum<Q>(fxa);
            fya = phase_sum<Q>(fya);
            fza = phase_sum<Q>(fza);
            if (ph == 0 && force_row) {
                // undo the power-of-two scaling of the bond coefficient (exact)
                const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
                const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
                const double fzr = f64_of_pair_scaled(fza.h, fza.l, A.kexp);
                row_epilogue<3, EPI>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
            }
        }
        if (EPI == EPI_VERLET && A.do_next && ph == 0 && !force_row && r < P.N) boundary_row<3>(A, r);
    }
    if (EPI == EPI_ADR) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// The compact layout with several warps per slice (as k_bond_split): warp
// `sub` computes the slots sub, sub + split, ... into shared memory and the
// group's first warp adds them in slot order (bit for bit the one-warp sums).
// Shared memory per group: wmax slots x 2 components x 32 lanes pairs and one
// alive word per slot.
template <int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kBondMinBlocks) k_bond_compact_split(const ForceArgs A) {
    extern __shared__ __align__(16) unsigned char sm_groups[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int split = A.split, G = (int)(blockDim.x >> 5) / split;
    const int g = wib / split, sub = wib % split;
    const int Wm = A.wmax;
    float2* contrib = reinterpret_cast<float2*>(sm_groups) + (size_t)g * Wm * 64;
    uint32_t* alive_w =
        reinterpret_cast<uint32_t*>(reinterpret_cast<float2*>(sm_groups) + (size_t)G * Wm * 64) + g * Wm;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const int64_t groups = (int64_t)gridDim.x * G;
    const int64_t rounds = (A.nslices + groups - 1) / groups;
    for (int64_t it = 0; it < rounds; it++) {
        const int64_t s = it * groups + (int64_t)blockIdx.x * G + g;
        const int64_t r = s * 32 + lane;
        const bool in = s < A.nslices;
        const bool force_row = in && r < A.nforce;
        const bool work = in && s * 32 < A.nforce;
        const int64_t rr = force_row ? r : (A.nforce > 0 ? A.nforce - 1 : 0);
        double xi = 0.0, yi = 0.0, uxi = 0.0, uyi = 0.0;
        int W = 0;
        if (work) {
            xi = A.x[rr], yi = A.y[rr], uxi = A.ux[rr], uyi = A.uy[rr];
            const double s0 = A.node_s0 ? A.node_s0[rr] : P.critical_s;
            const float s0f = __double2float_rn(s0);
            const bt::Tpl* tpls = slice_templates(A, s);
            W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            for (int k = sub; k < W; k += split) {
                const int64_t slot = b + (int64_t)k * 32 + lane;
                const uint32_t word = wbits[k];
                const bool alive = force_row && ((word >> lane) & 1u);
                bool brk = false;
                bt::f2 cf[2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
                if (alive)
                    brk = bond_compact(A, tpls, __ldg(reinterpret_cast<const int4*>(A.rec16 + slot)), xi, yi, uxi, uyi,
                                       s0, s0f, cf);
                contrib[(k * 2 + 0) * 32 + lane] = make_float2(cf[0].h, cf[0].l);
                contrib[(k * 2 + 1) * 32 + lane] = make_float2(cf[1].h, cf[1].l);
                const uint32_t am = __ballot_sync(0xffffffffu, alive);
                if (lane == 0) alive_w[k] = am;
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
            }
        }
        __syncthreads();
        if (sub == 0 && work) {
            bt::f2 fxa{0.0f, 0.0f}, fya{0.0f, 0.0f};
            for (int k = 0; k < W; k++) {
                if (!((alive_w[k] >> lane) & 1u)) continue;
                const float2 cx = contrib[(k * 2 + 0) * 32 + lane], cy = contrib[(k * 2 + 1) * 32 + lane];
                bt::acc_add(fxa, bt::f2{cx.x, cx.y});
                bt::acc_add(fya, bt::f2{cy.x, cy.y});
            }
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
            if (force_row) row_epilogue<2, EPI>(A, r, fxr, fyr, 0.0, xi, yi, 0.0, uxi, uyi, 0.0, red);
            if (EPI == EPI_ADR && A.slice_part) slice_partials(A, s, red);
        }
        if (sub == 0 && EPI == EPI_VERLET && A.do_next && in && !force_row && r < P.N) boundary_row<2>(A, r);
        __syncthreads();
    }
    if (EPI == EPI_ADR && !A.slice_part) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// 3-D bond force with several warps per slice (A.split of them).  A 3-D row
// (about 120 slots at a horizon of three spacings) is summed in blocks of 32
// slots, each block from zero in slot order and the block sums in block order
// (as k_bond_force<3> does), so warp `sub` of a slice group takes the blocks
// sub, sub + split, ... and leaves their sums in shared memory for the
// group's first warp: bit for bit the one-warp result.  It turns the 5,652
// slices of the impact slab into four times as many shorter tasks, which
// fill the SMs evenly where one slice per warp leaves a partial second wave.
// Shared memory per group: ceil(wmax / 32) blocks x 3 components x 32 lanes
// pairs.
template <int EPI>
__global__ void __launch_bounds__(kMaxBondBlock, kBondMinBlocks) k_bond_split3(const ForceArgs A) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int split = A.split, G = (int)(blockDim.x >> 5) / split;
    const int g = wib / split, sub = wib % split;
    const int nbm = (A.wmax + 31) / 32;
    float2* bsum = reinterpret_cast<float2*>(sm_raw) + (size_t)g * nbm * 96;  // [block][component][lane]
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const int64_t groups = (int64_t)gridDim.x * G;
    const int64_t rounds = (A.nslices + groups - 1) / groups;
    for (int64_t it = 0; it < rounds; it++) {
        const int64_t s = it * groups + (int64_t)blockIdx.x * G + g;
        const int64_t r = s * 32 + lane;
        const bool in = s < A.nslices;
        const bool force_row = in && r < A.nforce;
        const bool work = in && s * 32 < A.nforce;
        const int64_t rr = force_row ? r : (A.nforce > 0 ? A.nforce - 1 : 0);
        double xi = 0.0, yi = 0.0, zi = 0.0, uxi = 0.0, uyi = 0.0, uzi = 0.0;
        int W = 0;
        if (work) {
            xi = A.x[rr], yi = A.y[rr], zi = A.z[rr];
            uxi = A.ux[rr], uyi = A.uy[rr], uzi = A.uz[rr];
            W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            for (int kb = sub * 32; kb < W; kb += split * 32) {
                const int ke = kb + 32 < W ? kb + 32 : W;
                ff bx{0.0f, 0.0f}, by{0.0f, 0.0f}, bz{0.0f, 0.0f};
                int4 q0_next = rec_q0(A.rec, b + (int64_t)kb * 32 + lane);
                for (int k = kb; k < ke; k++) {
                    const int64_t slot = b + (int64_t)k * 32 + lane;
                    const int4 q0 = q0_next;
                    if (k + 1 < ke) q0_next = rec_q0(A.rec, slot + 32);
                    const uint32_t word = wbits[k];
                    const bool alive = force_row && ((word >> lane) & 1u);
                    bool brk = false;
                    if (alive) {
                        ff cf[3];
                        brk = bond3<3>(A, q0, rec_q1(A.rec, slot), rec_q2(A.rec, slot), xi, yi, zi, uxi, uyi, uzi,
                                       cf);
                        bx = ff_add(bx, cf[0]);
                        by = ff_add(by, cf[1]);
                        bz = ff_add(bz, cf[2]);
                    }
                    const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                    if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
                }
                float2* o = bsum + (size_t)(kb >> 5) * 96;
                o[lane] = make_float2(bx.h, bx.l);
                o[32 + lane] = make_float2(by.h, by.l);
                o[64 + lane] = make_float2(bz.h, bz.l);
            }
        }
        __syncthreads();
        if (sub == 0 && work) {
            ff fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
            for (int kb = 0; kb < W; kb += 32) {
                const float2* o = bsum + (size_t)(kb >> 5) * 96;
                const float2 cx = o[lane], cy = o[32 + lane], cz = o[64 + lane];
                fxa = ff_add(fxa, ff{cx.x, cx.y});
                fya = ff_add(fya, ff{cy.x, cy.y});
                fza = ff_add(fza, ff{cz.x, cz.y});
            }
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.kexp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.kexp);
            const double fzr = f64_of_pair_scaled(fza.h, fza.l, A.kexp);
            if (force_row) row_epilogue<3, EPI>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
            if (EPI == EPI_ADR && A.slice_part) slice_partials(A, s, red);
        }
        if (sub == 0 && EPI == EPI_VERLET && A.do_next && in && !force_row && r < P.N) boundary_row<3>(A, r);
        __syncthreads();
    }
    if (EPI == EPI_ADR && !A.slice_part) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// Dilatation pass (kernel_cal_theta_2D/3D): every row of [0, N).  Stores the
// extension e per bond with the reference's operand order for this pass,
// ((x_c - x_i) + u_c) - u_i, and theta/m per node.  The 2-D pass counts every
// bond of the family, intact or not (Force_State.cu:65); the 3-D pass intact
// ones only (:214).
template <int DIM>
__device__ __forceinline__ void theta_pass(const ForceArgs& A) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const KParams& P = A.P;
    for (int64_t s = (int64_t)blockIdx.x * kWarpsPerBlock + wib; s < A.nslices;
         s += (int64_t)gridDim.x * kWarpsPerBlock) {
        const int64_t r = s * 32 + lane;
        const bool row = r < P.N;
        const int64_t rr = row ? r : P.N - 1;
        const int nn = row ? A.NN[rr] : 0;
        const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = DIM == 3 ? A.uz[rr] : 0.0;
        const bool check_bits = DIM == 3 && r < P.N_int;
        const int W = A.width[s];
        const int64_t b = A.base[s];
        const uint32_t* wbits = A.bits + A.fbase[s];
        ff acc{0.0f, 0.0f};  // sum of the weighted extensions, times 2^sth_exp
        for (int k = 0; k < W; k++) {
            const int64_t slot = b + (int64_t)k * 32 + lane;
            bool use = k < nn;
            if (check_bits) use = use && ((wbits[k] >> lane) & 1u);
            if (use) {
                const float4 w0 = srec_w(A.sgeo, slot, 0), w1 = srec_w(A.sgeo, slot, 1);
                const float4 w2 = srec_w(A.sth, slot, 0), w3 = srec_w(A.sth, slot, 1);
                const int c = __float_as_int(w0.x);
                const float xf[3] = {w0.y, w0.z, w0.w};
                // d = (xi + u_c) - u_i, the dilatation pass's operand order, then
                // its exact offset from xf and the extension in pairs
                ff eta[3], dp[3], y, e2;
                eta[0] = exact_offset((lo_f64(w2) + A.ux[c]) - uxi, xf[0]);
                eta[1] = exact_offset((hi_f64(w2) + A.uy[c]) - uyi, xf[1]);
                if (DIM == 3) eta[2] = exact_offset((lo_f64(w3) + A.uz[c]) - uzi, xf[2]);
                pair_stretch<DIM>(eta, xf, make_float2(w1.x, w1.y), make_float2(w1.z, w1.w), dp, y, e2);
                // e stays a pair for the force pass; the weighted sum is formed in
                // pairs too (no FP64 instruction per bond beyond the bond vector)
                A.e[slot] = make_float2(e2.h, e2.l);
                acc = ff_add(acc, ff_mul(ff{w3.z, w3.w}, e2));
            }
        }
        if (row) {
            // theta = acc / m and theta / m through 1/m (nb, IEEE-rounded at set-up)
            const double m = A.m[r], rm = A.nb[r];
            const double a = f64_of_pair_scaled(acc.h, acc.l, -A.sth_exp);
            const double th = div_recip(a, m, rm);
            A.theta[r] = th;
            const ff na = ff_split(div_recip(th, m, rm) * A.sn_scale);
            *reinterpret_cast<float2*>(A.nab + r) = make_float2(na.h, na.l);
        }
    }
}

// The 2-D dilatation pass is left to the compiler (50 registers; a cap at 48
// was measured 1 % slower).  The 3-D pass is compiled for five resident
// 256-thread blocks per SM (48 registers, a few spilled bytes): 40 warps in
// flight instead of 32, measured 1.025 -> 0.989 ms per step on the
// 180,873-node impact slab.
template <int DIM>
__global__ void __launch_bounds__(kForceBlock) k_theta(const ForceArgs A) {
    theta_pass<DIM>(A);
}
template <>
__global__ void __launch_bounds__(kForceBlock, 5) k_theta<3>(const ForceArgs A) {
    theta_pass<3>(A);
}

// State-based force pass (kernel_state_force_2D/3D) on rows [0, N_int):
// t_i + t_j = c1 (theta_i/m_i + theta_j/m_j) + c2 e (1/m_i + 1/m_j) per bond.
template <int DIM, int EPI>
__global__ void __launch_bounds__(kForceBlock, kStateMinBlocks) k_state_force(const ForceArgs A) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    for (int64_t s = (int64_t)blockIdx.x * kWarpsPerBlock + wib; s < A.nslices;
         s += (int64_t)gridDim.x * kWarpsPerBlock) {
        const int64_t r = s * 32 + lane;
        const bool force_row = r < A.nforce;
        if (s * 32 < A.nforce) {
            const int64_t rr = force_row ? r : A.nforce - 1;
            const double xi = A.x[rr], yi = A.y[rr], zi = DIM == 3 ? A.z[rr] : 0.0;
            const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = DIM == 3 ? A.uz[rr] : 0.0;
            const float4 nab_i = A.nab[rr];
            const ff nai{nab_i.x, nab_i.y}, nbi{nab_i.z, nab_i.w};
            double fxr = 0.0, fyr = 0.0, fzr = 0.0;
            ff fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
            const int W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            for (int k = 0; k < W; k++) {
                const int64_t slot = b + (int64_t)k * 32 + lane;
                const uint32_t word = wbits[k];
                const bool alive = force_row && ((word >> lane) & 1u);
                bool brk = false;
                if (alive) {
                    const float4 w0 = srec_w(A.sgeo, slot, 0), w1 = srec_w(A.sgeo, slot, 1);
                    const float4 w4 = srec_w(A.sfo, slot, 0), w5 = srec_w(A.sfo, slot, 1);
                    const int c = __float_as_int(w0.x);
                    const float xf[3] = {w0.y, w0.z, w0.w};
                    // d = (P_c - x_i) - u_i, the force pass's operand order, then its
                    // exact offsets from xf and the stretch in pairs
                    ff eta[3], dp[3], y, e2, etaz{0.0f, 0.0f};
                    const double2 pxy = A.pc[c];
                    eta[0] = bond_offset(pxy.x, xi, uxi, xf[0]);
                    eta[1] = bond_offset(pxy.y, yi, uyi, xf[1]);
                    if (DIM == 3) {
                        // the reference's 3-D force kernel takes the z term of the
                        // length in the dilatation pass's operand order (Force_State.cu:272)
                        eta[2] = exact_offset((hi_f64(w5) + A.uz[c]) - uzi, xf[2]);
                        etaz = bond_offset(A.pcz[c], zi, uzi, xf[2]);
                    }
                    pair_stretch<DIM>(eta, xf, make_float2(w1.x, w1.y), make_float2(w1.z, w1.w), dp, y, e2);
                    // T = c1 (theta_i/m_i + theta_j/m_j) + c2 e (1/m_i + 1/m_j), times 2^-st_exp,
                    // in pair arithmetic on the scaled pairs (no FP64 instruction)
                    const float2 ec = A.e[slot];
                    const float4 nc = __ldg(A.nab + c);
                    const ff T = ff_add(ff_mul(ff{w4.x, w4.y}, ff_add(nai, ff{nc.x, nc.y})),
                                        ff_mul(ff_mul(ff{w4.z, w4.w}, ff{ec.x, ec.y}), ff_add(nbi, ff{nc.z, nc.w})));
                    // t = T / (2 L) and f += t d in pair arithmetic (as in the bond-based kernel)
                    const ff t = ff_mul(T, ff{0.5f * y.h, 0.5f * y.l});
                    fxa = ff_add(fxa, ff_mul(t, dp[0]));
                    fya = ff_add(fya, ff_mul(t, dp[1]));
                    if (DIM == 3) fza = ff_add(fza, ff_mul(t, ff_add_f(xf[2], etaz)));
                    brk = pair_exceeds(e2, lo_f64(w5));
                }
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
            }
            // undo the power-of-two scale of T (exact)
            fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.st_exp);
            fyr = f64_of_pair_scaled(fya.h, fya.l, A.st_exp);
            if (DIM == 3) fzr = f64_of_pair_scaled(fza.h, fza.l, A.st_exp);
            if (force_row) row_epilogue<DIM, EPI>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
        }
        if (EPI == EPI_VERLET && A.do_next && !force_row && r < P.N) boundary_row<DIM>(A, r);
    }
    if (EPI == EPI_ADR) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}


// The 3-D state-based force pass without epilogue (the explicit step's node
// pass follows it), each warp on R = 32 / Q rows of a slice: lane j + R p
// takes row j's slots p, p + Q, p + 2Q, ... and the Q partial sums of a row
// are added as a tree over the lane groups (pair addition is commutative, so
// every lane of the row gets the same sum).  The impact slab has 5,652 slices
// of about 104 slots against 4,864 warps resident at this kernel's 64
// registers: one warp per slice leaves a second round of 788 slices on a
// nearly empty GPU; units of a quarter slice fill five rounds of a quarter
// the length.  The sum order depends on Q only, not on the launch shape.
// Intact flags of other units of the slice share the words, so breaks clear
// their bits with atomicAnd.  Measured on the compact layout (impact slab,
// ms per step): Q = 1: 0.823, 2: 0.789, 4: 0.770, 8: 0.841.
constexpr int kStatePhases3 = 4;
template <int Q>
__global__ void __launch_bounds__(kForceBlock, kStateMinBlocks) k_state_force3_phased(const ForceArgs A) {
    constexpr int R = 32 / Q;
    static_assert(Q >= 1 && Q <= 8 && 32 % Q == 0, "1 to 8 phases");
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int j = lane % R, ph = lane / R;
    const int64_t units = A.nslices * Q;
    double red[3] = {0.0, 0.0, 0.0};
    for (int64_t u = (int64_t)blockIdx.x * wpb + wib; u < units; u += (int64_t)gridDim.x * wpb) {
        const int64_t s = u / Q;
        const int h = (int)(u - s * Q);
        if (s * 32 + h * R >= A.nforce) continue;  // warp-uniform: no force row in the unit
        const int rl = h * R + j;  // the row's lane in the slice
        const int64_t r = s * 32 + rl;
        const bool force_row = r < A.nforce;
        const int64_t rr = force_row ? r : A.nforce - 1;
        const double xi = A.x[rr], yi = A.y[rr], zi = A.z[rr];
        const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = A.uz[rr];
        const float4 nab_i = A.nab[rr];
        const ff nai{nab_i.x, nab_i.y}, nbi{nab_i.z, nab_i.w};
        ff fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
        const int W = A.width[s];
        const int64_t b = A.base[s];
        uint32_t* wbits = A.bits + A.fbase[s];
        const int iters = (W + Q - 1) / Q;
        for (int i = 0; i < iters; i++) {
            const int k = i * Q + ph;
            const int64_t slot = b + (int64_t)k * 32 + rl;
            const uint32_t word = k < W ? wbits[k] : 0u;
            const bool alive = force_row && ((word >> rl) & 1u);
            bool brk = false;
            if (alive) {
                const float4 w0 = srec_w(A.sgeo, slot, 0), w1 = srec_w(A.sgeo, slot, 1);
                const float4 w4 = srec_w(A.sfo, slot, 0), w5 = srec_w(A.sfo, slot, 1);
                const int c = __float_as_int(w0.x);
                const float xf[3] = {w0.y, w0.z, w0.w};
                // as k_state_force<3>: the force pass's operand order, the z term of
                // the length in the dilatation pass's (Force_State.cu:272)
                ff eta[3], dp[3], y, e2, etaz;
                const double2 pxy = A.pc[c];
                eta[0] = bond_offset(pxy.x, xi, uxi, xf[0]);
                eta[1] = bond_offset(pxy.y, yi, uyi, xf[1]);
                eta[2] = exact_offset((hi_f64(w5) + A.uz[c]) - uzi, xf[2]);
                etaz = bond_offset(A.pcz[c], zi, uzi, xf[2]);
                pair_stretch<3>(eta, xf, make_float2(w1.x, w1.y), make_float2(w1.z, w1.w), dp, y, e2);
                const float2 ec = A.e[slot];
                const float4 nc = __ldg(A.nab + c);
                const ff T = ff_add(ff_mul(ff{w4.x, w4.y}, ff_add(nai, ff{nc.x, nc.y})),
                                    ff_mul(ff_mul(ff{w4.z, w4.w}, ff{ec.x, ec.y}), ff_add(nbi, ff{nc.z, nc.w})));
                const ff t = ff_mul(T, ff{0.5f * y.h, 0.5f * y.l});
                fxa = ff_add(fxa, ff_mul(t, dp[0]));
                fya = ff_add(fya, ff_mul(t, dp[1]));
                fza = ff_add(fza, ff_mul(t, ff_add_f(xf[2], etaz)));
                brk = pair_exceeds(e2, lo_f64(w5));
            }
            const uint32_t broke = __ballot_sync(0xffffffffu, brk);
            if (broke && j == 0 && !A.nobreak) {
                constexpr uint32_t kRows = R >= 32 ? 0xffffffffu : ((1u << (R % 32)) - 1u);
                const uint32_t mine = (broke >> (ph * R)) & kRows;
                if (mine) atomicAnd(wbits + k, ~(mine << ((h * R) % 32)));
            }
        }
#pragma unroll
        for (int off = R; off < 32; off <<= 1) {
            fxa = ff_add(fxa, ff{__shfl_xor_sync(0xffffffffu, fxa.h, off), __shfl_xor_sync(0xffffffffu, fxa.l, off)});
            fya = ff_add(fya, ff{__shfl_xor_sync(0xffffffffu, fya.h, off), __shfl_xor_sync(0xffffffffu, fya.l, off)});
            fza = ff_add(fza, ff{__shfl_xor_sync(0xffffffffu, fza.h, off), __shfl_xor_sync(0xffffffffu, fza.l, off)});
        }
        if (ph == 0 && force_row) {
            // undo the power-of-two scale of T (exact)
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.st_exp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.st_exp);
            const double fzr = f64_of_pair_scaled(fza.h, fza.l, A.st_exp);
            row_epilogue<3, EPI_NONE>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
        }
    }
}

// ---- 2-D state-based passes on the compact layout -------------------------
//
// Per slot a 16-byte record for the dilatation pass (column; dl with the
// offset class id; kx, ky) and an 8-byte record for the force pass (column;
// dl with the class id).  The reference vector x_c - x_i, as the reference
// rounds it in the dilatation pass, is the class's float vector as a double
// moved by kx, ky representable doubles: an integer addition on the bit
// pattern instead of an FP64 subtraction and two gathered coordinates.  The
// bond coefficients come from the class (StateTpl); the stretch arithmetic is
// bt::stretch2 on the class template; e goes from the first pass to the
// second in a pair per slot (recomputing it in the force pass would take the
// dilatation order's bond vector, four more FP64 instructions per bond, on
// the pipe that bounds the dilatation pass).  Per slot and step: 16 + 8
// bytes in the dilatation pass, 8 + 8 in the force pass.

// One bond's exact offsets from its class's float reference vector.
__device__ __forceinline__ void offsets2(const bt::Tpl& T, const double d[2], bt::f2 eta[2]) {
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const uint64_t xb = T.xd[a];
        if (xb == 0)
            eta[a] = bt::split_bits(d[a]);
        else if (!bt::offset_pair(d[a], xb, eta[a]))
            eta[a] = bt::split_bits(d[a] - bt::dfrom(xb));  // exact by Sterbenz's lemma
    }
}

// Dilatation pass (kernel_cal_theta_2D, Force_State.cu:56-85) on every row of
// [0, N), every bond of the family (the 2-D kernel counts broken bonds too).
// Work units of R = 32 / Q rows of a slice: lane j + R p takes row j's slots
// p, p + Q, ... (Q = 1: one warp per slice); the sum order depends on Q only.
template <int Q>
__global__ void __launch_bounds__(kForceBlock) k_theta_compact(const ForceArgs A) {
    constexpr int R = 32 / Q;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int j = lane % R, ph = lane / R;
    const KParams& P = A.P;
    const int64_t units = A.nslices * Q;
    for (int64_t u = (int64_t)blockIdx.x * wpb + wib; u < units; u += (int64_t)gridDim.x * wpb) {
        const int64_t s = u / Q;
        const int h = (int)(u - s * Q);
        const int rl = h * R + j;
        const int64_t r = s * 32 + rl;
        const bool row = r < P.N;
        const int64_t rr = row ? r : P.N - 1;
        const int nn = row ? A.NN[rr] : 0;
        const double uxi = A.ux[rr], uyi = A.uy[rr];
        const int64_t b = A.base[s];
        const int4* rp = A.srec + b + rl;
        bt::f2 acc{0.0f, 0.0f};  // sum of the weighted extensions, times 2^sth_exp
        // the lane's next slot's record loaded one iteration ahead
        int4 rq_next = ph < nn ? __ldg(rp + (int64_t)ph * 32) : make_int4(0, 0, 0, 0);
        for (int k = ph; k < nn; k += Q) {
            const int4 rq = rq_next;
            if (k + Q < nn) rq_next = __ldg(rp + (int64_t)(k + Q) * 32);
            const int c = rq.x;
            const uint32_t dlb = (uint32_t)rq.y;
            const int id = (int)(dlb & 0xffu);
            const bt::Tpl& T = A.tpl[id];
            const float dl = __uint_as_float(dlb & ~0xffu);
            // x_c - x_i as the reference rounds it, then d = (that + u_c) - u_i,
            // the dilatation pass's operand order
            const double xa = __longlong_as_double((long long)T.xd[0] + rq.z);
            const double ya = __longlong_as_double((long long)T.xd[1] + rq.w);
            const double d[2] = {(xa + __ldg(A.ux + c)) - uxi, (ya + __ldg(A.uy + c)) - uyi};
            bt::f2 eta[2], w[2], y, e;
            offsets2(T, d, eta);
            bt::stretch2(eta, T, dl, w, y, e);
            A.e[b + (int64_t)k * 32 + rl] = make_float2(e.h, e.l);
            // cth of the class moved to this bond's length: cth (1 + g1 dl)
            const float4 ct = __ldg(reinterpret_cast<const float4*>(A.stpl + id) + 1);
            const bt::f2 cth{ct.x, fmaf(ct.x, ct.z * dl, ct.y)};
            acc = bt::add(acc, bt::mul(cth, e));
        }
        if (Q > 1) acc = phase_sum<Q>(acc);
        if (row && ph == 0) {
            // theta = acc / m and theta / m through 1/m (nb, IEEE-rounded at set-up)
            const double m = A.m[r], rm = A.nb[r];
            const double a = f64_of_pair_scaled(acc.h, acc.l, -A.sth_exp);
            const double th = div_recip(a, m, rm);
            A.theta[r] = th;
            const ff na = ff_split(div_recip(th, m, rm) * A.sn_scale);
            *reinterpret_cast<float2*>(A.nab + r) = make_float2(na.h, na.l);
        }
    }
}

// State-based force pass (kernel_state_force_2D, Force_State.cu:88-134) on
// rows [0, N_int): t_i + t_j = c1 (theta_i/m_i + theta_j/m_j) + c2 e (1/m_i +
// 1/m_j) per bond with e from the dilatation pass, the length and direction
// in the force pass's operand order.  Work units as k_theta_compact<Q>;
// with Q > 1 the units of a slice share its intact-flag words, so breaks
// clear their bits with atomicAnd.
template <int EPI, int Q>
__global__ void __launch_bounds__(kForceBlock, kStateMinBlocks) k_state_compact(const ForceArgs A) {
    constexpr int R = 32 / Q;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int j = lane % R, ph = lane / R;
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    const double s0 = P.critical_s;
    const float s0f = __double2float_rn(s0);
    const int64_t units = A.nslices * Q;
    for (int64_t u = (int64_t)blockIdx.x * wpb + wib; u < units; u += (int64_t)gridDim.x * wpb) {
        const int64_t s = u / Q;
        const int h = (int)(u - s * Q);
        const int rl = h * R + j;
        const int64_t r = s * 32 + rl;
        const bool force_row = r < A.nforce;
        if (s * 32 + h * R < A.nforce) {  // warp-uniform: the unit holds a force row
            const int64_t rr = force_row ? r : A.nforce - 1;
            const double xi = A.x[rr], yi = A.y[rr];
            const double uxi = A.ux[rr], uyi = A.uy[rr];
            const float4 nab_i = A.nab[rr];
            const bt::f2 nai{nab_i.x, nab_i.y}, nbi{nab_i.z, nab_i.w};
            bt::f2 fxa{0.0f, 0.0f}, fya{0.0f, 0.0f};
            const int W = A.width[s];
            const int64_t b = A.base[s];
            uint32_t* wbits = A.bits + A.fbase[s];
            const int2* rp = A.srec8 + b + rl;
            const int iters = (W + Q - 1) / Q;
            // the lane's next slot's record loaded one iteration ahead
            int2 rq_next = ph < W ? __ldg(rp + (int64_t)ph * 32) : make_int2(0, 0);
            for (int i = 0; i < iters; i++) {
                const int k = i * Q + ph;
                const int64_t slot = b + (int64_t)k * 32 + rl;
                const int2 rq = rq_next;
                if (k + Q < W) rq_next = __ldg(rp + (int64_t)(k + Q) * 32);
                const uint32_t word = k < W ? wbits[k] : 0u;
                const bool alive = force_row && ((word >> rl) & 1u);
                bool brk = false;
                if (alive) {
                    const int c = rq.x;
                    const uint32_t dlb = (uint32_t)rq.y;
                    const int id = (int)(dlb & 0xffu);
                    const bt::Tpl& T = A.tpl[id];
                    const float dl = __uint_as_float(dlb & ~0xffu);
                    // d = (P_c - x_i) - u_i, the force pass's operand order
                    const double2 pxy = __ldg(A.pc + c);
                    const double d[2] = {(pxy.x - xi) - uxi, (pxy.y - yi) - uyi};
                    bt::f2 eta[2], w[2], y, ef;
                    offsets2(T, d, eta);
                    bt::stretch2(eta, T, dl, w, y, ef);
                    // T = c1 (theta_i/m_i + theta_j/m_j) + c2 e (1/m_i + 1/m_j), times 2^-st_exp;
                    // c1, c2 of the class moved to this bond's length (1 + g dl)
                    const float4 cc = __ldg(reinterpret_cast<const float4*>(A.stpl + id));
                    const float2 gg = __ldg(reinterpret_cast<const float2*>(A.stpl + id) + 3);
                    const bt::f2 c1{cc.x, fmaf(cc.x, gg.x * dl, cc.y)}, c2{cc.z, fmaf(cc.z, gg.y * dl, cc.w)};
                    const float2 ec = A.e[slot];
                    const float4 nc = __ldg(A.nab + c);
                    const bt::f2 Tt = bt::add(bt::mul(c1, bt::add(nai, bt::f2{nc.x, nc.y})),
                                              bt::mul(bt::mul(c2, bt::f2{ec.x, ec.y}),
                                                      bt::add(nbi, bt::f2{nc.z, nc.w})));
                    // t = T / (2 L) and f += t d
                    const bt::f2 t = bt::mul(Tt, bt::f2{0.5f * y.h, 0.5f * y.l});
                    bt::acc_add(fxa, bt::mul(t, w[0]));
                    bt::acc_add(fya, bt::mul(t, w[1]));
                    brk = bt::exceeds(ef, s0, s0f, T, dl);
                }
                const uint32_t broke = __ballot_sync(0xffffffffu, brk);
                if (Q == 1) {
                    if (broke && lane == 0 && !A.nobreak) wbits[k] = word & ~broke;
                } else if (broke && j == 0 && !A.nobreak) {
                    constexpr uint32_t kRows = R >= 32 ? 0xffffffffu : ((1u << (R % 32)) - 1u);
                    const uint32_t mine = (broke >> (ph * R)) & kRows;
                    if (mine) atomicAnd(wbits + k, ~(mine << (h * R)));
                }
            }
            if (Q > 1) {
                fxa = phase_sum<Q>(fxa);
                fya = phase_sum<Q>(fya);
            }
            if (ph == 0) {
                // undo the power-of-two scale of T (exact)
                const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.st_exp);
                const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.st_exp);
                if (force_row) row_epilogue<2, EPI>(A, r, fxr, fyr, 0.0, xi, yi, 0.0, uxi, uyi, 0.0, red);
            }
        }
        if (EPI == EPI_VERLET && A.do_next && ph == 0 && !force_row && r < P.N) boundary_row<2>(A, r);
    }
    if (EPI == EPI_ADR) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
    if (EPI == EPI_VERLET && A.contact) finish_reduction<EPI>(A, red, 3);
}

// ---- 3-D state-based passes on the compact layout -------------------------
//
// Per slot an 8-byte record (column; dl with the offset class id) read by
// both passes, {kx, ky, kz, flags} read by the dilatation pass and {kz,
// flags} by the force pass; 80-byte class templates (bt::Tpl3) and the class
// coefficients (StateTpl) as in 2-D.  Per slot and step: 8 + 16 + 8 bytes in
// the dilatation pass, 8 + 8 + 8 in the force pass, against 72 and 72 with
// the three 32-byte records.

// Dilatation pass (kernel_cal_theta_3D, Force_State.cu:200-239) on rows [0,
// N): the reference kernel skips broken bonds (its fail test); boundary rows,
// which carry no flags in the reference (Memory.cu:39), count every bond.
__global__ void __launch_bounds__(kForceBlock, 5) k_theta_compact3(const ForceArgs A) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const KParams& P = A.P;
    for (int64_t s = (int64_t)blockIdx.x * wpb + wib; s < A.nslices; s += (int64_t)gridDim.x * wpb) {
        const int64_t r = s * 32 + lane;
        const bool row = r < P.N;
        const int64_t rr = row ? r : P.N - 1;
        const int nn = row ? A.NN[rr] : 0;
        const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = A.uz[rr];
        const bool check_bits = r < P.N_int;
        const int W = A.width[s];
        const int64_t b = A.base[s];
        const uint32_t* wbits = A.bits + A.fbase[s];
        const int2* rp = A.srec8 + b + lane;
        const int4* kp = A.sk + b + lane;
        bt::f2 acc{0.0f, 0.0f};  // sum of the weighted extensions, times 2^sth_exp
        for (int k = 0; k < W; k++) {
            bool use = k < nn;
            if (check_bits) use = use && ((wbits[k] >> lane) & 1u);
            if (use) {
                const int2 rq = __ldg(rp + (int64_t)k * 32);
                const int4 kq = __ldg(kp + (int64_t)k * 32);
                const int c = rq.x;
                const uint32_t dlb = (uint32_t)rq.y;
                const int id = (int)(dlb & 0xffu);
                const bt::Tpl3& T = A.tpl3[id];
                const float dl = __uint_as_float(dlb & ~0xffu);
                // x_c - x_i as the reference rounds it (the class vector moved by
                // kx, ky, kz doubles), then d = (that + u_c) - u_i
                const double xa = __longlong_as_double((long long)T.xd[0] + kq.x);
                const double ya = __longlong_as_double((long long)T.xd[1] + kq.y);
                const double za = __longlong_as_double((long long)T.xd[2] + kq.z);
                const double d[3] = {(xa + __ldg(A.ux + c)) - uxi, (ya + __ldg(A.uy + c)) - uyi,
                                     (za + __ldg(A.uz + c)) - uzi};
                bt::f2 eta[3], w[3], y, e;
                offsets_n<3>(T, d, eta);
                bt::stretch3(eta, T, dl, w, y, e);
                // e for T and the exact z offset for the force pass's length
                A.e4[b + (int64_t)k * 32 + lane] = make_float4(e.h, e.l, eta[2].h, eta[2].l);
                const float4 ct = __ldg(reinterpret_cast<const float4*>(A.stpl + id) + 1);
                const bt::f2 cth{ct.x, fmaf(ct.x, ct.z * dl, ct.y)};
                acc = bt::add(acc, bt::mul(cth, e));
            }
        }
        if (row) {
            const double m = A.m[r], rm = A.nb[r];
            const double a = f64_of_pair_scaled(acc.h, acc.l, -A.sth_exp);
            const double th = div_recip(a, m, rm);
            A.theta[r] = th;
            const ff na = ff_split(div_recip(th, m, rm) * A.sn_scale);
            *reinterpret_cast<float2*>(A.nab + r) = make_float2(na.h, na.l);
        }
    }
}

// Force pass (kernel_state_force_3D, Force_State.cu:242-306) on rows [0,
// N_int), on quarter-slice units as k_state_force3_phased: the length takes
// x and y in the force pass's operand order and z in the dilatation pass's
// (Force_State.cu:270-272), the direction the force pass's order in all three.
// Epilogues without the next step's half-kick (the explicit step runs the
// node pass after this kernel: the length gathers u_z of the neighbours).
template <int EPI>
__global__ void __launch_bounds__(kForceBlock, kStateMinBlocks) k_state_compact3(const ForceArgs A) {
    constexpr int Q = kStatePhases3, R = 32 / Q;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int j = lane % R, ph = lane / R;
    const int64_t units = A.nslices * Q;
    const double s0 = A.P.critical_s;
    const float s0f = __double2float_rn(s0);
    double red[3] = {0.0, 0.0, 0.0};
    for (int64_t u = (int64_t)blockIdx.x * wpb + wib; u < units; u += (int64_t)gridDim.x * wpb) {
        const int64_t s = u / Q;
        const int h = (int)(u - s * Q);
        if (s * 32 + h * R >= A.nforce) continue;  // warp-uniform: no force row in the unit
        const int rl = h * R + j;
        const int64_t r = s * 32 + rl;
        const bool force_row = r < A.nforce;
        const int64_t rr = force_row ? r : A.nforce - 1;
        const double xi = A.x[rr], yi = A.y[rr], zi = A.z[rr];
        const double uxi = A.ux[rr], uyi = A.uy[rr], uzi = A.uz[rr];
        const float4 nab_i = A.nab[rr];
        const bt::f2 nai{nab_i.x, nab_i.y}, nbi{nab_i.z, nab_i.w};
        bt::f2 fxa{0.0f, 0.0f}, fya{0.0f, 0.0f}, fza{0.0f, 0.0f};
        const int W = A.width[s];
        const int64_t b = A.base[s];
        uint32_t* wbits = A.bits + A.fbase[s];
        const uint32_t* bbits = A.bbits + A.fbase[s];
        const int iters = (W + Q - 1) / Q;
        for (int i = 0; i < iters; i++) {
            const int k = i * Q + ph;
            const int64_t slot = b + (int64_t)k * 32 + rl;
            const uint32_t word = k < W ? wbits[k] : 0u;
            const bool alive = force_row && ((word >> rl) & 1u);
            bool brk = false;
            if (alive) {
                const int2 rq = __ldg(A.srec8 + slot);
                const int c = rq.x;
                const uint32_t dlb = (uint32_t)rq.y;
                const int id = (int)(dlb & 0xffu);
                const bt::Tpl3& T = A.tpl3[id];
                const float dl = __uint_as_float(dlb & ~0xffu);
                // the length's components: x, y in the force order; z in the
                // dilatation order, whose exact offset the dilatation pass kept
                // (the same FP64 expression on the same values); then the force
                // order's z for the direction
                const float4 ez = A.e4[slot];
                const double2 pxy = __ldg(A.pc + c);
                const double dlen[2] = {(pxy.x - xi) - uxi, (pxy.y - yi) - uyi};
                const double dzf = (__ldg(A.pcz + c) - zi) - uzi;
                bt::f2 eta[3], w[3], y, ef, etz;
                offsets_n<2>(T, dlen, eta);
                eta[2] = bt::f2{ez.z, ez.w};
                etz = offset1(dzf, T.xd[2]);
                bt::stretch3(eta, T, dl, w, y, ef);
                const bt::f2 sz = bt::two_sum(T.xf[2], etz.h);
                const bt::f2 wz{sz.h, sz.l + etz.l};
                // c1, c2 of the class moved to this bond's length (1 + g dl)
                const float4 cc = __ldg(reinterpret_cast<const float4*>(A.stpl + id));
                const float2 gg = __ldg(reinterpret_cast<const float2*>(A.stpl + id) + 3);
                const bt::f2 c1{cc.x, fmaf(cc.x, gg.x * dl, cc.y)}, c2{cc.z, fmaf(cc.z, gg.y * dl, cc.w)};
                const float4 nc = __ldg(A.nab + c);
                const bt::f2 Tt = bt::add(bt::mul(c1, bt::add(nai, bt::f2{nc.x, nc.y})),
                                          bt::mul(bt::mul(c2, bt::f2{ez.x, ez.y}), bt::add(nbi, bt::f2{nc.z, nc.w})));
                const bt::f2 t = bt::mul(Tt, bt::f2{0.5f * y.h, 0.5f * y.l});
                bt::acc_add(fxa, bt::mul(t, w[0]));
                bt::acc_add(fya, bt::mul(t, w[1]));
                bt::acc_add(fza, bt::mul(t, wz));
                brk = ((bbits[k] >> rl) & 1u) && bt::exceeds(ef, s0, s0f, T, dl);
            }
            const uint32_t broke = __ballot_sync(0xffffffffu, brk);
            if (broke && j == 0 && !A.nobreak) {
                constexpr uint32_t kRows = R >= 32 ? 0xffffffffu : ((1u << (R % 32)) - 1u);
                const uint32_t mine = (broke >> (ph * R)) & kRows;
                if (mine) atomicAnd(wbits + k, ~(mine << ((h * R) % 32)));
            }
        }
#pragma unroll
        for (int off = R; off < 32; off <<= 1) {
            fxa = bt::add(fxa, bt::f2{__shfl_xor_sync(0xffffffffu, fxa.h, off), __shfl_xor_sync(0xffffffffu, fxa.l, off)});
            fya = bt::add(fya, bt::f2{__shfl_xor_sync(0xffffffffu, fya.h, off), __shfl_xor_sync(0xffffffffu, fya.l, off)});
            fza = bt::add(fza, bt::f2{__shfl_xor_sync(0xffffffffu, fza.h, off), __shfl_xor_sync(0xffffffffu, fza.l, off)});
        }
        if (ph == 0 && force_row) {
            const double fxr = f64_of_pair_scaled(fxa.h, fxa.l, A.st_exp);
            const double fyr = f64_of_pair_scaled(fya.h, fya.l, A.st_exp);
            const double fzr = f64_of_pair_scaled(fza.h, fza.l, A.st_exp);
            row_epilogue<3, EPI>(A, r, fxr, fyr, fzr, xi, yi, zi, uxi, uyi, uzi, red);
        }
    }
    if (EPI == EPI_ADR) finish_reduction<EPI>(A, red, A.res_out ? 3 : 2);
}

// Standalone kernel_cnn + cal_cn (Integrate.cu:7-49, :108-129) on the current forces.
template <int DIM>
__global__ void __launch_bounds__(kForceBlock) k_adr_cnn(const ForceArgs A) {
    double red[3] = {0.0, 0.0, 0.0};
    const KParams& P = A.P;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.N_int; r += (int64_t)gridDim.x * blockDim.x) {
        const double uxi = A.ux[r], uyi = A.uy[r], uzi = DIM == 3 ? A.uz[r] : 0.0;
        // the damping terms as the fused epilogue forms them (damping_term)
        const double rmass = A.node_mass ? A.node_rmass[r] : P.rmass;
        double cn = 0.0, disp;
        if (nonzero(A.vhx[r])) cn = damping_term(uxi, A.fx[r], A.fox[r], rmass, P.dt, A.vhx[r]);
        disp = uxi * uxi;
        if (nonzero(A.vhy[r])) cn += damping_term(uyi, A.fy[r], A.foy[r], rmass, P.dt, A.vhy[r]);
        disp += uyi * uyi;
        if (DIM == 3) {
            if (nonzero(A.vhz[r])) cn += damping_term(uzi, A.fz[r], A.foz[r], rmass, P.dt, A.vhz[r]);
            disp += uzi * uzi;
        }
        red[0] += cn;
        red[1] += disp;
        const double rx = A.fx[r] + A.bx[r], ry = A.fy[r] + A.by[r];
        double rr = rx * rx + ry * ry;
        if (DIM == 3) {
            const double rz = A.fz[r] + A.bz[r];
            rr += rz * rz;
        }
        red[2] += rr;
    }
    finish_reduction<EPI_ADR>(A, red, 3);
}

// Standalone kernel_contact (Solve_Kalthoff_Winkler.cu:112-175) on nodes [0, N).
__global__ void __launch_bounds__(kForceBlock) k_contact(const ForceArgs A) {
    double red[3] = {0.0, 0.0, 0.0};
    const KParams& P = A.P;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.N; r += (int64_t)gridDim.x * blockDim.x) {
        if (!(A.dmg[r] < 1.0)) continue;
        double ux = A.ux[r], uy = A.uy[r], uz = A.uz[r], vx = A.vx[r], vy = A.vy[r], vz = A.vz[r];
        const double ox = ux, oy = uy, oz = uz;
        contact_node(P, *A.cyl, A.x[r], A.y[r], A.z[r], ux, uy, uz, vx, vy, vz, red);
        if (ux != ox || uy != oy || uz != oz || vx != A.vx[r] || vy != A.vy[r] || vz != A.vz[r]) {
            A.ux[r] = ux;
            A.uy[r] = uy;
            A.uz[r] = uz;
            A.vx[r] = vx;
            A.vy[r] = vy;
            A.vz[r] = vz;
        }
    }
    finish_reduction<EPI_NONE>(A, red, 3);
}

// Node pass after a force-only launch: the Verlet epilogue (contact, second
// half-kick, next step's loading and first half) for kernels whose gathers
// read u itself, which the fused epilogue must then not overwrite.
template <int DIM>
__global__ void __launch_bounds__(kForceBlock) k_node_post(const ForceArgs A) {
    const KParams& P = A.P;
    double red[3] = {0.0, 0.0, 0.0};
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.N; r += (int64_t)gridDim.x * blockDim.x) {
        if (r < A.nforce) {
            const double xi = A.x[r], yi = A.y[r], zi = DIM == 3 ? A.z[r] : 0.0;
            row_epilogue<DIM, EPI_VERLET>(A, r, A.fx[r], A.fy[r], DIM == 3 ? A.fz[r] : 0.0, xi, yi, zi, A.ux[r],
                                          A.uy[r], DIM == 3 ? A.uz[r] : 0.0, red);
        } else if (A.do_next) {
            boundary_row<DIM>(A, r);
        }
    }
    if (A.contact) finish_reduction<EPI_VERLET>(A, red, 3);
}

}  // namespace

static ForceArgs make_args(pd_ctx* c) {
    ForceArgs A{};
    A.P = kparams(c->p);
    const Sell& S = c->sell;
    A.nslices = S.nslices;
    A.nforce = c->p.N_int;
    A.width = S.width;
    A.base = S.base;
    A.fbase = S.fbase;
    A.rec = S.rec;
    A.sgeo = S.sgeo;
    A.sth = S.sth;
    A.sfo = S.sfo;
    A.e = S.e;
    A.sn_scale = std::ldexp(1.0, -S.sn_exp);
    A.kexp = S.kexp;
    A.sth_exp = S.sth_exp;
    A.st_exp = S.st_exp;
    A.bits = S.bits;
    A.S = S.S;
    A.NN = c->NN;
    A.x = c->nf[PD_F_X];
    A.y = c->nf[PD_F_Y];
    A.z = c->nf[PD_F_Z];
    A.ux = c->nf[PD_F_UX];
    A.uy = c->nf[PD_F_UY];
    A.uz = c->nf[PD_F_UZ];
    A.pc = c->posxy[c->parity];
    A.pcz = c->posz[c->parity];
    A.pn = c->posxy[c->parity ^ 1];
    A.pnz = c->posz[c->parity ^ 1];
    A.fx = c->nf[PD_F_FX];
    A.fy = c->nf[PD_F_FY];
    A.fz = c->nf[PD_F_FZ];
    A.vx = c->nf[PD_F_VX];
    A.vy = c->nf[PD_F_VY];
    A.vz = c->nf[PD_F_VZ];
    A.ax = c->nf[PD_F_AX];
    A.ay = c->nf[PD_F_AY];
    A.az = c->nf[PD_F_AZ];
    A.bx = c->nf[PD_F_BX];
    A.by = c->nf[PD_F_BY];
    A.bz = c->nf[PD_F_BZ];
    A.fox = c->nf[PD_F_FOX];
    A.foy = c->nf[PD_F_FOY];
    A.foz = c->nf[PD_F_FOZ];
    A.vhx = c->nf[PD_F_VHX];
    A.vhy = c->nf[PD_F_VHY];
    A.vhz = c->nf[PD_F_VHZ];
    A.nab = c->node_a;
    A.nb = c->node_b;
    A.m = c->nf[PD_F_M];
    A.theta = c->nf[PD_F_THETA];
    A.dmg = c->nf[PD_F_DMG];
    A.cyl = c->cyl;
    A.partials = c->partials;
    A.ticket = c->ticket;
    A.cn_out = c->cn;
    A.node_mass = c->batch.node_mass;
    A.node_rmass = c->batch.node_rmass;
    A.slice_part = c->batch.slice_part;
    A.res_out = c->res;
    A.rec16 = S.rec16;
    A.tpl = S.tpl;
    A.ntpl = S.ntpl;
    A.inst_tbase = S.inst_tbase;
    A.slice_inst = c->batch.slice_inst;
    A.node_s0 = c->batch.node_s0;
    A.srec = S.srec;
    A.srec8 = S.srec8;
    A.stpl = S.stpl;
    A.tpl3 = S.tpl3;
    A.sk = S.sk;
    A.e4 = S.e4;
    A.bbits = S.bbits;
    return A;
}

// Grid of the slice kernels: every block resident at once (blocks per SM from
// the occupancy of this kernel instance x SM count), so the grid-stride loop
// over slices runs in one wave with no tail; never more blocks than slices
// need, nor more than the partial-sum buffer holds.
static unsigned resident_grid(pd_ctx* c, const void* kernel, int64_t nslices, int block = kForceBlock,
                              int waves = 1) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t want = (nslices + block / 32 - 1) / (block / 32);
    const int64_t cap = (int64_t)c->num_sms * per_sm * waves;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(want, cap), kMaxPartials));
}

// Slot phases of the 2-D state passes on the compact layout (the Q of
// k_theta_compact<Q> / k_state_compact<EPI, Q>).  Measured on the crack-grow
// plate (7,906 slices of ~28 slots against 4,864-6,080 resident warps),
// dilatation / force phases 1/1: 0.192 ms per step; 2/1: 0.198; 1/4: 0.212;
// 2/2: 0.205; 4/4: 0.233.  Short rows gain nothing from the shorter rounds:
// each unit repeats its rows' set-up, and a warp's loads spread over Q slot
// rows.  (The 3-D force pass, ~104 slots per row, takes kStatePhases3.)
constexpr int kStatePhases2 = 1;

int launch_theta(pd_ctx* c, cudaStream_t s) {
    ForceArgs A = make_args(c);
    if (A.P.dim == 2 && A.srec) {
        // the launch shape's block size (at most kForceBlock) and waves
        const int blk = std::min(c->tune_block, kForceBlock);
        constexpr int Q = kStatePhases2;
        k_theta_compact<Q><<<resident_grid(c, (const void*)k_theta_compact<Q>, A.nslices * Q, blk, c->tune_waves), blk,
                             0, s>>>(A);
    }
    else if (A.P.dim == 2)
        k_theta<2><<<resident_grid(c, (const void*)k_theta<2>, A.nslices), kForceBlock, 0, s>>>(A);
    else if (A.sk)
        k_theta_compact3<<<resident_grid(c, (const void*)k_theta_compact3, A.nslices), kForceBlock, 0, s>>>(A);
    else
        k_theta<3><<<resident_grid(c, (const void*)k_theta<3>, A.nslices), kForceBlock, 0, s>>>(A);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "theta");
}

// The 2-D bond kernels on the compact layout (one warp or A.split warps per
// slice; the templates sit in dynamic shared memory before the split groups).
static int launch_compact(pd_ctx* c, ForceArgs& A, const StepFlags& f, int blk, int waves, cudaStream_t s) {
    const void* kern;
    size_t smem = 0;
    int64_t units = A.nslices;  // slices (one warp each) or slice groups
    int per_block = blk / 32;
    if (c->tune_split > 1) {
        A.split = c->tune_split;
        A.wmax = std::max(1, c->sell.wmax);
        const int G = (blk / 32) / A.split;
        smem += (size_t)G * A.wmax * (64 * sizeof(float2) + sizeof(uint32_t));
        per_block = G;
        kern = f.epi == EPI_VERLET ? (const void*)k_bond_compact_split<EPI_VERLET>
               : f.epi == EPI_ADR  ? (const void*)k_bond_compact_split<EPI_ADR>
                                   : (const void*)k_bond_compact_split<EPI_NONE>;
    } else {
        kern = f.epi == EPI_VERLET ? (const void*)k_bond_compact<EPI_VERLET>
               : f.epi == EPI_ADR  ? (const void*)k_bond_compact<EPI_ADR>
                                   : (const void*)k_bond_compact<EPI_NONE>;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, blk, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t want = (units + per_block - 1) / per_block;
    const unsigned grid = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>(std::min<int64_t>(want, (int64_t)c->num_sms * per_sm * waves), kMaxPartials));
    if (c->tune_split > 1) {
        if (f.epi == EPI_VERLET)
            k_bond_compact_split<EPI_VERLET><<<grid, blk, smem, s>>>(A);
        else if (f.epi == EPI_ADR)
            k_bond_compact_split<EPI_ADR><<<grid, blk, smem, s>>>(A);
        else
            k_bond_compact_split<EPI_NONE><<<grid, blk, smem, s>>>(A);
    } else if (f.epi == EPI_VERLET) {
        k_bond_compact<EPI_VERLET><<<grid, blk, smem, s>>>(A);
    } else if (f.epi == EPI_ADR) {
        k_bond_compact<EPI_ADR><<<grid, blk, smem, s>>>(A);
    } else {
        k_bond_compact<EPI_NONE><<<grid, blk, smem, s>>>(A);
    }
    c->launches++;
    if (f.epi == EPI_VERLET && f.do_next) c->parity ^= 1;
    c->csr_fail_current = false;
    return cuda_err(c, cudaGetLastError(), "bond force (compact)");
}

int launch_force(pd_ctx* c, const StepFlags& f, cudaStream_t s) {
    ForceArgs A = make_args(c);
    A.epi = f.epi;
    A.do_next = f.do_next;
    A.load = f.load;
    A.contact = f.contact;
    A.nobreak = f.nobreak;
    if (!f.residual) A.res_out = nullptr;
    if (f.epi != EPI_VERLET || !f.do_next) {
        // without the next step's half-kick only the force rows are visited
        A.nslices = (A.nforce + 31) / 32;
    }
    const bool state = A.P.model == PD_MODEL_STATE;
    const bool d3 = A.P.dim == 3;
    if (state && d3 && f.epi == EPI_VERLET && (f.do_next || f.contact)) {
        // 3-D state force gathers u_z of the neighbours: force first, then the node pass
        StepFlags g0 = f;
        g0.epi = EPI_NONE;
        int rc = launch_force(c, g0, s);
        if (rc) return rc;
        ForceArgs B = make_args(c);
        B.epi = EPI_VERLET;
        B.do_next = f.do_next;
        B.load = f.load;
        B.contact = f.contact;
        const unsigned gp = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((B.P.N + kForceBlock - 1) / kForceBlock, std::min<int64_t>(c->num_sms * 8, kMaxPartials)));
        k_node_post<3><<<gp, kForceBlock, 0, s>>>(B);
        c->launches++;
        if (f.do_next) c->parity ^= 1;
        if (f.contact && !f.do_next) c->pos_valid = false;
        return cuda_err(c, cudaGetLastError(), "node post");
    }
    const bool bond = !state;
    // the launch shape applies to the bond kernels and to the 2-D state passes
    // of the compact layout (block at most kForceBlock there)
    const bool shaped = bond || (!d3 && A.srec);
    const int blk = bond ? c->tune_block : shaped ? std::min(c->tune_block, kForceBlock) : kForceBlock;
    const int waves = shaped ? c->tune_waves : 1;
    A.chunked = bond ? c->tune_chunked : 0;
    if (bond && !d3 && A.rec16) return launch_compact(c, A, f, blk, waves, s);
    if (bond && d3 && A.rec16) {
        // the launch shape's block size and waves; order and split do not apply
        constexpr int Q = kBondPhases3;
        if (f.epi == EPI_VERLET)
            k_bond_compact3<EPI_VERLET><<<resident_grid(c, (const void*)k_bond_compact3<EPI_VERLET>, A.nslices * Q,
                                                        blk, waves), blk, 0, s>>>(A);
        else if (f.epi == EPI_ADR)
            k_bond_compact3<EPI_ADR><<<resident_grid(c, (const void*)k_bond_compact3<EPI_ADR>, A.nslices * Q, blk,
                                                     waves), blk, 0, s>>>(A);
        else
            k_bond_compact3<EPI_NONE><<<resident_grid(c, (const void*)k_bond_compact3<EPI_NONE>, A.nslices * Q, blk,
                                                      waves), blk, 0, s>>>(A);
        c->launches++;
        if (f.epi == EPI_VERLET && f.do_next) c->parity ^= 1;
        c->csr_fail_current = false;
        return cuda_err(c, cudaGetLastError(), "bond force (compact, 3-D)");
    }
    if (bond && c->tune_split > 1) {
        // several warps per slice (k_bond_split / k_bond_split3), one wave of slice groups
        A.split = c->tune_split;
        A.wmax = std::max(1, c->sell.wmax);
        const int G = (blk / 32) / A.split;
        const size_t smem = d3 ? (size_t)G * ((A.wmax + 31) / 32) * 96 * sizeof(float2)
                               : (size_t)G * A.wmax * (64 * sizeof(float2) + sizeof(uint32_t));
        const void* kern = d3 ? (f.epi == EPI_VERLET ? (const void*)k_bond_split3<EPI_VERLET>
                                 : f.epi == EPI_ADR  ? (const void*)k_bond_split3<EPI_ADR>
                                                     : (const void*)k_bond_split3<EPI_NONE>)
                              : (f.epi == EPI_VERLET ? (const void*)k_bond_split<EPI_VERLET>
                                 : f.epi == EPI_ADR  ? (const void*)k_bond_split<EPI_ADR>
                                                     : (const void*)k_bond_split<EPI_NONE>);
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, blk, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        const int64_t want = (A.nslices + G - 1) / G;
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(std::min<int64_t>(want, (int64_t)c->num_sms * per_sm * waves), kMaxPartials));
        if (d3) {
            if (f.epi == EPI_VERLET)
                k_bond_split3<EPI_VERLET><<<grid, blk, smem, s>>>(A);
            else if (f.epi == EPI_ADR)
                k_bond_split3<EPI_ADR><<<grid, blk, smem, s>>>(A);
            else
                k_bond_split3<EPI_NONE><<<grid, blk, smem, s>>>(A);
        } else if (f.epi == EPI_VERLET) {
            k_bond_split<EPI_VERLET><<<grid, blk, smem, s>>>(A);
        } else if (f.epi == EPI_ADR) {
            k_bond_split<EPI_ADR><<<grid, blk, smem, s>>>(A);
        } else {
            k_bond_split<EPI_NONE><<<grid, blk, smem, s>>>(A);
        }
        c->launches++;
        if (f.epi == EPI_VERLET && f.do_next) c->parity ^= 1;
        if (f.epi == EPI_VERLET && f.contact && !f.do_next) c->pos_valid = false;  // contact moved u, not P
        c->csr_fail_current = false;
        return cuda_err(c, cudaGetLastError(), "bond force (split)");
    }
#define PD_LAUNCH(KER, D, E) \
    KER<D, E><<<resident_grid(c, (const void*)KER<D, E>, A.nslices, blk, waves), blk, 0, s>>>(A)
#define PD_DISPATCH(KER)                                  \
    do {                                                  \
        if (!d3) {                                        \
            if (f.epi == EPI_NONE) PD_LAUNCH(KER, 2, EPI_NONE);   \
            else if (f.epi == EPI_VERLET) PD_LAUNCH(KER, 2, EPI_VERLET); \
            else PD_LAUNCH(KER, 2, EPI_ADR);              \
        } else {                                          \
            if (f.epi == EPI_NONE) PD_LAUNCH(KER, 3, EPI_NONE);   \
            else if (f.epi == EPI_VERLET) PD_LAUNCH(KER, 3, EPI_VERLET); \
            else PD_LAUNCH(KER, 3, EPI_ADR);              \
        }                                                 \
    } while (0)
    if (state && !d3 && A.srec) {
        constexpr int Q = kStatePhases2;
        if (f.epi == EPI_NONE)
            k_state_compact<EPI_NONE, Q><<<resident_grid(c, (const void*)k_state_compact<EPI_NONE, Q>, A.nslices * Q,
                                                         blk, waves), blk, 0, s>>>(A);
        else if (f.epi == EPI_VERLET)
            k_state_compact<EPI_VERLET, Q><<<resident_grid(c, (const void*)k_state_compact<EPI_VERLET, Q>,
                                                           A.nslices * Q, blk, waves), blk, 0, s>>>(A);
        else
            k_state_compact<EPI_ADR, Q><<<resident_grid(c, (const void*)k_state_compact<EPI_ADR, Q>, A.nslices * Q,
                                                        blk, waves), blk, 0, s>>>(A);
    } else if (state && d3 && A.sk) {
        constexpr int Q = kStatePhases3;
        if (f.epi == EPI_NONE)
            k_state_compact3<EPI_NONE><<<resident_grid(c, (const void*)k_state_compact3<EPI_NONE>, A.nslices * Q),
                                         kForceBlock, 0, s>>>(A);
        else if (f.epi == EPI_VERLET)
            k_state_compact3<EPI_VERLET><<<resident_grid(c, (const void*)k_state_compact3<EPI_VERLET>, A.nslices * Q),
                                           kForceBlock, 0, s>>>(A);
        else
            k_state_compact3<EPI_ADR><<<resident_grid(c, (const void*)k_state_compact3<EPI_ADR>, A.nslices * Q),
                                        kForceBlock, 0, s>>>(A);
    } else if (state && d3 && f.epi == EPI_NONE) {
        constexpr int Q = kStatePhases3;
        k_state_force3_phased<Q><<<resident_grid(c, (const void*)k_state_force3_phased<Q>, A.nslices * Q), kForceBlock,
                                   0, s>>>(A);
    } else if (state) {
        PD_DISPATCH(k_state_force);
    } else {
        PD_DISPATCH(k_bond_force);
    }
#undef PD_DISPATCH
#undef PD_LAUNCH
    c->launches++;
    if (f.epi == EPI_VERLET && f.do_next) c->parity ^= 1;
    if (f.epi == EPI_VERLET && f.contact && !f.do_next) c->pos_valid = false;  // contact moved u, not P
    c->csr_fail_current = false;
    return cuda_err(c, cudaGetLastError(), "force");
}

}  // namespace pdg

namespace pdg {

int launch_adr_cnn(pd_ctx* c, cudaStream_t s) {
    ForceArgs A = make_args(c);
    const unsigned g = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((A.P.N_int + kForceBlock - 1) / kForceBlock, std::min<int64_t>(c->num_sms * 8, kMaxPartials)));
    if (A.P.dim == 2)
        k_adr_cnn<2><<<g, kForceBlock, 0, s>>>(A);
    else
        k_adr_cnn<3><<<g, kForceBlock, 0, s>>>(A);
    c->launches++;
    return cuda_err(c, cudaGetLastError(), "adr_cnn");
}

int launch_contact(pd_ctx* c, cudaStream_t s) {
    if (!c->has_cyl) return set_err(c, PD_ERR_STATE, "contact needs an impactor (pd_cylinder_init)");
    if (c->p.dim != 3) return set_err(c, PD_ERR_UNSUPPORTED, "contact is 3-D only");
    ForceArgs A = make_args(c);
    const unsigned g = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((A.P.N + kForceBlock - 1) / kForceBlock, std::min<int64_t>(c->num_sms * 8, kMaxPartials)));
    k_contact<<<g, kForceBlock, 0, s>>>(A);
    c->launches++;
    c->pos_valid = false;
    return cuda_err(c, cudaGetLastError(), "contact");
}

}  // namespace pdg
