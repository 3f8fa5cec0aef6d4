// Setup passes over the CSR bond family, and the build of the SELL-32 layout
// the force kernels read.
//
//   vol_corr          kernel_vol_Corr (Surf_Corr.cu:7-35)
//   surface_correct   surface_correct_gpu (Surf_Corr.cu:235-310): the reference
//                     runs 5-8 launches with a displacement array per test
//                     field and cudaMalloc/cudaFree temporaries; here one warp
//                     per node computes idist, fac and the strain energy of all
//                     test fields at once (u_axis = 0.001 x_axis is analytic),
//                     in a state-based context w and m as well, then one pass
//                     forms scr per bond.
//   initial_weight    kernel_initial_weight_2D/3D (Force_State.cu:8-54), in the
//                     same family pass as vol_corr (k_family_setup)
//   set_crack_*       kernel_set_crack_2D (Base_Function.cu:39-81) and the
//                     Kalthoff-Winkler notch cut (Solve_Kalthoff_Winkler.cu:40-63)
//   prepare           per-bond coefficients in SELL order (see pd_internal.cuh)
//
// This file is compiled without FMA contraction: idist, fac, w and the crack
// tests then round exactly like the reference's host code, so NL, idist, fac
// and the fail flags agree bit for bit with it.
#include <cmath>

#include "ff.cuh"
#include <algorithm>
#include <cmath>

#include "pd_internal.cuh"

namespace pdg {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return __shfl_sync(0xffffffffu, v, 0);
}

// One pass over node i's bonds, one warp per node:
//   * idist and fac per bond (kernel_vol_Corr, Surf_Corr.cu:17-32);
//   * with ENERGY, the strain energy density of node i under the test fields
//     u_a = 0.001 x_a (kernel_Disp + kernel_surface_F/_3D, Surf_Corr.cu:38-158),
//     all axes at once, and fncst_a = sedload / energy.  A batch of specimens
//     passes bc and sedload per node (its specimen's values); bonds never
//     cross specimens;
//   * with WEIGHT, w per bond and m per node (kernel_initial_weight_2D/3D,
//     Force_State.cu:8-54).
// The reference runs these as separate passes that re-read idist and fac;
// here they come from registers.  Every sum runs in the order a pass of its
// own would use (lane-strided, then the warp tree), so fused and separate
// calls give the same bits.
template <bool ENERGY, bool WEIGHT>
__global__ void k_family_setup(KParams P, double sedload, const double* __restrict__ node_bc,
                               const double* __restrict__ node_sed, const double* __restrict__ x,
                               const double* __restrict__ y, const double* __restrict__ z,
                               const int64_t* __restrict__ rowptr, const int* __restrict__ NL,
                               double* __restrict__ idist, double* __restrict__ fac, double* __restrict__ fx,
                               double* __restrict__ fy, double* __restrict__ fz, double* __restrict__ w,
                               double* __restrict__ m) {
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= P.N) return;
    if (ENERGY && node_bc) {
        P.bc = node_bc[i];
        sedload = node_sed[i];
    }
    const int dim = P.dim;
    double st[3] = {0.0, 0.0, 0.0};
    double acc = 0.0;
    const double xi = x[i], yi = y[i], zi = dim == 3 ? z[i] : 0.0;
    const double ui[3] = {0.001 * xi, 0.001 * yi, 0.001 * zi};
    for (int64_t q = rowptr[i] + lane; q < rowptr[i + 1]; q += 32) {
        const int64_t c = NL[q];
        const double xc = x[c], yc = y[c], zc = dim == 3 ? z[c] : 0.0;
        const double a0 = xc - xi, b0 = yc - yi;
        double L0;
        if (dim == 2) {
            L0 = sqrt(a0 * a0 + b0 * b0);
        } else {
            const double d0 = zc - zi;
            L0 = sqrt(a0 * a0 + b0 * b0 + d0 * d0);
        }
        idist[q] = L0;
        double f;
        if (L0 <= P.delta - P.dx / 2.0)
            f = 1.0;
        else if (L0 <= P.delta + P.dx / 2.0)
            f = (P.delta + P.dx / 2.0 - L0) / P.dx;
        else
            f = 0.0;
        fac[q] = f;
        if (ENERGY) {
            for (int a = 0; a < dim; a++) {
                // displacement only along axis a (the other components are
                // zero, and adding zero is exact, so the reference's expression
                // reduces to the plain coordinate difference on those axes)
                const double uxc = a == 0 ? 0.001 * xc : 0.0, uxi = a == 0 ? ui[0] : 0.0;
                const double uyc = a == 1 ? 0.001 * yc : 0.0, uyi = a == 1 ? ui[1] : 0.0;
                const double ddx = xc + uxc - xi - uxi;
                const double ddy = yc + uyc - yi - uyi;
                double L;
                if (dim == 2) {
                    L = sqrt(ddx * ddx + ddy * ddy);
                } else {
                    const double uzc = a == 2 ? 0.001 * zc : 0.0, uzi = a == 2 ? ui[2] : 0.0;
                    const double ddz = zc + uzc - zi - uzi;
                    L = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                }
                st[a] += 0.25 * P.bc * (L - L0) * (L - L0) / L0 * P.vol * f;
            }
        }
        if (WEIGHT) {
            const double wq = exp(-(L0 * L0) / (P.delta * P.delta));
            w[q] = wq;
            acc += wq * (L0 * L0) * P.vol * f;
        }
    }
    if (ENERGY) {
        const double sx = warp_sum(st[0]);
        const double sy = warp_sum(st[1]);
        const double sz = warp_sum(st[2]);
        if (lane == 0) {
            fx[i] = sedload / sx;
            fy[i] = sedload / sy;
            if (dim == 3) fz[i] = sedload / sz;
        }
    }
    if (WEIGHT) {
        acc = warp_sum(acc);
        if (lane == 0) m[i] = acc;
    }
}

// scr per bond (kernel_cal_surf_coff_F, Surf_Corr.cu:160-232).
__global__ void k_surface_coeff(KParams P, const double* __restrict__ x, const double* __restrict__ y,
                                const double* __restrict__ z, const int64_t* __restrict__ rowptr,
                                const int* __restrict__ NL, const double* __restrict__ idist,
                                const double* __restrict__ fnx, const double* __restrict__ fny,
                                const double* __restrict__ fnz, double* __restrict__ scr) {
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= P.N) return;
    const double half_pi = 90.0 * P.pi / 180.0;
    for (int64_t q = rowptr[i] + lane; q < rowptr[i + 1]; q += 32) {
        const int64_t c = NL[q];
        const double scx = (fnx[i] + fnx[c]) / 2.0;
        const double scy = (fny[i] + fny[c]) / 2.0;
        const double adx = fabs(x[c] - x[i]), ady = fabs(y[c] - y[i]);
        if (P.dim == 2) {
            double th;
            if (ady <= 1.0e-10)
                th = 0.0;
            else if (adx <= 1.0e-10)
                th = half_pi;
            else
                th = atan(ady / adx);
            scr[q] = sqrt(1.0 / (cos(th) * cos(th) / (scx * scx) + sin(th) * sin(th) / (scy * scy)));
        } else {
            const double scz = (fnz[i] + fnz[c]) / 2.0;
            const double adz = fabs(z[c] - z[i]);
            if (adz < 1.0e-10) {
                double th;
                if (ady < 1.0e-10)
                    th = 0.0;
                else if (adx < 1.0e-10)
                    th = half_pi;
                else
                    th = atan(ady / adx);
                const double phi = half_pi;
                scr[q] = sqrt(1.0 / (cos(th) * cos(th) / (scx * scx) + sin(th) * sin(th) / (scy * scy) +
                                     cos(phi) * cos(phi) / (scz * scz)));
            } else if (adx < 1.0e-10 && ady < 1.0e-10) {
                scr[q] = scz;
            } else {
                const double th = atan(ady / adx);
                const double phi = acos(adz / idist[q]);
                scr[q] = sqrt(1.0 / (cos(th) * cos(th) / (scx * scx) + sin(th) * sin(th) / (scy * scy) +
                                     cos(phi) * cos(phi) / (scz * scz)));
            }
        }
    }
}

// Pre-crack segment test (Base_Function.cu:39-81) on nodes [r0, r1)
// (the reference tests [0, N_int); a batch cracks one specimen at a time).
__global__ void k_set_crack_2d(KParams P, int64_t r0, int64_t r1, double clength, double lx, double ly,
                               double theta, const double* __restrict__ x, const double* __restrict__ y,
                               const int64_t* __restrict__ rowptr, const int* __restrict__ NL,
                               int* __restrict__ fail) {
    const int64_t i = r0 + ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= r1) return;
    for (int64_t q = rowptr[i] + lane; q < rowptr[i + 1]; q += 32) {
        const int64_t c = NL[q];
        if (fabs(theta - P.pi / 2.0) < 0.0001) {
            if (fabs(y[c] - ly) < clength * sin(theta) / 2.0 && fabs(y[i] - ly) < clength * sin(theta) / 2.0)
                if ((x[c] - lx) * (x[i] - lx) < 0.0) fail[q] = 0;
        } else {
            const double t = tan(theta);
            const double dist_c = (y[c] - ly) * (y[c] - ly) + (x[c] - lx) * (x[c] - lx);
            const double dist_i = (y[i] - ly) * (y[i] - ly) + (x[i] - lx) * (x[i] - lx);
            const double vc0 = (t * x[c] - y[c] - lx * t + ly) / sqrt(1 + t * t);
            const double vi0 = (t * x[i] - y[i] - lx * t + ly) / sqrt(1 + t * t);
            const double len_c = sqrt(dist_c - vc0 * vc0);
            const double len_i = sqrt(dist_i - vi0 * vi0);
            if (len_c < clength / 2.0 && len_i < clength / 2.0) {
                const double bcn = t * x[c] - lx * t + ly - y[c];
                const double bi = t * x[i] - lx * t + ly - y[i];
                if (bcn * bi <= 0) fail[q] = 0;
            }
        }
    }
}

// Notch cut of the Kalthoff-Winkler slab (Solve_Kalthoff_Winkler.cu:40-63).
__global__ void k_set_crack_kw(KParams P, double rad, const double* __restrict__ x, const double* __restrict__ y,
                               const int64_t* __restrict__ rowptr, const int* __restrict__ NL,
                               int* __restrict__ fail) {
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= P.N_int) return;
    for (int64_t q = rowptr[i] + lane; q < rowptr[i + 1]; q += 32) {
        const int64_t c = NL[q];
        const bool upper = (y[c] >= -1.0e-10) | (y[i] >= -1.0e-10);
        if (((x[c] > -rad && x[i] < -rad) | (x[i] > -rad && x[c] < -rad)) && upper) fail[q] = 0;
        if (((x[c] > rad && x[i] < rad) | (x[i] > rad && x[c] < rad)) && upper) fail[q] = 0;
    }
}

// ---- SELL-32 layout -------------------------------------------------------

__global__ void k_slice_width(int64_t N, int64_t nslices, const int* __restrict__ NN, int* __restrict__ width) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int64_t r = s * 32 + lane;
    int v = r < N ? NN[r] : 0;
    for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, off));
    if (lane == 0) width[s] = v;
}

// The reference vector xa rounded to float per component (xf, z = 0 in 2-D)
// and the exact constant |xf|^2 - l0^2 as a float pair (c0): products of
// floats are exact doubles, and the sums are carried as double pairs
// (TwoSum / FMA TwoProduct); sh - ph is exact, both within a factor 2 of
// l0^2.  l0 itself as a float pair (lf).
__device__ void float_reference(const double xa[3], int dim, double L0, float xf[3], float2& c0, float2& lf) {
    double sh = 0.0, sl = 0.0;
    xf[2] = 0.0f;
    for (int a = 0; a < dim; a++) {
        const float f = __double2float_rn(xa[a]);
        xf[a] = f;
        const double sq = (double)f * (double)f;  // exact: 24-bit x 24-bit mantissas
        const double t = sh + sq;
        const double bb = t - sh;
        sl += (sh - (t - bb)) + (sq - bb);
        sh = t;
    }
    const double ph = L0 * L0;
    const double pl = fma(L0, L0, -ph);
    const ff cf = ff_split((sh - ph) + (sl - pl));
    c0 = make_float2(cf.h, cf.l);
    const ff l = ff_split(L0);
    lf = make_float2(l.h, l.l);
}

// One thread per slot.  Padding slots point at their own row, carry zero
// coefficients and a cleared intact bit, so they contribute nothing.
__global__ void k_sell_fill(KParams P, int64_t nslices, const int* __restrict__ width,
                            const int64_t* __restrict__ base, const int* __restrict__ NN,
                            const int64_t* __restrict__ rowptr, const int* __restrict__ NL,
                            const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                            const double* __restrict__ idist, const double* __restrict__ fac,
                            const double* __restrict__ scr, const double* __restrict__ w, const double* __restrict__ m,
                            const double* __restrict__ node_bc, const double* __restrict__ node_s0, Sell S) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int k = t >> 5, l = t & 31;
        const int64_t r = s * 32 + l;
        const int64_t slot = b + t;
        const bool used = r < P.N && k < NN[r];
        const int64_t q = used ? rowptr[r] + k : -1;
        S.csr[slot] = (int)(used ? q : -1);
        if (!used) {
            if (S.rec) {
                BondRec R;
                R.col = (int)(r < P.N ? r : 0);
                R.xf[0] = R.xf[1] = R.xf[2] = 0.0f;
                R.c0 = make_float2(0.0f, 0.0f);
                R.l0 = make_float2(1.0f, 0.0f);
                R.k2 = make_float2(0.0f, 0.0f);
                R.ecrit = HUGE_VAL;
                S.rec[slot] = R;
            }
            if (S.sgeo) {
                StateGeo G{};
                G.col = (int)(r < P.N ? r : 0);
                G.l0 = make_float2(1.0f, 0.0f);
                S.sgeo[slot] = G;
                S.sth[slot] = StateTheta{};
                StateForce F{};
                F.ecrit = HUGE_VAL;
                S.sfo[slot] = F;
                S.e[slot] = make_float2(0.0f, 0.0f);
            }
            continue;
        }
        const int64_t c = NL[q];
        const double L0 = idist[q];
        // break when s = (L - L0)/L0 > s0, i.e. e = L - L0 > s0 L0; the 3-D
        // kernels break only bonds whose ends both have y >= -0.04 (Force_Bond.cu:117)
        bool breakable = true;
        if (P.dim == 3) breakable = y[r] >= P.break_ymin && y[c] >= P.break_ymin;
        // a batch of specimens carries bc and s0 per node (the row's specimen)
        const double s0 = node_s0 ? node_s0[r] : P.critical_s;
        const double bc = node_bc ? node_bc[r] : P.bc;
        const double ecrit = breakable ? s0 * L0 : HUGE_VAL;
        if (S.rec) {
            const double k2 = 2.0 * (P.vol * fac[q] * bc * scr[q]) / L0;
            BondRec R;
            R.col = (int)c;
            R.ecrit = ecrit;
            const ff kf = ff_split(k2 * S.kscale_inv);
            R.k2 = make_float2(kf.h, kf.l);
            const double xa[3] = {x[c] - x[r], y[c] - y[r], P.dim == 3 ? z[c] - z[r] : 0.0};
            float_reference(xa, P.dim, L0, R.xf, R.c0, R.l0);
            S.rec[slot] = R;
        }
        if (S.sgeo) {
            const double pr = P.pratio;
            double a_coef, b_coef, th_coef;
            if (P.dim == 2) {
                a_coef = (2.0 * pr - 1.0) / (pr - 1.0) * (2.0 * P.K - 32.0 * P.G / 9.0);
                b_coef = 8.0 * P.G;
                th_coef = 2.0 * (2.0 * pr - 1.0) / (pr - 1.0);
            } else {
                a_coef = 3.0 * P.K - 5.0 * P.G;  // 3K th w L0/m + 15G/m w (e - th L0/3)
                b_coef = 15.0 * P.G;
                th_coef = 3.0;
            }
            const double wf = w[q] * fac[q] * P.vol;
            StateTheta T;
            T.xi[0] = x[c] - x[r];
            T.xi[1] = y[c] - y[r];
            T.xi[2] = P.dim == 3 ? z[c] - z[r] : 0.0;
            // the coefficients as float pairs, scaled by powers of two (exact)
            const ff cth = ff_split(th_coef * w[q] * L0 * fac[q] * P.vol * ldexp(1.0, S.sth_exp));
            T.cth = make_float2(cth.h, cth.l);
            StateGeo G;
            G.col = (int)c;
            float_reference(T.xi, P.dim, L0, G.xf, G.c0, G.l0);
            StateForce F;
            const double cs = ldexp(1.0, S.sn_exp - S.st_exp);
            const ff c1 = ff_split(2.0 * a_coef * wf * L0 * cs), c2 = ff_split(2.0 * b_coef * wf * cs);
            F.c1 = make_float2(c1.h, c1.l);
            F.c2 = make_float2(c2.h, c2.l);
            F.ecrit = ecrit;
            F.xiz = T.xi[2];
            S.sgeo[slot] = G;
            S.sth[slot] = T;
            S.sfo[slot] = F;
            S.e[slot] = make_float2(0.0f, 0.0f);
        }
    }
}

// ---- compact layout of the 2-D bond-based kernels ---------------------------
//
// Offset classes: the bonds of one specimen whose reference vectors round to
// the same float vector xf (on a lattice, one class per lattice offset).  A
// hash table in device memory, one region of kRegion slots per specimen (a
// single plate is one specimen), collects the classes with the smallest bond
// length of each (l0t); the host numbers them per specimen in key order
// (deterministic, and the same for a plate alone and inside a batch) and
// builds one template per class; each slot then stores dl = l0 - l0t, the
// class id and k2 / 2 in a 16-byte record (bondtpl.h).

constexpr int kRegion = 256;  // hash slots per specimen (power of two)
constexpr unsigned long long kEmptyKey = ~0ull;

__device__ __forceinline__ unsigned long long class_key(double xa, double ya) {
    return ((unsigned long long)__float_as_uint(__double2float_rn(xa)) << 32) |
           (unsigned long long)__float_as_uint(__double2float_rn(ya));
}
__device__ __forceinline__ unsigned class_hash(unsigned long long k) {
    return (unsigned)((k * 0x9E3779B97F4A7C15ull) >> 56);  // 8 bits
}
// 3-D: a 64-bit mix of the three float components.  Not injective: the
// inserting thread stores its float vector beside the key, and the record
// fill checks every member's vector against its class's (a collision makes
// the layout unsupported, never a wrong class).
__device__ __forceinline__ unsigned long long class_key3(double xa, double ya, double za) {
    unsigned long long k = ((unsigned long long)__float_as_uint(__double2float_rn(xa)) << 32) |
                           (unsigned long long)__float_as_uint(__double2float_rn(ya));
    k ^= (unsigned long long)__float_as_uint(__double2float_rn(za)) * 0xD6E8FEB86659FD93ull;
    k ^= k >> 31;
    k *= 0xBF58476D1CE4E5B9ull;
    k ^= k >> 29;
    return k == kEmptyKey ? 0ull : k;
}

// z null: 2-D keys (the float vector itself); otherwise 3-D keys, and the
// thread that inserts a key writes its float vector into vec.
__global__ void k_class_insert(int64_t nslices, const int* __restrict__ width, const int64_t* __restrict__ base,
                               const int* __restrict__ csr, const int* __restrict__ NL, const int* __restrict__ grp,
                               const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, const double* __restrict__ idist,
                               unsigned long long* __restrict__ keys, unsigned long long* __restrict__ l0min,
                               float4* __restrict__ vec, int* __restrict__ overflow) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int q = csr[b + t];
        if (q < 0) continue;
        const int64_t r = s * 32 + (t & 31), c = NL[q];
        const int64_t region = grp ? grp[r] : 0;
        const double xa = x[c] - x[r], ya = y[c] - y[r], za = z ? z[c] - z[r] : 0.0;
        const unsigned long long key = z ? class_key3(xa, ya, za) : class_key(xa, ya);
        const unsigned long long lb = (unsigned long long)__double_as_longlong(idist[q]);
        unsigned h = class_hash(key);
        bool done = false;
        for (int probe = 0; probe < kRegion && !done; probe++, h = (h + 1) & (kRegion - 1)) {
            const int64_t i = region * kRegion + h;
            const unsigned long long prev = atomicCAS(keys + i, kEmptyKey, key);
            if (prev == kEmptyKey || prev == key) {
                atomicMin(l0min + i, lb);  // positive doubles order like their bit patterns
                if (prev == kEmptyKey && vec)
                    vec[i] = make_float4(__double2float_rn(xa), __double2float_rn(ya), __double2float_rn(za), 0.0f);
                done = true;
            }
        }
        if (!done) atomicExch(overflow, 1);
    }
}

// Records of the compact layout; *bad is set where a slot cannot be
// represented (dl not a float with a free low byte).
__global__ void k_rec16_fill(KParams P, int64_t nslices, const int* __restrict__ width,
                             const int64_t* __restrict__ base, const int* __restrict__ csr, const int* __restrict__ NL,
                             const int* __restrict__ grp, const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ idist, const double* __restrict__ fac,
                             const double* __restrict__ scr, const double* __restrict__ node_bc,
                             const unsigned long long* __restrict__ keys, const int* __restrict__ ids,
                             const int* __restrict__ inst_tbase, const bt::Tpl* __restrict__ tpl,
                             double kscale_half_inv, bt::Rec* __restrict__ rec, int* __restrict__ bad) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int64_t slot = b + t;
        const int q = csr[slot];
        const int64_t r = s * 32 + (t & 31);
        bt::Rec R;
        if (q < 0) {
            R.col = (int)(r < P.N ? r : 0);
            R.dl = 0.0f;  // class 0, zero coefficient: a padding slot contributes nothing
            R.k2h = R.k2l = 0.0f;
            rec[slot] = R;
            continue;
        }
        const int64_t c = NL[q];
        const int64_t region = grp ? grp[r] : 0;
        const unsigned long long key = class_key(x[c] - x[r], y[c] - y[r]);
        unsigned h = class_hash(key);
        int id = -1;
        for (int probe = 0; probe < kRegion; probe++, h = (h + 1) & (kRegion - 1)) {
            const int64_t i = region * kRegion + h;
            if (keys[i] == key) {
                id = ids[i];
                break;
            }
            if (keys[i] == kEmptyKey) break;
        }
        const double L0 = idist[q];
        const int64_t tb = inst_tbase ? inst_tbase[region] : 0;
        const double dlv = id >= 0 ? L0 - tpl[tb + id].l0d : 0.0;  // exact: l0 and l0t within a factor two
        const float dl = __double2float_rn(dlv);
        const unsigned dlb = __float_as_uint(dl);
        if (id < 0 || id > 255 || (double)dl != dlv || (dlb & 0xffu) != 0u) atomicExch(bad, 1);
        R.col = (int)c;
        R.dl = __uint_as_float((dlb & ~0xffu) | (unsigned)(id & 0xff));
        const double bc = node_bc ? node_bc[r] : P.bc;
        const double k2 = 2.0 * (P.vol * fac[q] * bc * scr[q]) / L0;
        const ff kf = ff_split(k2 * kscale_half_inv);
        R.k2h = kf.h;
        R.k2l = kf.l;
        rec[slot] = R;
    }
}

// The coefficients of one state-based bond (the state records of
// k_sell_fill), with the context's power-of-two scales, in doubles.
__device__ __forceinline__ void state_coefs(const KParams& P, double L0, double w, double fac, int sn_exp,
                                            int sth_exp, int st_exp, double& cth, double& c1, double& c2) {
    const double pr = P.pratio;
    double a_coef, b_coef, th_coef;
    if (P.dim == 2) {
        a_coef = (2.0 * pr - 1.0) / (pr - 1.0) * (2.0 * P.K - 32.0 * P.G / 9.0);
        b_coef = 8.0 * P.G;
        th_coef = 2.0 * (2.0 * pr - 1.0) / (pr - 1.0);
    } else {
        a_coef = 3.0 * P.K - 5.0 * P.G;  // 3K th w L0/m + 15G/m w (e - th L0/3)
        b_coef = 15.0 * P.G;
        th_coef = 3.0;
    }
    const double wf = w * fac * P.vol;
    cth = th_coef * w * L0 * fac * P.vol * ldexp(1.0, sth_exp);
    const double cs = ldexp(1.0, sn_exp - st_exp);
    c1 = 2.0 * a_coef * wf * L0 * cs;
    c2 = 2.0 * b_coef * wf * cs;
}

// Records of the 3-D bond-based compact layout: {column, dl with the class
// id, k2 / 2 as a pair}, the pair negated where the bond may not break (an
// end below y = -0.04, Force_Bond.cu:117).  *bad as in k_rec16_fill, and also
// where a slot's float vector is not its class's (a key collision).
__global__ void k_rec16_fill3(KParams P, int64_t nslices, const int* __restrict__ width,
                              const int64_t* __restrict__ base, const int* __restrict__ csr,
                              const int* __restrict__ NL, const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z, const double* __restrict__ idist,
                              const double* __restrict__ fac, const double* __restrict__ scr,
                              const unsigned long long* __restrict__ keys, const int* __restrict__ ids,
                              const bt::Tpl3* __restrict__ tpl, double kscale_half_inv, bt::Rec* __restrict__ rec,
                              int* __restrict__ bad) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int64_t slot = b + t;
        const int q = csr[slot];
        const int64_t r = s * 32 + (t & 31);
        bt::Rec R;
        if (q < 0) {
            R.col = (int)(r < P.N ? r : 0);
            R.dl = 0.0f;  // class 0, zero coefficient: a padding slot contributes nothing
            R.k2h = R.k2l = 0.0f;
            rec[slot] = R;
            continue;
        }
        const int64_t c = NL[q];
        const double xv[3] = {x[c] - x[r], y[c] - y[r], z[c] - z[r]};
        const unsigned long long key = class_key3(xv[0], xv[1], xv[2]);
        unsigned h = class_hash(key);
        int id = -1;
        for (int probe = 0; probe < kRegion; probe++, h = (h + 1) & (kRegion - 1)) {
            if (keys[h] == key) {
                id = ids[h];
                break;
            }
            if (keys[h] == kEmptyKey) break;
        }
        bool fail = id < 0 || id > 255;
        const double L0 = idist[q];
        double dlv = 0.0;
        if (!fail) {
            const bt::Tpl3& T = tpl[id];
            dlv = L0 - T.l0d;
            for (int a = 0; a < 3; a++)
                if (__double2float_rn(xv[a]) != T.xf[a]) fail = true;  // another vector under the same key
        }
        const float dl = __double2float_rn(dlv);
        const unsigned dlb = __float_as_uint(dl);
        if ((double)dl != dlv || (dlb & 0xffu) != 0u) fail = true;
        if (fail) atomicExch(bad, 1);
        R.col = (int)c;
        R.dl = __uint_as_float((dlb & ~0xffu) | (unsigned)(id & 0xff));
        const double k2 = 2.0 * (P.vol * fac[q] * P.bc * scr[q]) / L0;
        const ff kf = ff_split(k2 * kscale_half_inv);
        const bool breakable = y[r] >= P.break_ymin && y[c] >= P.break_ymin;
        R.k2h = breakable ? kf.h : -kf.h;
        R.k2l = breakable ? kf.l : -kf.l;
        rec[slot] = R;
    }
}

// Records of the 2-D state-based compact layout: rec = {column, dl with the
// class id, kx, ky}, where the reference vector x_c - x_i as the reference
// rounds it (a double) is the class's float vector (as a double) moved by kx
// and ky representable doubles (the difference of the bit patterns); rec8 =
// {column, dl with the class id}.  A slot whose bond has the class's
// reference length (dl = 0; every class has one) writes the class's
// coefficients into stpl (such slots compute identical values).  *bad as in
// k_rec16_fill, and also where kx or ky leaves the int32 range or the signs
// differ.
__global__ void k_state_compact_fill(KParams P, int64_t nslices, const int* __restrict__ width,
                                     const int64_t* __restrict__ base, const int* __restrict__ csr,
                                     const int* __restrict__ NL, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ idist,
                                     const double* __restrict__ fac, const double* __restrict__ w,
                                     const unsigned long long* __restrict__ keys, const int* __restrict__ ids,
                                     const bt::Tpl* __restrict__ tpl, int sn_exp, int sth_exp, int st_exp,
                                     int4* __restrict__ rec, int2* __restrict__ rec8, StateTpl* __restrict__ stpl,
                                     int* __restrict__ bad) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int64_t slot = b + t;
        const int q = csr[slot];
        const int64_t r = s * 32 + (t & 31);
        if (q < 0) {
            const int col = (int)(r < P.N ? r : 0);
            rec[slot] = make_int4(col, 0, 0, 0);
            rec8[slot] = make_int2(col, 0);
            continue;
        }
        const int64_t c = NL[q];
        const double xa = x[c] - x[r], ya = y[c] - y[r];  // the reference's rounding (Force_State.cu:71-72)
        const unsigned long long key = class_key(xa, ya);
        unsigned h = class_hash(key);
        int id = -1;
        for (int probe = 0; probe < kRegion; probe++, h = (h + 1) & (kRegion - 1)) {
            if (keys[h] == key) {
                id = ids[h];
                break;
            }
            if (keys[h] == kEmptyKey) break;
        }
        const double L0 = idist[q];
        const double dlv = id >= 0 ? L0 - tpl[id].l0d : 0.0;
        const float dl = __double2float_rn(dlv);
        const unsigned dlb = __float_as_uint(dl);
        bool fail = id < 0 || id > 255 || (double)dl != dlv || (dlb & 0xffu) != 0u;
        long long k[2] = {0, 0};
        if (!fail) {
            const double xv[2] = {xa, ya};
            for (int a = 0; a < 2; a++) {
                const long long xb = (long long)tpl[id].xd[a];
                const long long vb = __double_as_longlong(xv[a]);
                k[a] = vb - xb;
                if ((vb < 0) != (xb < 0) || k[a] < INT_MIN || k[a] > INT_MAX) fail = true;
            }
        }
        if (fail) atomicExch(bad, 1);
        const int dlw = (int)((dlb & ~0xffu) | (unsigned)(id & 0xff));
        rec[slot] = make_int4((int)c, dlw, (int)k[0], (int)k[1]);
        rec8[slot] = make_int2((int)c, dlw);
        if (!fail && dlv == 0.0) {
            double cth, c1, c2;
            state_coefs(P, L0, w[q], fac[q], sn_exp, sth_exp, st_exp, cth, c1, c2);
            const ff a = ff_split(c1), bb = ff_split(c2), t3 = ff_split(cth);
            StateTpl& T = stpl[id];  // g1, g2 come from the host
            T.c1h = a.h, T.c1l = a.l, T.c2h = bb.h, T.c2l = bb.l;
            T.cth_h = t3.h, T.cth_l = t3.l;
        }
    }
}

// Records of the 3-D state-based compact layout: rec8 = {column, dl with
// the class id}; sk = {kx, ky, kz, flags} (the reference vector x_c - x_i as
// the class's float vector moved by kx, ky, kz representable doubles; flags
// bit 0: the bond may break, both ends at y >= -0.04, Force_State.cu:283);
// skz = {kz, flags}.  The class coefficients come from the slots with dl = 0
// as in k_state_compact_fill.  *bad also where a slot's float vector is not
// its class's (a key collision).
__global__ void k_state_compact3_fill(KParams P, int64_t nslices, const int* __restrict__ width,
                                      const int64_t* __restrict__ base, const int* __restrict__ csr,
                                      const int* __restrict__ NL, const double* __restrict__ x,
                                      const double* __restrict__ y, const double* __restrict__ z,
                                      const double* __restrict__ idist, const double* __restrict__ fac,
                                      const double* __restrict__ w, const unsigned long long* __restrict__ keys,
                                      const int* __restrict__ ids, const bt::Tpl3* __restrict__ tpl, int sn_exp,
                                      int sth_exp, int st_exp, int2* __restrict__ rec8, int4* __restrict__ sk,
                                      int2* __restrict__ skz, StateTpl* __restrict__ stpl, int* __restrict__ bad) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int64_t slot = b + t;
        const int q = csr[slot];
        const int64_t r = s * 32 + (t & 31);
        if (q < 0) {
            rec8[slot] = make_int2((int)(r < P.N ? r : 0), 0);
            sk[slot] = make_int4(0, 0, 0, 0);
            skz[slot] = make_int2(0, 0);
            continue;
        }
        const int64_t c = NL[q];
        // the reference's roundings of the reference vector (Force_State.cu:217-219)
        const double xv[3] = {x[c] - x[r], y[c] - y[r], z[c] - z[r]};
        const unsigned long long key = class_key3(xv[0], xv[1], xv[2]);
        unsigned h = class_hash(key);
        int id = -1;
        for (int probe = 0; probe < kRegion; probe++, h = (h + 1) & (kRegion - 1)) {
            if (keys[h] == key) {
                id = ids[h];
                break;
            }
            if (keys[h] == kEmptyKey) break;
        }
        bool fail = id < 0 || id > 255;
        const double L0 = idist[q];
        double dlv = 0.0;
        long long k[3] = {0, 0, 0};
        if (!fail) {
            const bt::Tpl3& T = tpl[id];
            dlv = L0 - T.l0d;
            for (int a = 0; a < 3; a++) {
                if (__double2float_rn(xv[a]) != T.xf[a]) fail = true;  // another vector under the same key
                const long long xb = (long long)T.xd[a];
                const long long vb = __double_as_longlong(xv[a]);
                k[a] = vb - xb;
                if ((vb < 0) != (xb < 0) || k[a] < INT_MIN || k[a] > INT_MAX) fail = true;
            }
        }
        const float dl = __double2float_rn(dlv);
        const unsigned dlb = __float_as_uint(dl);
        if ((double)dl != dlv || (dlb & 0xffu) != 0u) fail = true;
        if (fail) atomicExch(bad, 1);
        const int dlw = (int)((dlb & ~0xffu) | (unsigned)(id & 0xff));
        const int flags = (y[r] >= P.break_ymin && y[c] >= P.break_ymin) ? 1 : 0;
        rec8[slot] = make_int2((int)c, dlw);
        sk[slot] = make_int4((int)k[0], (int)k[1], (int)k[2], flags);
        skz[slot] = make_int2((int)k[2], flags);
        if (!fail && dlv == 0.0) {
            double cth, c1, c2;
            state_coefs(P, L0, w[q], fac[q], sn_exp, sth_exp, st_exp, cth, c1, c2);
            const ff a = ff_split(c1), bb = ff_split(c2), t3 = ff_split(cth);
            StateTpl& T = stpl[id];  // g1, g2 come from the host
            T.c1h = a.h, T.c1l = a.l, T.c2h = bb.h, T.c2l = bb.l;
            T.cth_h = t3.h, T.cth_l = t3.l;
        }
    }
}

// The "may break" flags of the 3-D state-based records as one bit word per
// (slice, slot), like the intact flags.
__global__ void k_break_bits(int64_t nslices, const int* __restrict__ width, const int64_t* __restrict__ base,
                             const int64_t* __restrict__ fbase, const int2* __restrict__ skz,
                             uint32_t* __restrict__ bbits) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int W = width[s];
    for (int k = 0; k < W; k++) {
        const uint32_t word = __ballot_sync(0xffffffffu, (skz[base[s] + (int64_t)k * 32 + lane].y & 1) != 0);
        if (lane == 0) bbits[fbase[s] + k] = word;
    }
}

// Every slot's coefficients against its class's moved to the slot's length
// (c (1 + g dl)): *bad where one differs from the bond's own by more than
// 2^-45 of it.
__global__ void k_state_compact_check(KParams P, int64_t nslices, const int* __restrict__ width,
                                      const int64_t* __restrict__ base, const int* __restrict__ csr,
                                      const double* __restrict__ idist, const double* __restrict__ fac,
                                      const double* __restrict__ w, const int2* __restrict__ rec8,
                                      const StateTpl* __restrict__ stpl, int sn_exp, int sth_exp, int st_exp,
                                      int* __restrict__ bad) {
    const int64_t s = blockIdx.y * (int64_t)gridDim.x + blockIdx.x;
    if (s >= nslices) return;
    const int W = width[s];
    const int64_t b = base[s];
    for (int t = threadIdx.x; t < W * 32; t += blockDim.x) {
        const int64_t slot = b + t;
        const int q = csr[slot];
        if (q < 0) continue;
        const unsigned dlb = (unsigned)rec8[slot].y;
        const StateTpl T = stpl[dlb & 0xffu];
        const double dl = (double)__uint_as_float(dlb & ~0xffu);
        double cth, c1, c2;
        state_coefs(P, idist[q], w[q], fac[q], sn_exp, sth_exp, st_exp, cth, c1, c2);
        const double tol = ldexp(1.0, -45);
        const double f1 = 1.0 + (double)T.g1 * dl, f2 = 1.0 + (double)T.g2 * dl;
        const double d1 = fabs(((double)T.c1h + (double)T.c1l) * f1 - c1);
        const double d2 = fabs(((double)T.c2h + (double)T.c2l) * f2 - c2);
        const double d3 = fabs(((double)T.cth_h + (double)T.cth_l) * f1 - cth);
        if (!(d1 <= tol * fabs(c1)) || !(d2 <= tol * fabs(c2)) || !(d3 <= tol * fabs(cth))) atomicExch(bad, 1);
    }
}

// Intact flags: CSR int32 <-> SELL bit words.
__global__ void k_bits_from_csr(int64_t nslices, const int* __restrict__ width, const int64_t* __restrict__ base,
                                const int64_t* __restrict__ fbase, const int* __restrict__ csr,
                                const int* __restrict__ fail, int64_t n_rows_breakable, uint32_t* __restrict__ bits) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int W = width[s];
    for (int k = 0; k < W; k++) {
        const int64_t slot = base[s] + k * 32 + lane;
        const int q = csr[slot];
        // rows past N_int have no fail storage in the reference (Memory.cu:39):
        // their bonds count as intact
        const bool alive = q >= 0 && ((s * 32 + lane) >= n_rows_breakable || fail[q] == 1);
        const uint32_t word = __ballot_sync(0xffffffffu, alive);
        if (lane == 0) bits[fbase[s] + k] = word;
    }
}

__global__ void k_csr_from_bits(int64_t nslices, const int* __restrict__ width, const int64_t* __restrict__ base,
                                const int64_t* __restrict__ fbase, const int* __restrict__ csr,
                                const uint32_t* __restrict__ bits, int* __restrict__ fail) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslices) return;
    const int W = width[s];
    for (int k = 0; k < W; k++) {
        const int64_t slot = base[s] + k * 32 + lane;
        const int q = csr[slot];
        if (q >= 0) fail[q] = (bits[fbase[s] + k] >> lane) & 1u;
    }
}

// 1/m per node (IEEE-rounded, the dilatation pass's divisor reciprocal) and
// the same times 2^-sn as a float pair (the force pass's operand).
__global__ void k_inv_m(int64_t N, const double* __restrict__ m, double sn_scale, double* __restrict__ inv,
                        float4* __restrict__ nab) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) {
        const double v = 1.0 / m[i];
        inv[i] = v;
        const ff p = ff_split(v * sn_scale);
        reinterpret_cast<float2*>(nab + i)[1] = make_float2(p.h, p.l);  // the second pair of {theta/m, 1/m}
    }
}

unsigned warps_grid(int64_t nwarps) { return (unsigned)((nwarps * 32 + 255) / 256); }

template <typename T>
void free_ptr(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

// The family pass with the stages asked for (energy: the surface test
// fields; weight: w and m); idist and fac are always written.
template <bool ENERGY, bool WEIGHT>
static void launch_family_setup(pd_ctx* c, const KParams& P, cudaStream_t s) {
    const double sedload = P.dim == 3 ? 0.6 * P.emod * 1.0e-6 : 0.5 * P.emod / (1.0 - P.pratio * P.pratio) * 1.0e-6;
    k_family_setup<ENERGY, WEIGHT><<<warps_grid(P.N), 256, 0, s>>>(
        P, sedload, c->batch.node_bc, c->batch.node_sed, c->nf[PD_F_X], c->nf[PD_F_Y], c->nf[PD_F_Z], c->rowptr, c->NL,
        c->idist, c->fac, c->nf[PD_F_FNCST_X], c->nf[PD_F_FNCST_Y], c->nf[PD_F_FNCST_Z], c->w, c->nf[PD_F_M]);
    c->launches++;
}

int vol_corr(pd_ctx* c, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "vol_corr needs the bond family");
    launch_family_setup<false, false>(c, kparams(c->p), s);
    c->volcorr = true;
    c->prepared = false;
    return cuda_err(c, cudaGetLastError(), "vol_corr");
}

// vol_Corr and the surface energies in one family pass, then the coefficient
// pass (scr of a bond needs both end nodes' fncst: a grid-wide dependency).
// A state-based context also gets w and m from the first pass.
int surface_correct(pd_ctx* c, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "surface_correct needs the bond family");
    const KParams P = kparams(c->p);
    const bool state = c->p.model == PD_MODEL_STATE;
    if (state)
        launch_family_setup<true, true>(c, P, s);
    else
        launch_family_setup<true, false>(c, P, s);
    double *X = c->nf[PD_F_X], *Y = c->nf[PD_F_Y], *Z = c->nf[PD_F_Z];
    k_surface_coeff<<<warps_grid(P.N), 256, 0, s>>>(P, X, Y, Z, c->rowptr, c->NL, c->idist, c->nf[PD_F_FNCST_X],
                                                     c->nf[PD_F_FNCST_Y], c->nf[PD_F_FNCST_Z], c->scr);
    c->launches++;
    c->volcorr = c->surfcorr = true;
    c->weights = c->weights || state;
    c->prepared = false;
    return cuda_err(c, cudaGetLastError(), "surface_correct");
}

// w and m in the family pass, which also (re)writes idist and fac: after a
// vol_corr call the same values again, without one the call stands for both.
int initial_weight(pd_ctx* c, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "initial_weight needs the bond family");
    launch_family_setup<false, true>(c, kparams(c->p), s);
    c->volcorr = true;
    c->weights = true;
    c->prepared = false;
    return cuda_err(c, cudaGetLastError(), "initial_weight");
}

int sync_fail_to_csr(pd_ctx* c, cudaStream_t s) {
    if (c->csr_fail_current) return PD_OK;
    const Sell& S = c->sell;
    k_csr_from_bits<<<warps_grid(S.nslices), 256, 0, s>>>(S.nslices, S.width, S.base, S.fbase, S.csr, S.bits,
                                                           c->fail);
    c->launches++;
    c->csr_fail_current = true;
    return cuda_err(c, cudaGetLastError(), "fail flags to CSR");
}

int sync_fail_to_bits(pd_ctx* c, cudaStream_t s) {
    if (c->bits_current) return PD_OK;
    const Sell& S = c->sell;
    k_bits_from_csr<<<warps_grid(S.nslices), 256, 0, s>>>(S.nslices, S.width, S.base, S.fbase, S.csr, c->fail,
                                                           c->p.N_int, S.bits);
    c->launches++;
    c->bits_current = true;
    return cuda_err(c, cudaGetLastError(), "fail flags to bits");
}

int set_crack_2d_rows(pd_ctx* c, int64_t r0, int64_t r1, double clength, double lx, double ly, double theta,
                      cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "set_crack needs the bond family");
    if (r0 < 0 || r1 > c->p.N || r0 > r1) return set_err(c, PD_ERR_ARG, "set_crack row range out of bounds");
    if (r0 == r1) return PD_OK;
    int rc = sync_fail_to_csr(c, s);
    if (rc) return rc;
    const KParams P = kparams(c->p);
    k_set_crack_2d<<<warps_grid(r1 - r0), 256, 0, s>>>(P, r0, r1, clength, lx, ly, theta, c->nf[PD_F_X],
                                                        c->nf[PD_F_Y], c->rowptr, c->NL, c->fail);
    c->launches++;
    c->bits_current = false;
    return cuda_err(c, cudaGetLastError(), "set_crack_2d");
}

int set_crack_2d(pd_ctx* c, double clength, double lx, double ly, double theta, cudaStream_t s) {
    return set_crack_2d_rows(c, 0, c->p.N_int, clength, lx, ly, theta, s);
}

int set_crack_kw(pd_ctx* c, double rad, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "set_crack needs the bond family");
    int rc = sync_fail_to_csr(c, s);
    if (rc) return rc;
    const KParams P = kparams(c->p);
    k_set_crack_kw<<<warps_grid(P.N_int), 256, 0, s>>>(P, rad, c->nf[PD_F_X], c->nf[PD_F_Y], c->rowptr, c->NL,
                                                        c->fail);
    c->launches++;
    c->bits_current = false;
    return cuda_err(c, cudaGetLastError(), "set_crack_kw");
}

static void free_sell(Sell& S) {
    free_ptr(S.width);
    free_ptr(S.base);
    free_ptr(S.fbase);
    free_ptr(S.csr);
    free_ptr(S.rec);
    free_ptr(S.sgeo);
    free_ptr(S.sth);
    free_ptr(S.sfo);
    free_ptr(S.e);
    free_ptr(S.bits);
    free_ptr(S.rec16);
    free_ptr(S.tpl);
    free_ptr(S.inst_tbase);
    free_ptr(S.srec);
    free_ptr(S.srec8);
    free_ptr(S.stpl);
    free_ptr(S.tpl3);
    free_ptr(S.sk);
    free_ptr(S.skz);
    free_ptr(S.e4);
    free_ptr(S.bbits);
    S.ntpl = 0;
    S.nslices = S.S = S.F = 0;
}

void release_sell(pd_ctx* c) {
    drop_graphs(c);
    free_sell(c->sell);
}

// The compact layout (S.csr filled): offset classes per specimen, their
// templates and the slot records, for 2-D bond-based problems (one specimen
// or a batch) and state-based problems in 2-D and 3-D.  Returns
// PD_ERR_UNSUPPORTED (arrays released) where the problem does not fit it:
// more than 255 classes in a specimen (or a region of the hash table full), a
// bond length that differs from its class's smallest by more than a float
// with a free low byte can hold, a reference vector too far from its class's
// float vector, a coefficient off its class's by more than 2^-45, or (3-D) a
// key shared by two float vectors.
int build_compact(pd_ctx* c, cudaStream_t s) {
    const KParams P = kparams(c->p);
    Sell& S = c->sell;
    const int* grp = c->batch.node_group;
    const int64_t regions = c->batch.count > 0 ? c->batch.count : 1;
    const int64_t tsize = regions * kRegion;
    const bool state = c->p.model == PD_MODEL_STATE;
    const bool d3 = c->p.dim == 3;
    unsigned long long *keys = nullptr, *l0min = nullptr;
    int *ids = nullptr, *flags = nullptr;
    float4* vec = nullptr;
    auto cleanup = [&]() {
        cudaFreeAsync(keys, s);
        cudaFreeAsync(l0min, s);
        cudaFreeAsync(ids, s);
        cudaFreeAsync(flags, s);
        if (vec) cudaFreeAsync(vec, s);
    };
    auto release = [&]() {
        free_ptr(S.tpl);
        free_ptr(S.rec16);
        free_ptr(S.inst_tbase);
        free_ptr(S.srec);
        free_ptr(S.srec8);
        free_ptr(S.stpl);
        free_ptr(S.tpl3);
        free_ptr(S.sk);
        free_ptr(S.skz);
        free_ptr(S.e4);
        free_ptr(S.bbits);
        S.ntpl = 0;
    };
    if (cudaMallocAsync(&keys, tsize * 8, s) || cudaMallocAsync(&l0min, tsize * 8, s) ||
        cudaMallocAsync(&ids, tsize * 4, s) || cudaMallocAsync(&flags, 2 * 4, s) ||
        (d3 && cudaMallocAsync(&vec, tsize * sizeof(float4), s))) {
        cleanup();
        return set_err(c, PD_ERR_NOMEM, "offset-class table");
    }
    cudaMemsetAsync(keys, 0xff, tsize * 8, s);
    cudaMemsetAsync(l0min, 0xff, tsize * 8, s);
    cudaMemsetAsync(flags, 0, 2 * 4, s);
    if (vec) cudaMemsetAsync(vec, 0, tsize * sizeof(float4), s);
    const unsigned gx = (unsigned)std::min<int64_t>(S.nslices, 65535);
    const unsigned gy = (unsigned)((S.nslices + gx - 1) / gx);
    k_class_insert<<<dim3(gx, gy), 256, 0, s>>>(S.nslices, S.width, S.base, S.csr, c->NL, grp, c->nf[PD_F_X],
                                                 c->nf[PD_F_Y], d3 ? c->nf[PD_F_Z] : nullptr, c->idist, keys, l0min,
                                                 vec, flags);
    c->launches++;
    std::vector<unsigned long long> hk((size_t)tsize), hl((size_t)tsize);
    std::vector<float4> hv(d3 ? (size_t)tsize : 0);
    int hflags[2] = {0, 0};
    cudaMemcpyAsync(hk.data(), keys, tsize * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hl.data(), l0min, tsize * 8, cudaMemcpyDeviceToHost, s);
    if (d3) cudaMemcpyAsync(hv.data(), vec, tsize * sizeof(float4), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hflags, flags, 2 * 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_err(c, e, "offset classes");
    }
    if (hflags[0]) {
        cleanup();
        return set_err(c, PD_ERR_UNSUPPORTED, "compact layout: a specimen with more offset classes than its table");
    }
    // templates, numbered per specimen in key order: a float vector xf and
    // the smallest bond length l0t of the class; |xf|^2, |xf|^2 - l0t^2 and
    // l0t as exact pairs
    std::vector<bt::Tpl> tp;
    std::vector<bt::Tpl3> tp3;
    std::vector<double> l0ts;
    std::vector<int> hid((size_t)tsize, -1), tbase((size_t)regions, 0);
    for (int64_t g = 0; g < regions; g++) {
        std::vector<std::pair<unsigned long long, int64_t>> used;
        for (int64_t h = 0; h < kRegion; h++)
            if (hk[g * kRegion + h] != kEmptyKey) used.push_back({hk[g * kRegion + h], g * kRegion + h});
        std::sort(used.begin(), used.end());
        if (used.size() > 255) {
            cleanup();
            return set_err(c, PD_ERR_UNSUPPORTED,
                           "compact layout: " + std::to_string(used.size()) + " offset classes in a specimen");
        }
        tbase[g] = (int)l0ts.size();
        for (size_t k = 0; k < used.size(); k++) {
            const unsigned long long key = used[k].first;
            const int64_t slot = used[k].second;
            hid[slot] = (int)k;
            float xf[3] = {0.0f, 0.0f, 0.0f};
            if (d3) {
                xf[0] = hv[slot].x, xf[1] = hv[slot].y, xf[2] = hv[slot].z;
            } else {
                xf[0] = bt::ffrom((uint32_t)(key >> 32)), xf[1] = bt::ffrom((uint32_t)key);
            }
            const int nd = d3 ? 3 : 2;
            double sh = 0.0, sl = 0.0;
            for (int a = 0; a < nd; a++) {
                const double sq = (double)xf[a] * (double)xf[a];  // exact: 24-bit significands
                const double t = sh + sq, bb = t - sh;
                sl += (sh - (t - bb)) + (sq - bb);
                sh = t;
            }
            const double l0t = bt::dfrom(hl[slot]);
            const double ph = l0t * l0t, pl = std::fma(l0t, l0t, -ph);
            const bt::f2 c0 = bt::split_bits((sh - ph) + (sl - pl));  // sh - ph exact (Sterbenz)
            const bt::f2 q0 = bt::split_bits(sh + sl);
            const bt::f2 l0 = bt::split_bits(l0t);
            l0ts.push_back(l0t);
            if (d3) {
                bt::Tpl3 T{};
                for (int a = 0; a < 3; a++) {
                    T.xf[a] = xf[a];
                    T.xd[a] = bt::dbits((double)xf[a]);
                }
                T.c0h = c0.h, T.c0l = c0.l, T.q0h = q0.h, T.q0l = q0.l, T.l0h = l0.h, T.l0l = l0.l;
                T.l0d = l0t;
                tp3.push_back(T);
            } else {
                bt::Tpl T{};
                for (int a = 0; a < 2; a++) {
                    T.xf[a] = xf[a];
                    T.xd[a] = bt::dbits((double)xf[a]);
                }
                T.c0h = c0.h, T.c0l = c0.l, T.q0h = q0.h, T.q0l = q0.l, T.l0h = l0.h, T.l0l = l0.l;
                T.l0d = l0t;
                tp.push_back(T);
            }
        }
    }
    const size_t ntpl = l0ts.size();
    if (ntpl == 0) {
        cleanup();
        return set_err(c, PD_ERR_UNSUPPORTED, "compact layout: no bonds");
    }
    S.ntpl = (int)ntpl;
    const size_t nrec = (size_t)std::max<int64_t>(S.S, 1);
    bool ok = true;
    if (d3 && state)
        ok = !cudaMalloc(&S.tpl3, ntpl * sizeof(bt::Tpl3)) && !cudaMalloc(&S.srec8, nrec * sizeof(int2)) &&
             !cudaMalloc(&S.sk, nrec * sizeof(int4)) && !cudaMalloc(&S.skz, nrec * sizeof(int2)) &&
             !cudaMalloc(&S.stpl, ntpl * sizeof(StateTpl)) && !cudaMalloc(&S.e4, nrec * sizeof(float4)) &&
             !cudaMemsetAsync(S.e4, 0, nrec * sizeof(float4), s) &&
             !cudaMalloc(&S.bbits, (size_t)std::max<int64_t>(S.F, 1) * sizeof(uint32_t));
    else if (d3)
        ok = !cudaMalloc(&S.tpl3, ntpl * sizeof(bt::Tpl3)) && !cudaMalloc(&S.rec16, nrec * sizeof(bt::Rec));
    else if (state)
        ok = !cudaMalloc(&S.tpl, ntpl * sizeof(bt::Tpl)) && !cudaMalloc(&S.srec, nrec * sizeof(int4)) &&
             !cudaMalloc(&S.srec8, nrec * sizeof(int2)) && !cudaMalloc(&S.stpl, ntpl * sizeof(StateTpl));
    else
        ok = !cudaMalloc(&S.tpl, ntpl * sizeof(bt::Tpl)) && !cudaMalloc(&S.rec16, nrec * sizeof(bt::Rec));
    if (ok && regions > 1) ok = !cudaMalloc(&S.inst_tbase, regions * sizeof(int));
    if (!ok) {
        cleanup();
        release();
        return set_err(c, PD_ERR_NOMEM, "compact records");
    }
    if (d3)
        cudaMemcpyAsync(S.tpl3, tp3.data(), ntpl * sizeof(bt::Tpl3), cudaMemcpyHostToDevice, s);
    else
        cudaMemcpyAsync(S.tpl, tp.data(), ntpl * sizeof(bt::Tpl), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ids, hid.data(), tsize * 4, cudaMemcpyHostToDevice, s);
    if (S.inst_tbase) cudaMemcpyAsync(S.inst_tbase, tbase.data(), regions * sizeof(int), cudaMemcpyHostToDevice, s);
    std::vector<StateTpl> st;
    if (state) {
        // logarithmic derivatives of the coefficients at each class's l0t: the
        // weight exp(-l0^2/delta^2) gives -2 l0 / delta^2; the partial-volume
        // factor (delta + dx/2 - l0) / dx (kernel_vol_Corr, Surf_Corr.cu:26-31)
        // above delta - dx/2 gives -1 / (delta + dx/2 - l0); l0 itself 1 / l0
        st.resize(ntpl);
        const double dlt = c->p.delta, hdx = c->p.dx / 2.0;
        for (size_t k = 0; k < ntpl; k++) {
            const double l0t = l0ts[k];
            double g2 = -2.0 * l0t / (dlt * dlt);
            if (l0t > dlt - hdx) g2 -= 1.0 / (dlt + hdx - l0t);
            st[k] = StateTpl{};
            st[k].g2 = (float)g2;
            st[k].g1 = (float)(g2 + 1.0 / l0t);
        }
        cudaMemcpyAsync(S.stpl, st.data(), ntpl * sizeof(StateTpl), cudaMemcpyHostToDevice, s);
    }
    if (d3 && !state) {
        k_rec16_fill3<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, S.csr, c->NL, c->nf[PD_F_X],
                                                    c->nf[PD_F_Y], c->nf[PD_F_Z], c->idist, c->fac, c->scr, keys, ids,
                                                    S.tpl3, 0.5 * S.kscale_inv, S.rec16, flags + 1);
    } else if (d3) {
        k_state_compact3_fill<<<dim3(gx, gy), 256, 0, s>>>(
            P, S.nslices, S.width, S.base, S.csr, c->NL, c->nf[PD_F_X], c->nf[PD_F_Y], c->nf[PD_F_Z], c->idist, c->fac,
            c->w, keys, ids, S.tpl3, S.sn_exp, S.sth_exp, S.st_exp, S.srec8, S.sk, S.skz, S.stpl, flags + 1);
        k_break_bits<<<(unsigned)((S.nslices * 32 + 255) / 256), 256, 0, s>>>(S.nslices, S.width, S.base, S.fbase,
                                                                                S.skz, S.bbits);
        c->launches++;
    } else if (state) {
        k_state_compact_fill<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, S.csr, c->NL, c->nf[PD_F_X],
                                                           c->nf[PD_F_Y], c->idist, c->fac, c->w, keys, ids, S.tpl,
                                                           S.sn_exp, S.sth_exp, S.st_exp, S.srec, S.srec8, S.stpl,
                                                           flags + 1);
    } else {
        k_rec16_fill<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, S.csr, c->NL, grp, c->nf[PD_F_X],
                                                   c->nf[PD_F_Y], c->idist, c->fac, c->scr, c->batch.node_bc, keys,
                                                   ids, S.inst_tbase, S.tpl, 0.5 * S.kscale_inv, S.rec16, flags + 1);
    }
    c->launches++;
    if (state) {
        k_state_compact_check<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, S.csr, c->idist, c->fac,
                                                            c->w, S.srec8, S.stpl, S.sn_exp, S.sth_exp, S.st_exp,
                                                            flags + 1);
        c->launches++;
    }
    cudaMemcpyAsync(hflags + 1, flags + 1, 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) {
        release();
        return cuda_err(c, e, "compact records");
    }
    if (hflags[1]) {
        release();
        return set_err(c, PD_ERR_UNSUPPORTED, "compact layout: a bond outside its offset class's ranges");
    }
    return PD_OK;
}

int prepare(pd_ctx* c, cudaStream_t s) {
    if (!c->family) return set_err(c, PD_ERR_STATE, "prepare needs the bond family");
    drop_graphs(c);  // the SELL arrays are reallocated below
    int rc;
    const bool state = c->p.model == PD_MODEL_STATE;
    if (state && !c->weights && (rc = initial_weight(c, s))) return rc;  // vol_corr included
    if (!c->volcorr && (rc = vol_corr(c, s))) return rc;
    // the SELL fail bits are rebuilt from the CSR flags
    if ((rc = sync_fail_to_csr(c, s))) return rc;
    const KParams P = kparams(c->p);
    Sell& S = c->sell;
    free_sell(S);
    S.nslices = (P.N + 31) / 32;
    cudaError_t e;
    if ((e = cudaMalloc(&S.width, S.nslices * sizeof(int))) || (e = cudaMalloc(&S.base, S.nslices * 8)) ||
        (e = cudaMalloc(&S.fbase, (S.nslices + 1) * 8)))
        return set_err(c, PD_ERR_NOMEM, "slice tables");
    k_slice_width<<<warps_grid(S.nslices), 256, 0, s>>>(P.N, S.nslices, c->NN, S.width);
    c->launches++;
    std::vector<int> w((size_t)S.nslices);
    if ((e = cudaMemcpyAsync(w.data(), S.width, w.size() * sizeof(int), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return cuda_err(c, e, "slice widths");
    std::vector<int64_t> fb((size_t)S.nslices + 1), bs((size_t)S.nslices);
    int64_t acc = 0;
    int wmax = 0;
    for (int64_t k = 0; k < S.nslices; k++) {
        fb[k] = acc;
        bs[k] = acc * 32;
        acc += w[k];
        wmax = std::max(wmax, w[k]);
    }
    fb[S.nslices] = acc;
    S.wmax = wmax;
    S.F = acc;
    S.S = acc * 32;
    cudaMemcpyAsync(S.fbase, fb.data(), fb.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(S.base, bs.data(), bs.size() * 8, cudaMemcpyHostToDevice, s);
    const size_t n8 = (size_t)std::max<int64_t>(S.S, 1) * 8, n4 = (size_t)std::max<int64_t>(S.S, 1) * 4;
    bool ok = !cudaMalloc(&S.csr, n4) && !cudaMalloc(&S.bits, (size_t)std::max<int64_t>(S.F, 1) * 4);
    // every problem tries the compact layout first (small per-slot records on
    // offset-class templates); the 48-byte (bond-based) and three 32-byte
    // (state-based) records are the general layout, taken where the compact
    // one does not fit
    const bool try_compact = c->layout_pref != LAYOUT_RECORDS;
    if (ok && !state && !try_compact)
        ok = !cudaMalloc(&S.rec, n8 * 6);
    // power-of-two scale bringing the bond coefficient 2 vol bc / dx near one,
    // so that the pair arithmetic of the force kernels stays in float range
    {
        const double ref = 2.0 * P.vol * P.bc / P.dx;
        S.kexp = (ref > 0.0 && std::isfinite(ref)) ? (int)std::lround(std::log2(ref)) : 0;
        S.kscale = std::ldexp(1.0, S.kexp);
        S.kscale_inv = std::ldexp(1.0, -S.kexp);
    }
    // state-based: powers of two near 1/m, the dilatation weight and the force
    // coefficient c2/m, from the lattice (m ~ half of delta^2 vol over a family
    // of pi (delta/dx)^2 or 4/3 pi (delta/dx)^3 members); any estimate within a
    // few binades keeps the pairs in float range, and the scalings are exact
    if (state) {
        const double r = P.delta / P.dx;
        const double nfam = P.dim == 2 ? M_PI * r * r : 4.0 / 3.0 * M_PI * r * r * r;
        const double m_est = 0.25 * P.delta * P.delta * P.vol * nfam;
        const double pr = P.pratio;
        const double th_coef = P.dim == 2 ? 2.0 * (2.0 * pr - 1.0) / (pr - 1.0) : 3.0;
        const double b_coef = P.dim == 2 ? 8.0 * P.G : 15.0 * P.G;
        auto lg = [](double v) { return (v > 0.0 && std::isfinite(v)) ? (int)std::lround(std::log2(v)) : 0; };
        S.sn_exp = lg(1.0 / m_est);
        S.sth_exp = -lg(std::fabs(th_coef) * P.delta * P.vol);
        S.st_exp = S.sn_exp + lg(std::fabs(2.0 * b_coef) * P.vol);
    }
    if (ok && state) ok = !cudaMalloc(&S.e, n8) && !cudaMemsetAsync(S.e, 0, n8, s);
    if (ok && state && !try_compact)
        ok = !cudaMalloc(&S.sgeo, n8 * 4) && !cudaMalloc(&S.sth, n8 * 4) && !cudaMalloc(&S.sfo, n8 * 4);
    if (!ok) {
        free_sell(S);
        return set_err(c, PD_ERR_NOMEM, "SELL bond arrays");
    }
    const unsigned gx = (unsigned)std::min<int64_t>(S.nslices, 65535);
    const unsigned gy = (unsigned)((S.nslices + gx - 1) / gx);
    k_sell_fill<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, c->NN, c->rowptr, c->NL, c->nf[PD_F_X],
                                              c->nf[PD_F_Y], c->nf[PD_F_Z], c->idist, c->fac, c->scr, c->w,
                                              c->nf[PD_F_M], c->batch.node_bc, c->batch.node_s0, S);
    c->launches++;
    if (try_compact) {
        rc = build_compact(c, s);
        if (rc && c->layout_pref == LAYOUT_COMPACT) {
            free_sell(S);
            return rc;
        }
        if (rc) {
            // the general layout
            c->err.clear();
            if (state ? (cudaMalloc(&S.sgeo, n8 * 4) || cudaMalloc(&S.sth, n8 * 4) || cudaMalloc(&S.sfo, n8 * 4))
                      : cudaMalloc(&S.rec, n8 * 6) != cudaSuccess) {
                free_sell(S);
                return set_err(c, PD_ERR_NOMEM, "SELL bond arrays");
            }
            k_sell_fill<<<dim3(gx, gy), 256, 0, s>>>(P, S.nslices, S.width, S.base, c->NN, c->rowptr, c->NL,
                                                      c->nf[PD_F_X], c->nf[PD_F_Y], c->nf[PD_F_Z], c->idist, c->fac,
                                                      c->scr, c->w, c->nf[PD_F_M], c->batch.node_bc,
                                                      c->batch.node_s0, S);
            c->launches++;
        }
    }
    if (state) {
        k_inv_m<<<(unsigned)((P.N + 255) / 256), 256, 0, s>>>(P.N, c->nf[PD_F_M], std::ldexp(1.0, -S.sn_exp),
                                                             c->node_b, c->node_a);
        c->launches++;
    }
    c->bits_current = false;
    if ((rc = sync_fail_to_bits(c, s))) return rc;
    c->prepared = true;
    return cuda_err(c, cudaGetLastError(), "prepare");
}

}  // namespace pdg
