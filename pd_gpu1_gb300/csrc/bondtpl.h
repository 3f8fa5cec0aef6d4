// Per-bond arithmetic of the 2-D bond-based force kernels on lattice offset
// templates (the compact layout of force.cu: a 16-byte record per slot plus
// one template per lattice offset class).
//
// The reference computes, per bond (Force_Bond.cu:72-77),
//   d = ((x_c + u_c) - x_i) - u_i  (per component, FP64),
//   L = |d|, s = (L - l0) / l0,
//   f = vol fac bc scr s d / L,  broken when s > s0.
// Here d keeps the reference's FP64 roundings (P_c = x_c + u_c is stored per
// node, so d = (P_c - x_i) - u_i: two FP64 instructions per component), and
// everything after d runs on pairs of floats (value h + l, about 48 bits):
//   eta = d - xf exactly, xf the offset class's float reference vector;
//   S   = eta . (2 xf + eta)  = |d|^2 - |xf|^2,
//   D   = S + c0 - 2 l0t dl   = L^2 - l0^2  (c0 = |xf|^2 - l0t^2, l0 = l0t + dl),
//   L^2 = S + |xf|^2,
//   e   = D / (L + l0)        = L - l0, without cancellation,
//   t   = (k2 / 2) e / L,  f += t (xf + eta)  with k2 = 2 vol fac bc scr / l0.
// Per bond that is four FP64 instructions (the reference's roundings of d) and
// about two hundred FP32 and integer instructions, against the reference's
// 58-odd FP64 instructions (three divides and a square root).
//
// The offset class (template) holds what every bond of one lattice offset
// shares: xf, |xf|^2, c0 and the class's reference length l0t (the smallest
// l0 of the class).  The slot keeps only what varies from row to row: the
// neighbour id, dl = l0 - l0t (a float: the bond lengths of one class differ
// in their last bits only), k2 and the class id (in the low byte of dl,
// whose significand has at most 15 bits).
//
// Plain C++ apart from the two approximate reciprocals, so that the host test
// suite compiles the same code and checks it against extended precision.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "exact_sub.h"

#if defined(__CUDACC__)
#define PD_BT_HD __host__ __device__ __forceinline__
#else
#define PD_BT_HD inline
#endif

namespace pdg {
namespace bt {

struct f2 {
    float h, l;  // value h + l
};

// One offset class: four 16-byte words, ordered so that a bond's stretch
// reads the first three (the fourth holds l0t as a double, read only by the
// break test's exact path).
struct alignas(16) Tpl {
    uint64_t xd[2];  // xf as double bit patterns
    float xf[2];     // the class's float reference vector
    float c0h, c0l;  // |xf|^2 - l0t^2 as a pair (computed exactly)
    float q0h, q0l;  // |xf|^2 as a pair
    float l0h, l0l;  // l0t as a pair
    double l0d;      // l0t
    double pad;
};
static_assert(sizeof(Tpl) == 64, "four 16-byte words");

// One 3-D offset class: the same quantities as Tpl with three components
// (five 16-byte words; a stretch reads the first four).
struct alignas(16) Tpl3 {
    uint64_t xd[3];  // xf as double bit patterns
    float xf[3];     // the class's float reference vector
    float c0h, c0l;  // |xf|^2 - l0t^2 as a pair (computed exactly)
    float q0h, q0l;  // |xf|^2 as a pair
    float l0h, l0l;  // l0t as a pair
    float pad;
    double l0d;      // l0t
    double pad2;
};
static_assert(sizeof(Tpl3) == 80, "five 16-byte words");

// Per-slot record: 16 bytes, one 128-bit load.
struct alignas(16) Rec {
    int col;      // neighbour id (the row itself for padding)
    float dl;     // l0 - l0t; the class id in the low 8 bits of its significand
    float k2h;    // k2 / 2 times 2^-kexp as a pair (zero for padding)
    float k2l;
};
static_assert(sizeof(Rec) == 16, "one 16-byte word");

PD_BT_HD uint32_t fbits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
PD_BT_HD float ffrom(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
PD_BT_HD uint64_t dbits(double v) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t u;
    memcpy(&u, &v, 8);
    return u;
#endif
}
PD_BT_HD double dfrom(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double v;
    memcpy(&v, &u, 8);
    return v;
#endif
}

// Error-free transformations (Knuth's TwoSum, Dekker's fast TwoSum for
// |a| >= |b| or a == 0, the FMA TwoProduct).
PD_BT_HD f2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return f2{s, (a - (s - bb)) + (b - bb)};
}
PD_BT_HD f2 fast_sum(float a, float b) {
    const float s = a + b;
    return f2{s, b - (s - a)};
}
// a * b for pairs (relative error about 2^-47)
PD_BT_HD f2 mul(f2 a, f2 b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return fast_sum(p, e);
}

// FP32 estimates of 1/sqrt(x) and 1/x (the hardware's approximate
// instructions, relative error below 2^-22).  The host build, which has no
// such instructions, uses the correctly rounded values times a deterministic
// factor within 2^-22 of one, so that host checks of the refinements below
// see seeds as far off as the hardware's.
#if !defined(__CUDA_ARCH__)
PD_BT_HD float seed_noise(float x) {
    uint32_t h = fbits(x) * 2654435761u;
    h ^= h >> 15;
    return 1.0f + ldexpf((float)((int)(h & 0xffff) - 32768) / 32768.0f, -22);
}
#endif
PD_BT_HD float rsqrt_seed(float x) {
#if defined(__CUDA_ARCH__)
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return (1.0f / sqrtf(x)) * seed_noise(x);
#endif
}
PD_BT_HD float rcp_seed(float x) {
#if defined(__CUDA_ARCH__)
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
#else
    return (1.0f / x) * seed_noise(x);
#endif
}

// 1/sqrt(x) of a positive pair from the FP32 estimate y0: with the residual
// rho = 1 - x y0^2 formed exactly enough (y0^2 and x.h y0^2 split by FMA),
// 1/sqrt(x) = y0 (1 - rho)^(-1/2) = y0 (1 + rho/2 + 3 rho^2/8 + ...); the
// second-order term leaves a relative error of about 3 rho^3 (below 1e-19),
// so the result is limited by the pair format alone.
PD_BT_HD f2 rsqrt2(f2 x) {
    const float y0 = rsqrt_seed(x.h);
    const float p = y0 * y0;
    const float pe = fmaf(y0, y0, -p);
    const float q = x.h * p;
    const float qe = fmaf(x.h, p, -q);
    const float c = fmaf(x.h, pe, fmaf(x.l, p, qe));
    const float rho = (1.0f - q) - c;
    return fast_sum(y0, y0 * fmaf(0.375f * rho, rho, 0.5f * rho));
}
// 1/z of a positive pair from the FP32 estimate r0: 1/z = r0 / (1 - rho) =
// r0 (1 + rho + rho^2 + ...), rho = 1 - z r0, to second order.
PD_BT_HD f2 rcp2(f2 z) {
    const float r0 = rcp_seed(z.h);
    const float q = z.h * r0;
    const float qe = fmaf(z.h, r0, -q);
    const float c = fmaf(z.l, r0, qe);
    const float rho = (1.0f - q) - c;
    return fast_sum(r0, r0 * fmaf(rho, rho, rho));
}

// diff * 2^(e - 1075) as a normalized pair with the sign of sgn (a float bit
// pattern whose sign bit is the value's), for |diff| < 2^48 and e in
// [949, 1120]: diff = hi 2^24 + lo with 0 <= lo < 2^24, both exact floats.
PD_BT_HD f2 pair_of_scaled(int64_t diff, int e, uint32_t sgn) {
    const float sc = ffrom((((uint32_t)(e - 948)) << 23) | (sgn & 0x80000000u));
    const float h = (float)(int)(diff >> 24) * (sc * 16777216.0f);
    const float l = (float)(int)(diff & 0xffffff) * sc;
    return fast_sum(h, l);
}

// eta = d - x exactly as a pair, x the double value of a float (xb its bit
// pattern).  Usual case: d and x of the same sign and binade, where the
// difference of the bit patterns is the difference of the significands; then
// operands within one binade of each other (sub_exact_scaled); otherwise the
// caller's fallback (returns false): split_bits(d) for x = 0, an FP64
// subtraction otherwise.
PD_BT_HD bool offset_pair(double d, uint64_t xb, f2& eta) {
    const uint64_t db = dbits(d);
    const uint32_t hd = (uint32_t)(db >> 32), hx = (uint32_t)(xb >> 32);
    const int eb = (int)((hd >> 20) & 0x7ffu);
    const int64_t df = (int64_t)(db - xb);
    if (((hd ^ hx) & 0xfff00000u) == 0 && (unsigned)(eb - 949) <= (unsigned)(1120 - 949) &&
        (uint64_t)(df + (1ll << 48)) < (uint64_t)(1ll << 49)) {
        eta = pair_of_scaled(df, eb, hd);
        return true;
    }
    int64_t diff;
    int e;
    if (sub_exact_scaled(db, xb, diff, e) && e >= 949 && e <= 1120 && diff < (1ll << 48) && diff > -(1ll << 48)) {
        eta = pair_of_scaled(diff, e, 0u);
        return true;
    }
    return false;
}

// Double of a pair: fl(h + l) (both exact doubles).
PD_BT_HD double pair_sum_f64(f2 v) { return (double)v.h + (double)v.l; }

// A double as a pair with integer operations: h = v truncated to 24
// significant bits, l = the remaining 29 bits rounded to a float (relative
// error 2^-53; magnitudes below 2^-74 keep h only, below 2^-126 give zero).
PD_BT_HD f2 split_bits(double v) {
    const uint64_t b = dbits(v);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
    const uint32_t E = mag >> 20;
    const uint32_t hb = sign | ((mag - (896u << 20)) << 3) | (lo >> 29);
    const float rem = (float)(lo & 0x1fffffffu);
    const float scale = ffrom(((E - 948u) & 0xffu) << 23);  // 2^(E - 1075) when E >= 949
    const uint32_t lb = fbits(rem * scale) | sign;
    f2 r;
    r.h = E < 897u ? 0.0f : ffrom(hb);
    r.l = E < 949u ? 0.0f : ffrom(lb);
    return r;
}

struct BondOut {
    f2 f[2];  // force contribution per component, times 2^-kexp
    f2 e;     // extension L - l0
};

// The force contribution of one 2-D bond from its exact offsets eta (pairs),
// its offset class T and its record values (dl, k2 / 2 as a pair).
// The stretch of one 2-D bond from its exact offsets eta (pairs), its
// offset class T and dl = l0 - l0t: the bond vector W = xf + eta, 1/L and the
// extension e = L - l0, all as pairs.
PD_BT_HD void stretch2(const f2 eta[2], const Tpl& T, float dl, f2 w[2], f2& y, f2& e) {
    f2 v[2];
    float m[2], lo[2];
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int a = 0; a < 2; a++) {
        // W = xf + eta and V = 2 xf + eta as pairs (TwoSum of the high parts)
        f2 s = two_sum(T.xf[a], eta[a].h);
        w[a] = f2{s.h, s.l + eta[a].l};
        s = two_sum(2.0f * T.xf[a], eta[a].h);  // 2 xf (exact)
        v[a] = f2{s.h, s.l + eta[a].l};
        // eta_a V_a: exact product of the high parts, cross terms in the low part
        m[a] = eta[a].h * v[a].h;
        float r = fmaf(eta[a].h, v[a].h, -m[a]);
        r = fmaf(eta[a].h, v[a].l, r);
        lo[a] = fmaf(eta[a].l, v[a].h, r);
    }
    // S = eta . V (the sum of the high parts exact; S_low carries the rest)
    const f2 s = two_sum(m[0], m[1]);
    const float s_low = (lo[0] + lo[1]) + s.l;
    // D = S + c0 - 2 l0t dl = L^2 - l0^2
    const f2 dd = two_sum(s.h, T.c0h);
    const float d_low = ((s_low + dd.l) + T.c0l) + (-2.0f * T.l0h) * dl;
    const f2 D = fast_sum(dd.h, d_low);
    // L^2 = S + |xf|^2
    const f2 qq = two_sum(T.q0h, s.h);
    const f2 L2 = fast_sum(qq.h, (qq.l + s_low) + T.q0l);
    // 1/L, L, L + l0, e = D / (L + l0)
    y = rsqrt2(L2);
    const f2 L = mul(L2, y);
    const f2 lp = two_sum(L.h, T.l0h);
    const f2 Lp = fast_sum(lp.h, ((lp.l + L.l) + T.l0l) + dl);
    e = mul(D, rcp2(Lp));
}

// The stretch of one 3-D bond, as stretch2 with three components: the
// length from the exact offsets eta of the bond vector whose length the
// caller wants (w = xf + eta per component), 1/L and e = L - l0.
PD_BT_HD void stretch3(const f2 eta[3], const Tpl3& T, float dl, f2 w[3], f2& y, f2& e) {
    float m[3], lo[3];
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int a = 0; a < 3; a++) {
        f2 s = two_sum(T.xf[a], eta[a].h);
        w[a] = f2{s.h, s.l + eta[a].l};
        s = two_sum(2.0f * T.xf[a], eta[a].h);  // 2 xf (exact)
        const f2 v{s.h, s.l + eta[a].l};
        m[a] = eta[a].h * v.h;
        float r = fmaf(eta[a].h, v.h, -m[a]);
        r = fmaf(eta[a].h, v.l, r);
        lo[a] = fmaf(eta[a].l, v.h, r);
    }
    // S = eta . (2 xf + eta): the high parts summed exactly in two steps
    const f2 s01 = two_sum(m[0], m[1]);
    const f2 s = two_sum(s01.h, m[2]);
    const float s_low = ((lo[0] + lo[1]) + lo[2]) + (s01.l + s.l);
    const f2 dd = two_sum(s.h, T.c0h);
    const float d_low = ((s_low + dd.l) + T.c0l) + (-2.0f * T.l0h) * dl;
    const f2 D = fast_sum(dd.h, d_low);
    const f2 qq = two_sum(T.q0h, s.h);
    const f2 L2 = fast_sum(qq.h, (qq.l + s_low) + T.q0l);
    y = rsqrt2(L2);
    const f2 L = mul(L2, y);
    const f2 lp = two_sum(L.h, T.l0h);
    const f2 Lp = fast_sum(lp.h, ((lp.l + L.l) + T.l0l) + dl);
    e = mul(D, rcp2(Lp));
}

PD_BT_HD BondOut bond2(const f2 eta[2], const Tpl& T, float dl, f2 k2half) {
    BondOut o;
    f2 w[2], y;
    stretch2(eta, T, dl, w, y, o.e);
    // t = (k2 / 2) e / L, f = t W
    const f2 t = mul(mul(k2half, o.e), y);
    o.f[0] = mul(t, w[0]);
    o.f[1] = mul(t, w[1]);
    return o;
}

// a + b for pairs (TwoSum of the high parts, renormalized).
PD_BT_HD f2 add(f2 a, f2 b) {
    const f2 s = two_sum(a.h, b.h);
    return fast_sum(s.h, s.l + (a.l + b.l));
}

// Accumulate a pair into a running sum, renormalized at every addition (the
// low part stays within half an ulp of the high part, so the rounding of the
// low-part sum costs 2^-48 of the running sum, not of the low part's growth).
PD_BT_HD void acc_add(f2& acc, f2 v) {
    const f2 s = two_sum(acc.h, v.h);
    acc = fast_sum(s.h, s.l + (acc.l + v.l));
}

// e > ecrit with ecrit = fl(s0 l0), l0 = l0t + dl, given s0 and s0f = s0
// rounded to float: decided on floats unless e lies within a few float ulps
// of the threshold (tf = s0f * l0h is within 4 ulps of ecrit), then on the
// double sum of the pair against the double threshold, the test of the
// reference-rounded kernels.
template <class TT>
PD_BT_HD bool exceeds(f2 e, double s0, float s0f, const TT& T, float dl) {
    const float tf = s0f * T.l0h;
    const int hb = (int)fbits(e.h), tb = (int)fbits(tf);
    if (hb >= tb + 8) return true;   // e >= e.h - ulp/2 > tf (1 + 2^-21) > ecrit
    if (hb < tb - 8) return false;   // e < tf (1 - 2^-21) < ecrit (e.h < 0 included)
    const double ecrit = s0 * (T.l0d + (double)dl);
    return pair_sum_f64(e) > ecrit;
}

// The exact double of a float from its IEEE fields (zero and subnormal
// floats give zero): no FP64 conversion instruction.
PD_BT_HD double f64_exact(float f) {
    const uint32_t b = fbits(f), mag = b & 0x7fffffffu;
    if (mag < 0x00800000u) return 0.0;
    const uint32_t hi = (b & 0x80000000u) | ((mag >> 3) + (896u << 20));
    return dfrom(((uint64_t)hi << 32) | (uint64_t)(uint32_t)(mag << 29));
}

// One component's term of the ADR damping numerator (kernel_cnn,
// Integrate.cu:17-33),
//   -u^2 (F/m - F_old/m) / (dt vh),
// as -u^2 ((F - F_old) (1/m)) / (dt vh) with both divisions through
// reciprocals: 1/m (IEEE-rounded, rmass) and 1/(dt vh) from the FP32
// estimate of the divisor's leading bits refined by two Newton steps in FP64
// (relative error near 2^-53).  About eleven FP64 instructions instead of the
// reference's two quotients and one IEEE division (about 24).  The term is
// within a few units in the last place of the exact value of the reference's
// formula (the reference's own evaluation loses more when F and F_old are
// close); the damping coefficient sums these terms over all nodes in another
// order than the reference's in any case.  Divisors outside [2^-100, 2^101)
// in magnitude take the IEEE division.
PD_BT_HD double damping_term(double u, double f, double fo, double rmass, double dt, double vh) {
    const double d = dt * vh;
    const double n = -1.0 * u * u * ((f - fo) * rmass);
    const uint64_t b = dbits(d);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t mag = hi & 0x7fffffffu, E = mag >> 20;
    if (E < 923u || E > 1123u) return n / d;
    // d's leading bits as a float (truncated), then its reciprocal estimate
    const float df = ffrom((hi & 0x80000000u) | ((mag - (896u << 20)) << 3) | (lo >> 29));
    double y = f64_exact(rcp_seed(df));
    y = fma(y, fma(-d, y, 1.0), y);
    y = fma(y, fma(-d, y, 1.0), y);
#if defined(__CUDA_ARCH__)
    return __dmul_rn(n, y);  // a product of its own (no contraction into the caller's sum)
#else
    return n * y;
#endif
}

}  // namespace bt
}  // namespace pdg
