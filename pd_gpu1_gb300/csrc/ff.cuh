// Pair-of-floats ("double-float") arithmetic for the force kernels.
//
// GB300 issues FP64 instructions at about 1/64 of the FP32 rate, and every
// conversion between the two formats also occupies the FP64 pipe.  Work that
// does not need the reference's exact FP64 roundings is therefore done on
// unevaluated sums of two floats (value = h + l, |l| <= ulp(h)/2, about 46-48
// significant bits), with the classic error-free transformations:
//   Knuth's TwoSum (exact sum of two floats as a pair),
//   Dekker's fast TwoSum (the same when |a| >= |b|),
//   the FMA form of Dekker's TwoProduct (a*b = p + fma(a, b, -p) exactly).
// Conversions between double and pairs use integer operations on the IEEE-754
// fields (exponent rebias, mantissa shifts), which run on the integer pipe.
//
// Domain: magnitudes in (2^-74, 2^127); smaller values are treated as their
// leading float (or zero below 2^-126), which only affects terms far below
// the accuracy that matters here.
#pragma once
#include <cuda_runtime.h>

namespace pdg {

struct ff {
    float h, l;
};

// Sum of a and b as a normalized pair, assuming |a| >= |b| or a == 0.
__device__ __forceinline__ ff ff_fast(float a, float b) {
    const float s = a + b;
    return ff{s, b - (s - a)};
}

// Exact sum of two floats as a pair (no ordering assumption).
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return ff{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return ff_fast(p, e);
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.h, b.h);
    return ff_fast(s.h, s.l + (a.l + b.l));
}

// A float plus a pair (ff_add with a zero low part, one addition fewer).
__device__ __forceinline__ ff ff_add_f(float a, ff b) {
    ff s = ff_two_sum(a, b.h);
    return ff_fast(s.h, s.l + b.l);
}

// Double to pair with integer operations: h = v truncated to 24 significant
// bits, l = the remaining 29 mantissa bits rounded to a float.
__device__ __forceinline__ ff ff_split(double v) {
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
    const unsigned E = mag >> 20;  // biased exponent of the double
    const unsigned hb = sign | ((mag - (896u << 20)) << 3) | (lo >> 29);
    const float rem = __uint2float_rn(lo & 0x1fffffffu);
    const float scale = __uint_as_float(((E - 948u) & 0xffu) << 23);  // 2^(E - 1075) when E >= 949
    const unsigned lb = __float_as_uint(rem * scale) | sign;
    ff r;
    r.h = E < 897u ? 0.0f : __uint_as_float(hb);
    r.l = E < 949u ? 0.0f : __uint_as_float(lb);
    return r;
}

// Exact double of a float (zero and subnormal floats give zero), integer ops only.
__device__ __forceinline__ double f64_of_f32s(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned mag = b & 0x7fffffffu;
    const unsigned hi = (b & 0x80000000u) | ((mag >> 3) + (896u << 20));
    const double v = __hiloint2double((int)hi, (int)(mag << 29));
    return mag < 0x00800000u ? 0.0 : v;
}

// Exact double of f * 2^e (|e| < 800; zero and subnormal floats give zero),
// integer ops only: the power of two goes into the exponent field.
__device__ __forceinline__ double f64_of_f32s_scaled(float f, int e) {
    const unsigned b = __float_as_uint(f);
    const unsigned mag = b & 0x7fffffffu;
    const unsigned hi = (b & 0x80000000u) | ((mag >> 3) + ((unsigned)(896 + e) << 20));
    const double v = __hiloint2double((int)hi, (int)(mag << 29));
    return mag < 0x00800000u ? 0.0 : v;
}

// (h + l) * 2^e for a float pair in one FP64 addition: bit for bit the sum of
// the exact doubles times 2^e, since scaling by a power of two is exact and
// commutes with the sum's rounding while every value stays a normal double.
__device__ __forceinline__ double f64_of_pair_scaled(float h, float l, int e) {
    return f64_of_f32s_scaled(h, e) + f64_of_f32s_scaled(l, e);
}

__device__ __forceinline__ float rsqrt_approx_f32(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/sqrt(x) of a positive double as a pair, relative error ~2e-14: the FP32
// hardware estimate y0 and one Newton step y0 + y0 (1 - x y0^2) / 2, with the
// residual 1 - x y0^2 formed exactly enough in pair arithmetic (y0^2 and the
// products with both halves of x are split by FMA; 1 - q is exact because q
// is within a factor of two of one).
__device__ __forceinline__ ff ff_rsqrt(ff x) {
    const float y0 = rsqrt_approx_f32(x.h);
    const float p = y0 * y0;
    const float pe = fmaf(y0, y0, -p);
    const float q = x.h * p;
    const float qe = fmaf(x.h, p, -q);
    const float c = fmaf(x.h, pe, fmaf(x.l, p, qe));
    const float rho = (1.0f - q) - c;
    return ff_fast(y0, (0.5f * y0) * rho);
}

// a * b for a pair a and a float b.
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = a.h * b;
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return ff_fast(p, e);
}

// a^2 for a pair a.
__device__ __forceinline__ ff ff_sq(ff a) {
    const float p = a.h * a.h;
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(2.0f * a.h, a.l, e);
    return ff_fast(p, e);
}

__device__ __forceinline__ float rcp_approx_f32(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/z of a positive pair, relative error ~2e-14: the FP32 hardware estimate
// r0 and one Newton step r0 + r0 (1 - z r0), the residual formed as in ff_rsqrt.
__device__ __forceinline__ ff ff_rcp(ff z) {
    const float r0 = rcp_approx_f32(z.h);
    const float q = z.h * r0;
    const float qe = fmaf(z.h, r0, -q);
    const float c = fmaf(z.l, r0, qe);
    const float rho = (1.0f - q) - c;
    return ff_fast(r0, r0 * rho);
}

// a > b for normalized pairs (|l| <= ulp(h) / 2), as exact values.
__device__ __forceinline__ bool ff_gt(ff a, ff b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }

}  // namespace pdg
