// Exact differences of doubles by integer arithmetic, for the bond kernels.
//
// GB300 issues FP64 instructions at a small fraction of its integer and FP32
// rates.  Two of the three subtractions per component of a bond vector are
// exact by Sterbenz's lemma (operands of the same sign within a factor of two
// of each other): P_c - x_i (current position of the neighbour minus the
// reference coordinate of the node) and d - xif (the rounded bond vector
// minus its per-slot float reference).  Their results are computed here from
// the IEEE-754 fields on the integer pipe; the one rounding subtraction
// (the reference's  - u_i) stays in FP64.
//
// Both functions return false, leaving the caller to use an FP64
// subtraction, when an operand is zero, subnormal, infinite or NaN, when the
// signs differ or the binary exponents differ by more than one.
//
// Plain C++ (no CUDA types) so that the host test suite can compile and
// check it against the hardware subtraction.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PD_EXACT_HD __host__ __device__ __forceinline__
#else
#define PD_EXACT_HD inline
#endif

namespace pdg {

PD_EXACT_HD int pd_clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// a - b = diff * 2^(e - 1075) exactly (diff != 0 or a == b), for bit patterns
// ua, ub of normal doubles of the same sign with exponents within one.
PD_EXACT_HD bool sub_exact_scaled(uint64_t ua, uint64_t ub, int64_t& diff, int& e) {
    const uint64_t kFrac = (1ull << 52) - 1, kHidden = 1ull << 52;
    const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
    const bool ok = ((ua ^ ub) >> 63) == 0 && ea > 0 && eb > 0 && ea < 2047 && eb < 2047 && ea - eb <= 1 &&
                    eb - ea <= 1;
    if (!ok) return false;
    e = ea < eb ? ea : eb;
    const int64_t ma = (int64_t)(((ua & kFrac) | kHidden) << (ea - e));
    const int64_t mb = (int64_t)(((ub & kFrac) | kHidden) << (eb - e));
    diff = (ua >> 63) ? mb - ma : ma - mb;  // the value, signed
    return true;
}

// The same difference as a double bit pattern (exact by Sterbenz's lemma when
// the operands are within a factor of two; the caller guarantees that).
PD_EXACT_HD bool sub_exact(uint64_t ua, uint64_t ub, uint64_t& out) {
    int64_t diff;
    int e;
    if (!sub_exact_scaled(ua, ub, diff, e)) return false;
    if (diff == 0) {
        out = 0;  // x - x = +0 in round to nearest
        return true;
    }
    const uint64_t sign = diff < 0 ? (1ull << 63) : 0;
    uint64_t mag = diff < 0 ? (uint64_t)(-diff) : (uint64_t)diff;
    const int lead = 63 - pd_clz64(mag);  // position of the leading one
    const int shift = lead - 52;          // > 0 only for |diff| >= 2^53
    if (shift > 0) {
        if (mag & ((1ull << shift) - 1)) return false;  // not exact (outside Sterbenz's range)
        mag >>= shift;
    } else {
        mag <<= -shift;
    }
    const int er = e + shift;
    if (er <= 0 || er >= 2047) return false;
    out = sign | ((uint64_t)er << 52) | (mag & ((1ull << 52) - 1));
    return true;
}

}  // namespace pdg
