"""The update kernels' division by a divisor with a known reciprocal
(div_recip: y = 1/d by the IEEE division, then two FMA corrections, the last
one Markstein's correctly rounded step) against the GPU's IEEE division, bit
for bit, through pd_check_division.

Operands: the divisors the kernels use (densities, ADR masses, 2 + cn dt
for cn in [0, 1.9], weighted volumes m) with numerators over the whole
exponent range; random pairs over the whole exponent range (which also
exercise the fallback to the IEEE division near underflow and overflow);
raw random bit patterns (zeros, subnormals, infinities, NaNs); numerators
formed as a midpoint between two doubles times the divisor, rounded, so
that the quotient lies within about an ulp of a rounding boundary; exact
quotients; divisors whose significand is all ones or a power of two."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f64(mant, exp, sign):
    """sign * (1 + mant / 2^52) * 2^exp as float64 (exp inside the normal range)."""
    bits = ((exp.astype(np.int64) + 1023) << 52) | (mant.astype(np.int64) & ((1 << 52) - 1))
    v = bits.view(np.float64)
    return np.where(sign, -v, v)


def _cases(rng):
    n_each = 1 << 21
    out = []

    def mant(k):
        return rng.integers(0, 1 << 52, size=k, dtype=np.int64)

    def sign(k):
        return rng.integers(0, 2, size=k).astype(bool)

    # the kernels' divisors with numerators over the whole exponent range
    cn = rng.uniform(0.0, 1.9, n_each)
    for d in (2.0 + cn * 1.0,  # ADR: 2 + cn dt with dt = 1
              np.full(n_each, 8000.0), np.full(n_each, 2440.0),  # densities
              np.full(n_each, 2.866e18),  # an ADR fictitious mass
              10.0 ** rng.uniform(-20.0, -16.0, n_each)):  # state-based weighted volumes m
        n = _f64(mant(n_each), rng.integers(-1020, 1021, n_each), sign(n_each))
        out.append((n, d))
    # random pairs over the whole exponent range (fallback near under- and overflow)
    out.append((_f64(mant(n_each), rng.integers(-1022, 1024, n_each), sign(n_each)),
                _f64(mant(n_each), rng.integers(-1022, 1024, n_each), sign(n_each))))
    # raw bit patterns: subnormals, zeros, infinities, NaNs among them
    raw = rng.integers(-(1 << 62), 1 << 62, size=(2, n_each), dtype=np.int64) * 2
    expo = np.int64(0x7ff << 52)
    raw[:, : n_each // 8] &= ~expo                # exponent 0: zeros and subnormals
    raw[:, n_each // 8: n_each // 4] |= expo      # exponent 2047: infinities and NaNs
    out.append((raw[0].view(np.float64), raw[1].view(np.float64)))
    # quotients near a rounding boundary: n = RN(m d), m halfway between two doubles
    d = _f64(mant(n_each), rng.integers(-30, 31, n_each), np.zeros(n_each, bool))
    q = _f64(mant(n_each), rng.integers(-30, 31, n_each), sign(n_each))
    half_ulp = np.spacing(np.abs(q)) / 2.0
    n = (q + np.copysign(half_ulp, q)) * d  # q + half an ulp is not representable; numpy rounds its product
    n2 = q * d + np.copysign(half_ulp, q) * d
    out.append((np.concatenate([n, n2]), np.concatenate([d, d])))
    # exact quotients and special divisors
    qs = _f64(rng.integers(0, 1 << 20, n_each) << 32, rng.integers(-40, 41, n_each), sign(n_each))
    ds = _f64(rng.integers(0, 1 << 20, n_each) << 32, rng.integers(-40, 41, n_each), np.zeros(n_each, bool))
    out.append((qs * ds, ds))
    ones = np.full(n_each, float(np.nextafter(2.0, 0.0))) * 2.0 ** rng.integers(-60, 61, n_each)
    pow2 = 2.0 ** rng.integers(-60, 61, n_each).astype(np.float64)
    for d in (ones, pow2):
        out.append((_f64(mant(n_each), rng.integers(-300, 301, n_each), sign(n_each)), d))
    # every pair of special values
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.225073858507201e-308, 2.2250738585072014e-308,
                   1.7976931348623157e308, 1.0, -1.0, 3.0, 2.0 ** -900, 2.0 ** 900])
    a, b = np.meshgrid(sp, sp)
    out.append((a.ravel(), b.ravel()))
    n = np.concatenate([a for a, _ in out])
    d = np.concatenate([b for _, b in out])
    return n, d


def test_division_recipe_matches_ieee_division():
    import torch

    from pd_gpu1_gb300._lib import lib

    L = lib()
    rng = np.random.default_rng(2024)
    with np.errstate(all="ignore"):
        n, d = _cases(rng)
    assert n.size > 20_000_000
    dn = torch.from_numpy(n).cuda()
    dd = torch.from_numpy(d).cuda()
    bad = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert L.pd_check_division(dn.data_ptr(), dd.data_ptr(), n.size, bad.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert int(bad.item()) == 0
    # a negative count is refused
    assert L.pd_check_division(dn.data_ptr(), dd.data_ptr(), -1, bad.data_ptr(), stream) == -1
