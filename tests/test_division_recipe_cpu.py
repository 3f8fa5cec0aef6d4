"""The division recipe of the update kernels (div_recip in
pd_gpu1_gb300/csrc/pd_internal.cuh) restated on the CPU with exact fused
multiply-adds (rational arithmetic, one correctly rounded conversion per
FMA) against Python's IEEE division: y = 1/d, q0 = n y, one FMA correction
to a faithful q1, and Markstein's correction q2 = RN(q1 + (n - d q1) y),
which the theorem makes the correctly rounded n / d.  The GPU kernel itself
is held to the GPU's division in tests/test_gpu_division.py."""
import math
import struct
from fractions import Fraction

import numpy as np


def _fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))  # int / int rounds correctly (half to even)


def _exp(x):
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def div_recip(n, d, y):
    q0 = n * y
    if not all(123 <= _exp(v) <= 1923 for v in (n, y, q0)):
        return None  # the kernel takes the IEEE division here
    q1 = _fma(_fma(-q0, d, n), y, q0)
    return _fma(_fma(-q1, d, n), y, q1)


def _check(pairs):
    used = 0
    for n, d in pairs:
        q = div_recip(n, d, 1.0 / d)
        if q is None:
            continue
        used += 1
        assert struct.pack("<d", q) == struct.pack("<d", n / d), (n.hex(), d.hex(), q, n / d)
    return used


def test_recipe_is_the_correctly_rounded_quotient():
    rng = np.random.default_rng(7)
    k = 6000
    pairs = []
    # the kernels' divisors: 2 + cn dt, densities, an ADR mass, weighted volumes
    for d in list(2.0 + rng.uniform(0.0, 1.9, k)) + [8000.0, 2440.0, 2.866e18] * 200 + \
            list(10.0 ** rng.uniform(-20.0, -16.0, k)):
        pairs.append((float(rng.uniform(1.0, 2.0) * 2.0 ** int(rng.integers(-800, 800)) *
                            (1 if rng.integers(2) else -1)), float(d)))
    # random pairs over a wide exponent range
    for _ in range(k):
        pairs.append((math.ldexp(rng.uniform(1.0, 2.0), int(rng.integers(-950, 950))),
                      math.ldexp(rng.uniform(1.0, 2.0), int(rng.integers(-950, 950)))))
    # quotients within about an ulp of a midpoint: n = RN((q + ulp/2) d)
    for _ in range(k):
        q = math.ldexp(rng.uniform(1.0, 2.0), int(rng.integers(-30, 30)))
        d = math.ldexp(rng.uniform(1.0, 2.0), int(rng.integers(-30, 30)))
        m = Fraction(q) + Fraction(math.ulp(q)) / 2
        pairs.append((float(m * Fraction(d)), d))
    # divisors with an all-ones significand, and powers of two
    for _ in range(k // 4):
        n = math.ldexp(rng.uniform(1.0, 2.0), int(rng.integers(-300, 300)))
        pairs.append((n, math.ldexp(math.nextafter(2.0, 0.0), int(rng.integers(-60, 60)))))
        pairs.append((n, math.ldexp(1.0, int(rng.integers(-60, 60)))))
    used = _check(pairs)
    assert used > 0.9 * len(pairs)  # the rest fall back to the division (quotients beyond 2^900)


def test_recipe_leaves_extreme_operands_to_the_division():
    # zeros, subnormals and quotients beyond 2^900 take the IEEE division
    assert div_recip(0.0, 3.0, 1.0 / 3.0) is None
    assert div_recip(5e-324, 3.0, 1.0 / 3.0) is None
    assert div_recip(2.0 ** 899, 2.0 ** -10, 2.0 ** 10) is None
    assert div_recip(1.0, 3.0, 0.0) is None  # no reciprocal given
    assert div_recip(1.0, 3.0, 1.0 / 3.0) == 1.0 / 3.0
