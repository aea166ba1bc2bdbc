"""Exact-arithmetic identities the CUDA kernels rely on to match the oracle bit
for bit while using fewer instructions than the expression they replace.

UNORM8 decode (device unorm8, csrc/sgi_math.cuh): for every byte b the
product q = RN(b * RN(1/255)) followed by q' = RN(RN(b - q*255) * RN(1/255) + q)
(two fused multiply-adds) equals RN(b / 255), the quotient the oracle computes.
Checked exhaustively here in exact rational arithmetic, and the same step for
the 65536 UNORM16 values b / 65535 (device unorm16, the unorm16 depth cubes).

Exponential without range reduction (device expf_exact / expf_ieee2): for
|x| < 0.34 the Cody & Waite step gives k = floor(RN(RN(x * log2 e) + 0.5)) = 0,
the reduced argument (x - 0 * ln2_hi) - 0 * ln2_lo is x itself and the final
scaling multiplies by 2^0, so the result is the Taylor polynomial of x alone.
"""
from fractions import Fraction

import numpy as np


def rn32(x: Fraction) -> np.float32:
    """x rounded to the nearest binary32 (ties to even), from an exact rational."""
    f = np.float32(float(x))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - x), int(np.array(c, np.float32).view(np.uint32)) & 1))
    return np.float32(best)


def test_unorm8_reciprocal_step_equals_division():
    r = rn32(Fraction(1, 255))
    assert r == np.float32(1.0) / np.float32(255.0)
    for b in range(256):
        q = rn32(Fraction(b) * Fraction(float(r)))
        res = rn32(Fraction(b) - Fraction(float(q)) * 255)          # fma(-q, 255, b)
        q2 = rn32(Fraction(float(res)) * Fraction(float(r)) + Fraction(float(q)))   # fma(res, r, q)
        want = np.float32(b) / np.float32(255.0)
        assert q2 == want, b
        assert q2 == rn32(Fraction(b, 255)), b


def test_unorm16_reciprocal_step_equals_division():
    r = rn32(Fraction(1, 65535))
    assert r == np.float32(1.0) / np.float32(65535.0)
    fr = Fraction(float(r))
    for b in range(65536):
        q = rn32(Fraction(b) * fr)
        res = rn32(Fraction(b) - Fraction(float(q)) * 65535)          # fma(-q, 65535, b)
        q2 = rn32(Fraction(float(res)) * fr + Fraction(float(q)))     # fma(res, r, q)
        assert q2 == np.float32(b) / np.float32(65535.0), b


def test_difference_magnitude_is_symmetric():
    """|a - b| == |b - a| under round-to-nearest (the a-trous depth weight takes
    the tap-minus-centre difference): checked on random binary32 pairs."""
    rng = np.random.default_rng(3)
    a = rng.standard_normal(100000).astype(np.float32) * np.float32(50)
    b = (a + rng.standard_normal(100000).astype(np.float32)).astype(np.float32)
    assert np.array_equal(np.abs(a - b).view(np.uint32), np.abs(b - a).view(np.uint32))
    # x - y*c == x + y*(-c): the negated constant's product is the negated product
    c = np.float32(0.693145751953125)
    assert np.array_equal((a - b * c).view(np.uint32), (a + b * (-c)).view(np.uint32))


LOG2E = np.float32(1.44269502162933349609375)
LN2_HI = np.float32(0.693145751953125)
LN2_LO = np.float32(1.428606765330187045037746429443359375e-06)
NO_REDUCE = np.float32(0.34)


def _k(x):
    return np.floor((x * LOG2E).astype(np.float32) + np.float32(0.5)).astype(np.float32)


def test_exp_needs_no_reduction_below_the_bound():
    # k(x) is monotone in x (a product with a positive constant, a sum and floor, each rounded
    # monotonically), so k = 0 at the two extreme arguments below the bound gives k = 0 between them
    top = np.nextafter(NO_REDUCE, np.float32(0))
    ends = np.array([top, -top], np.float32)
    assert np.all(_k(ends) == 0)
    assert NO_REDUCE < np.float32(np.log(2.0) / 2.0)
    # the reduced argument is x, bit for bit (signed zeros and subnormals included)
    rng = np.random.default_rng(5)
    x = (rng.uniform(-1, 1, 1_000_000) * NO_REDUCE).astype(np.float32)
    x = np.concatenate([x, ends, np.array([0.0, -0.0, 1e-45, -1e-45, 2e-38, -2e-38], np.float32)])
    x = x[np.abs(x) < NO_REDUCE]
    kf = _k(x)
    assert np.all(kf == 0) and not np.any(np.signbit(kf))
    r = ((x - kf * LN2_HI).astype(np.float32) - kf * LN2_LO).astype(np.float32)
    assert np.array_equal(r.view(np.uint32), x.view(np.uint32))
    # and the scaling by 2^(k + 127 - 127) is a multiplication by 1
    p = rng.uniform(0.5, 2.0, 1000).astype(np.float32)
    assert np.array_equal((p * np.float32(1.0)).view(np.uint32), p.view(np.uint32))
