"""Exact-arithmetic identities the CUDA kernels rely on to match the oracle bit
for bit while using fewer instructions than the expression they replace.

UNORM8 decode (device unorm8, csrc/sgi_math.cuh): for every byte b the
product q = RN(b * RN(1/255)) followed by q' = RN(RN(b - q*255) * RN(1/255) + q)
(two fused multiply-adds) equals RN(b / 255), the quotient the oracle computes.
Checked exhaustively here in exact rational arithmetic.
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
