"""Accuracy of the compensated dot product that the float-float vertex-patch
application accumulates with (dot2_mac in movfem_gb300/csrc/mvf_patch.cu).

Each operand is an FP64 value split into FP32 halves hi + lo.  The high part of the sum
is carried by TwoSum; the rounding errors (the product's from FMA, the cross terms, the
sum's) go to a plain FP32 low part.  The same steps run here in IEEE single precision
(numpy float32; FMA emulated through the exact FP64 product) and are compared with
exact rational arithmetic: the error, relative to the sum of the terms' magnitudes, is
that of a sum carried at about twice FP32's precision.
"""
from fractions import Fraction

import numpy as np

f32 = np.float32


def fma32(a, b, c):
    # a*b is exact in FP64 (24 + 24 bits); the sum is rounded once to FP64, then FP32
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split(x):
    hi = f32(x)
    return hi, f32(np.float64(x) - np.float64(hi))


def dot2_mac(sh, sl, ah, al, bh, bl):
    p = f32(ah * bh)
    e = fma32(ah, bh, -p)
    e = fma32(ah, bl, fma32(al, bh, e))
    t = f32(sh + p)
    bb = f32(t - sh)
    err = f32(f32(sh - f32(t - bb)) + f32(p - bb))
    return t, f32(sl + f32(e + err))


def test_dot2_matches_exact_sum_to_about_twice_fp32_precision():
    rng = np.random.Generator(np.random.PCG64(5))
    worst = 0.0
    for trial in range(200):
        n = int(rng.integers(8, 64))
        a = rng.normal(size=n) * 10.0 ** rng.uniform(-3, 3, n)
        b = rng.normal(size=n) * 10.0 ** rng.uniform(-3, 3, n)
        if trial % 2:  # positive terms: no cancellation
            a, b = np.abs(a), np.abs(b)
        sh, sl = f32(0), f32(0)
        exact, scale = Fraction(0), Fraction(0)
        for x, y in zip(a, b):
            ah, al = split(x)
            bh, bl = split(y)
            sh, sl = dot2_mac(sh, sl, ah, al, bh, bl)
            term = (Fraction(float(ah)) + Fraction(float(al))) * (Fraction(float(bh)) + Fraction(float(bl)))
            exact += term
            scale += abs(term)
        got = Fraction(float(sh)) + Fraction(float(sl))
        worst = max(worst, float(abs(got - exact) / scale))
    # plain FP32 accumulation gives ~1e-6 relative to the sum of |terms| here; the
    # compensated dot stays near 5e-14
    assert worst < 1e-12, worst
