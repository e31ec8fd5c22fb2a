"""Error bound of the WENO weight normalisation's reciprocal, checked on the CPU.

The device computes 1/x for x in [1, 2^106] from a single-precision seed (x's
mantissa truncated to 23 bits, the hardware rcp.approx.f32 result, at most 1 ulp
of float off) refined once by the Newton–Raphson step y(1 + e + e^2) with
e = fma(-x, y, 1).  Here the seed is emulated with its worst cases (truncation
plus a ±1-ulp float reciprocal) and the FP64 fused operations are evaluated
exactly and rounded once, as a fused multiply-add does.
"""
from __future__ import annotations

import random
from fractions import Fraction

import numpy as np


def fma(a: float, b: float, c: float) -> float:
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def seed(x: float, ulps: int) -> float:
    xf = np.float32(x)
    # truncate (not round) the mantissa to float precision
    bits = np.float64(x).view(np.uint64)
    trunc = (bits >> np.uint64(29)) << np.uint64(29)
    xt = float(np.uint64(trunc).view(np.float64))
    assert abs(xt - float(xf)) <= abs(float(xf)) * 2.0 ** -23
    y = np.float32(1.0) / np.float32(xt)
    for _ in range(abs(ulps)):
        y = np.nextafter(y, np.float32(np.inf) if ulps > 0 else np.float32(0))
    return float(y)


def refine(x: float, y: float) -> float:
    e = fma(-x, y, 1.0)
    return fma(y, fma(e, e, e), y)


def test_reciprocal_within_two_ulp():
    rng = random.Random(5)
    worst = 0.0
    for n in range(3000):
        x = 2.0 ** rng.uniform(0.0, 106.0)
        for ulps in (-1, 0, 1):
            r = refine(x, seed(x, ulps))
            exact = 1 / Fraction(x)
            rel = abs(Fraction(r) - exact) / exact
            worst = max(worst, float(rel))
    assert worst <= 2.0 ** -52, worst  # two ulp of the correctly rounded value


def test_reciprocal_over_the_pressure_solve_range():
    """The same bound over the reciprocal's whole accepted range, [2^-124, 2^125) (its
    callers divide outside it)."""
    rng = random.Random(9)
    worst = 0.0
    for n in range(2000):
        x = 2.0 ** rng.uniform(-124.0, 125.0)
        for ulps in (-1, 0, 1):
            r = refine(x, seed(x, ulps))
            exact = 1 / Fraction(x)
            worst = max(worst, float(abs(Fraction(r) - exact) / exact))
    assert worst <= 2.0 ** -52, worst


def test_reciprocal_edges():
    for x in (1.0, 2.0 ** 106, 1.5, 3.0, 7.0, 2.0 ** 53 - 1):
        r = refine(x, seed(x, 1))
        assert abs(Fraction(r) * Fraction(x) - 1) <= Fraction(2) ** -52


def rsqrt_seed(x: float, ulps: int) -> float:
    bits = np.float64(x).view(np.uint64)
    xt = float(np.uint64((bits >> np.uint64(29)) << np.uint64(29)).view(np.float64))
    y = np.float32(1.0) / np.sqrt(np.float32(xt))
    for _ in range(abs(ulps) + 1):   # the hardware value may be a further ulp off
        y = np.nextafter(y, np.float32(np.inf) if ulps >= 0 else np.float32(0))
    return float(y)


def rsqrt_refine(x: float, y: float) -> float:
    """y(1 + e/2 + 3e^2/8), e = 1 - x y^2, with the device's fused operations."""
    e = fma(-float(Fraction(x) * Fraction(y)), y, 1.0)   # x*y rounded, then fused
    t = e * fma(e, 0.375, 0.5)
    return fma(y, t, y)


def test_inverse_sqrt_within_two_ulp():
    """The WENO5 update's 1/sqrt (FP64 form) from an FP32 seed and one second-order
    Newton step, checked against exact arithmetic over its range [2^-120, 2^120]."""
    import math
    rng = random.Random(7)
    worst = 0.0
    for _ in range(3000):
        x = 2.0 ** rng.uniform(-120.0, 120.0)
        for ulps in (-2, 0, 2):
            r = rsqrt_refine(x, rsqrt_seed(x, ulps))
            exact = 1 / math.sqrt(float(Fraction(x)))  # reference value in FP64
            # compare in exact arithmetic: |r^2 x - 1| ~ 2 * relative error
            rel = abs(Fraction(r) ** 2 * Fraction(x) - 1) / 2
            worst = max(worst, float(rel))
    assert worst <= 2.0 ** -52, worst


def sqrt_refine(x: float, y: float) -> float:
    """s(1 + e/2 + 3e^2/8) with s = x*y rounded and e = 1 - s*y: the FP64 update's square
    root, refined on s = x·y rather than on y, with the device's fused operations."""
    sq = float(Fraction(x) * Fraction(y))
    e = fma(-sq, y, 1.0)
    t = e * fma(e, 0.375, 0.5)
    return fma(sq, t, sq)


def test_square_root_within_two_ulp():
    """The WENO5 update's |∇φ| (FP64 form) from the FP32 inverse-square-root seed, over the
    same range [2^-120, 2^120], against exact arithmetic."""
    rng = random.Random(11)
    worst = 0.0
    for _ in range(3000):
        x = 2.0 ** rng.uniform(-120.0, 120.0)
        for ulps in (-2, 0, 2):
            r = sqrt_refine(x, rsqrt_seed(x, ulps))
            # |r^2/x - 1| ~ 2 * relative error of r
            rel = abs(Fraction(r) ** 2 / Fraction(x) - 1) / 2
            worst = max(worst, float(rel))
    assert worst <= 2.0 ** -52, worst
