"""Error bounds of the double-float scalar arithmetic of the mixed pressure solve, on the CPU.

The solve forms β, α and the kept 1/γ, 1/(γα) of its Chronopoulos–Gear recurrences from
double-float (hi + lo float pair) totals with Dekker products (the exact FMA product
error folded into the low part), error-free sums (Knuth's TwoSum) and a reciprocal from the
correctly rounded float reciprocal refined by one Newton step on the double-float value.
Here every float operation is evaluated exactly and rounded once to float32 (round to
nearest even), as the device's _rn intrinsics and fused multiply-adds do, and the results
are compared with exact rational arithmetic.
"""
from __future__ import annotations

import math
import random
from fractions import Fraction

import numpy as np


def rf(x: Fraction) -> float:
    """x rounded to the nearest float32 (ties to even), as a Python float."""
    if x == 0:
        return 0.0
    e = math.floor(math.log2(abs(x)))
    # correct a floating misestimate of the exponent
    while abs(x) >= Fraction(2) ** (e + 1):
        e += 1
    while abs(x) < Fraction(2) ** e:
        e -= 1
    q = Fraction(2) ** (e - 23)
    m = x / q
    n = math.floor(m)
    r = m - n
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and n % 2 == 1):
        n += 1
    v = float(n * q)
    assert float(np.float32(v)) == v
    return v


F = Fraction


def add(a, b): return rf(F(a) + F(b))
def sub(a, b): return rf(F(a) - F(b))
def mul(a, b): return rf(F(a) * F(b))
def fma(a, b, c): return rf(F(a) * F(b) + F(c))


# the device helpers, operation for operation
def two_sum(a, b):
    s = add(a, b)
    bb = sub(s, a)
    return s, add(sub(a, sub(s, bb)), sub(b, bb))


def df_merge(a, b):
    s_hi, s_lo = two_sum(a[0], b[0])
    lo = add(s_lo, add(a[1], b[1]))
    hi = add(s_hi, lo)
    return hi, sub(lo, sub(hi, s_hi))


def df_quick(hi, lo):
    s = add(hi, lo)
    return s, sub(lo, sub(s, hi))


def df_mul(a, b):
    p = mul(a[0], b[0])
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return df_quick(p, e)


def df_recip(b):
    y = rf(1 / F(b[0]))
    r = fma(-b[1], y, fma(-b[0], y, 1.0))
    return df_quick(y, mul(y, r))


def val(a):
    return F(a[0]) + F(a[1])


def rand_df(rng, lo_exp=-20, hi_exp=40):
    """A normalised double-float: hi a float, |lo| at most half an ulp of hi."""
    x = F(rng.uniform(1, 2)) * F(2) ** rng.randint(lo_exp, hi_exp)
    hi = rf(x)
    return df_quick(hi, rf(x - F(hi)))


def rel(a, exact):
    return abs(val(a) - exact) / abs(exact)


def test_products_reciprocals_and_sums():
    rng = random.Random(17)
    worst = {"mul": 0.0, "recip": 0.0, "merge": 0.0}
    for _ in range(1500):
        a, b = rand_df(rng), rand_df(rng)
        worst["mul"] = max(worst["mul"], float(rel(df_mul(a, b), val(a) * val(b))))
        worst["recip"] = max(worst["recip"], float(rel(df_recip(b), 1 / val(b))))
        worst["merge"] = max(worst["merge"], float(rel(df_merge(a, b), val(a) + val(b))))
    # measured: 2^-46.9, 2^-46.3 and 2^-47.6
    assert worst["mul"] <= 2.0 ** -45, worst
    assert worst["recip"] <= 2.0 ** -45, worst
    assert worst["merge"] <= 2.0 ** -45, worst


def test_step_sizes_of_one_iteration():
    """β = γ/γ_old, α = γ²/(γ·den) with den = δ - γ²/(γ_old α_old), and the kept
    1/γ and 1/(γα), as the lane that finishes the grid totals forms them, against exact
    arithmetic.  δ is drawn so that den keeps at least 1/64 of it, the cancellation
    CG's recurrence meets when consecutive directions are far from conjugate."""
    rng = random.Random(23)
    worst = 0.0
    for _ in range(600):
        g_old = F(rng.uniform(1, 2)) * F(2) ** rng.randint(0, 30)
        a_old = F(rng.uniform(0.1, 2))
        g = g_old * F(rng.uniform(0.05, 1.5))
        sub_term = g * g / (g_old * a_old)
        delta = sub_term / (1 - F(rng.uniform(1 / 64, 0.9)))
        to_df = lambda x: df_quick(rf(x), rf(x - F(rf(x))))
        gD, dD = to_df(g), to_df(delta)
        inv_g = to_df(1 / g_old)
        inv_ga = to_df(1 / (g_old * a_old))
        beta = df_mul(gD, inv_g)
        gg = df_mul(gD, gD)
        den = df_merge(dD, (-df_mul(gg, inv_ga)[0], -df_mul(gg, inv_ga)[1]))
        rq = df_recip(df_mul(gD, den))
        alpha = df_mul(gg, rq)
        new_inv_g = df_mul(den, rq)
        new_inv_ga = df_mul(df_mul(new_inv_g, new_inv_g), den)
        den_x = delta - sub_term
        exact = {"beta": g / g_old, "alpha": g / den_x, "inv_g": 1 / g, "inv_ga": den_x / (g * g)}
        got = {"beta": beta, "alpha": alpha, "inv_g": new_inv_g, "inv_ga": new_inv_ga}
        for k in exact:
            worst = max(worst, float(rel(got[k], exact[k])))
    # the inputs' own rounding (2^-48 each) grows by the cancellation factor of den (< 64)
    assert worst <= 2.0 ** -36, worst
