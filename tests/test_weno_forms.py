"""The two arrangements of the WENO5 one-sided derivatives used by the kernels,
restated in numpy and checked against the reference's form (Derivatives.h:134-159,
as the oracle computes it) on random lines.

Face form: the face between cells i and i+1 has five first differences
E1..E5 (φ_{i-2..i+3}); its second differences a, b, c, d give the smoothness
indicators (scaled by 12, with ε scaled alike) and its third differences
T1 = a-2b+c, T2 = b-2c+d.  With the central part 12C(i) = 7(D_i + D_{i+1}) -
(D_{i-1} + D_{i+2}) (Jiang & Peng 2000, "Weighted ENO schemes for Hamilton-Jacobi
equations"), one face gives both
    12 φ⁻(i+1) = 12C(i+1) + T2 - (.4 t2t3 T1 + .6 t1t2 T2) / (.1 t2t3 + .6 t1t3 + .3 t1t2)
    12 φ⁺(i)   = 12C(i)   - T1 + (.4 t1t2 T2 + .6 t2t3 T1) / (.1 t1t2 + .6 t1t3 + .3 t2t3)
with t_k = ((IS_k + ε')·2^-e)^2, 2^e ≤ ε' < 2^(e+1) (an exact scale that keeps the
products of two t_k in range).  The sweep kernel carries 6φ: with s = D_i + D_{i+1}
the bases 6C ± T/2 are 3s - (c-b) and 3s - (d-c); each ratio is halved and scaled by
5/3 above and below (U = t2t3 T1, V = t1t2 T2: numerators 2/3 U + V and U + 2/3 V
over 1/3 t2t3 + 2 t1t3 + t1t2 and t2t3 + 2 t1t3 + 1/3 t1t2); T2 is the difference of
the third differences c-b and d-c, and ε'·2^-e is ε''s significand.  face_form
follows that arrangement.

Cell form (the cell, column and pair kernels): each one-sided derivative from its own
face set, with the candidate stencils times six and the weights ten times the
reference's (q2²q3², 6 q1²q3², 3 q1²q2²), so that the first needs no product;
cell_form follows it.
"""
from __future__ import annotations

import numpy as np


def reference_weno(v):
    """weno5 of the oracle: (dm, dp) in difference units (no 1/dx) from 7 values."""
    out = []
    for side in (0, 1):
        if side:
            dev = [v[6] - v[5], v[5] - v[4], v[4] - v[3], v[3] - v[2], v[2] - v[1]]
        else:
            dev = [v[1] - v[0], v[2] - v[1], v[3] - v[2], v[4] - v[3], v[5] - v[4]]
        eps = max(d * d for d in dev) * 1e-6 + 1e-99
        p1 = dev[0] / 3 - dev[1] * 7 / 6 + dev[2] * 11 / 6
        p2 = -dev[1] / 6 + dev[2] * 5 / 6 + dev[3] / 3
        p3 = dev[2] / 3 + dev[3] * 5 / 6 - dev[4] / 6
        s1 = (dev[0] - 2 * dev[1] + dev[2]) ** 2 * 13 / 12 + (dev[0] - 4 * dev[1] + 3 * dev[2]) ** 2 / 4
        s2 = (dev[1] - 2 * dev[2] + dev[3]) ** 2 * 13 / 12 + (dev[1] - dev[3]) ** 2 / 4
        s3 = (dev[2] - 2 * dev[3] + dev[4]) ** 2 * 13 / 12 + (3 * dev[2] - 4 * dev[3] + dev[4]) ** 2 / 4
        a1, a2, a3 = .1 / (s1 + eps) ** 2, .6 / (s2 + eps) ** 2, .3 / (s3 + eps) ** 2
        out.append((a1 * p1 + a2 * p2 + a3 * p3) / (a1 + a2 + a3))
    return out


def face_form(phi):
    """(6 φ⁻, 6 φ⁺) of every cell of a clamped line, built face by face."""
    n = len(phi)
    at = lambda k: phi[min(max(k, 0), n - 1)]
    dm, dp = np.zeros(n), np.zeros(n)
    for f in range(-1, n):                      # face between f and f+1
        E = [at(f - 1 + q) - at(f - 2 + q) for q in range(5)]   # D_{f-1} .. D_{f+3}
        a, b, c, d = E[1] - E[0], E[2] - E[1], E[3] - E[2], E[4] - E[3]
        T1 = (c - b) - (b - a)                       # a - 2b + c
        T2 = (d - c) - (c - b)                       # b - 2c + d
        # the indicators and ε divided by 3 (12/3 = 4 times the reference's)
        is0 = 13 / 3 * (a - b) ** 2 + (a - 3 * b) ** 2
        is1 = 13 / 3 * (b - c) ** 2 + (b + c) ** 2
        is2 = 13 / 3 * (d - c) ** 2 + (3 * c - d) ** 2
        eps = max(e * e for e in E) * 4e-6 + 4e-99
        m, ex = np.frexp(eps)                        # eps = m·2^ex, m in [0.5, 1)
        sc, es = 2.0 ** (1 - ex), 2.0 * m            # exact power-of-two scale; es = eps·sc
        assert es == eps * sc and 1.0 <= es < 2.0
        t1, t2, t3 = (is0 * sc + es) ** 2, (is1 * sc + es) ** 2, (is2 * sc + es) ** 2
        A, T13, Cc = t2 * t3, t1 * t3, t1 * t2
        U, V = A * T1, Cc * T2
        s_left = E[1] + E[2]                          # D around cell f
        s_right = E[2] + E[3]                         # D around cell f+1
        if f + 1 < n:
            dm[f + 1] = 3 * s_right - (c - b) - (2 / 3 * U + V) / (A / 3 + 2 * T13 + Cc)
        if f >= 0:
            dp[f] = 3 * s_left - (c - b) + (U + 2 / 3 * V) / (A + 2 * T13 + Cc / 3)
    return dm, dp


def test_face_form_matches_reference():
    rng = np.random.default_rng(0)
    for trial in range(40):
        n = int(rng.integers(1, 24))
        kind = trial % 4
        x = np.arange(n) * 0.1
        if kind == 0:
            phi = rng.normal(size=n)
        elif kind == 1:
            phi = np.abs(x - rng.uniform(0, n * 0.1)) - 0.3          # kink
        elif kind == 2:
            phi = np.full(n, rng.normal())                             # flat: ε floor only
        else:
            phi = np.cumsum(rng.normal(size=n)) * 1e-3
        dm, dp = face_form(phi)
        for i in range(n):
            v = [phi[min(max(i + t - 3, 0), n - 1)] for t in range(7)]
            rm, rp = reference_weno(v)
            scale = max(1e-300, max(abs(q) for q in np.diff(v)) if n > 1 else 1.0)
            assert abs(dm[i] / 6 - rm) <= 1e-12 * scale, (trial, i)
            assert abs(dp[i] / 6 - rp) <= 1e-12 * scale, (trial, i)


def test_significand_equals_the_exact_scaling():
    """ε·2^-e, formed on the device by setting ε's exponent field to the bias, equals the
    product with the power-of-two scale bit for bit (both in FP64 and FP32)."""
    rng = np.random.default_rng(3)
    x = np.concatenate([4e-99 + rng.uniform(0, 1, 500) * 10.0 ** rng.uniform(-90, 10, 500), [4e-99, 1.0, 1.5, 2.0 ** 60]])
    bits = x.view(np.uint64)
    sig = ((bits & np.uint64(0x000FFFFFFFFFFFFF)) | np.uint64(0x3FF0000000000000)).view(np.float64)
    scale = ((np.uint64(2046) << np.uint64(52)) - (bits & np.uint64(0x7FF0000000000000))).view(np.float64)
    assert np.array_equal(sig, x * scale) and np.all((sig >= 1) & (sig < 2))
    xf = (4e-30 + rng.uniform(0, 1, 500) * 10.0 ** rng.uniform(-28, 10, 500)).astype(np.float32)
    fb = xf.view(np.uint32)
    sigf = ((fb & np.uint32(0x007FFFFF)) | np.uint32(0x3F800000)).view(np.float32)
    scalef = ((np.uint32(254) << np.uint32(23)) - (fb & np.uint32(0x7F800000))).view(np.float32)
    assert np.array_equal(sigf, xf * scalef)


def cell_form(v):
    """(6 φ⁻, 6 φ⁺) of one cell from its seven values in the cell, column and pair forms'
    arrangement (wenoCell): one face set per derivative, weights ten times the reference's
    (q2²q3², 6 q1²q3², 3 q1²q2²: the first without a product), candidate stencils six times."""
    D = [v[k + 1] - v[k] for k in range(6)]

    def weights(s1, s2, s3, eps):
        m, ex = np.frexp(eps)
        sc, es = 2.0 ** (1 - ex), 2.0 * m
        t1, t2, t3 = (s1 * sc + es) ** 2, (s2 * sc + es) ** 2, (s3 * sc + es) ** 2
        return t2 * t3, 6 * (t1 * t3), t1 * t2

    g = lambda a, b, c: 13 / 3 * (a - 2 * b + c) ** 2
    sL = lambda a, b, c: g(a, b, c) + (a - 4 * b + 3 * c) ** 2
    sM = lambda a, b, c: g(a, b, c) + (a - c) ** 2
    sR = lambda a, b, c: g(a, b, c) + (3 * a - 4 * b + c) ** 2
    st1 = lambda a, b, c: 2 * a - 7 * b + 11 * c
    st2 = lambda a, b, c: -a + 5 * b + 2 * c
    st3 = lambda a, b, c: 2 * a + 5 * b - c
    M = max(d * d for d in D[1:5])
    epsM, epsP = max(M, D[0] ** 2) * 4e-6 + 4e-99, max(M, D[5] ** 2) * 4e-6 + 4e-99
    a, b, c = weights(sL(*D[0:3]), sM(*D[1:4]), sR(*D[2:5]), epsM)
    P2, P3 = st2(*D[1:4]), st3(*D[2:5])
    m = (a * st1(*D[0:3]) + b * P2 + 3 * c * P3) / (a + b + 3 * c)
    a, b, c = weights(sL(*D[1:4]), sM(*D[2:5]), sR(*D[3:6]), epsP)
    p = (c * st1(D[5], D[4], D[3]) + b * P3 + 3 * a * P2) / (c + b + 3 * a)
    return m, p


def test_cell_form_matches_reference():
    rng = np.random.default_rng(1)
    for trial in range(400):
        kind = trial % 4
        x = np.arange(7) * 0.1
        if kind == 0:
            v = rng.normal(size=7)
        elif kind == 1:
            v = np.abs(x - rng.uniform(0, 0.7)) - 0.3          # kink
        elif kind == 2:
            v = np.full(7, rng.normal())                       # flat: ε floor only
        else:
            v = np.cumsum(rng.normal(size=7)) * 1e-3
        m, p = cell_form(list(v))
        rm, rp = reference_weno(list(v))
        scale = max(1e-300, max(abs(q) for q in np.diff(v)))
        assert abs(m / 6 - rm) <= 1e-12 * scale, trial
        assert abs(p / 6 - rp) <= 1e-12 * scale, trial
