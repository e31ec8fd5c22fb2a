"""Every launch plan of the WENO5 reinitialisation (one thread per cell, columns
along the last axis, one sweep per axis, columns reading TMA-staged plane tiles,
pairs of x-adjacent columns walked together, or those pairs reading TMA-staged plane
tiles, with several block sizes and walk lengths) gives the oracle's result, on ragged 2D and 3D shapes whose sizes are not
multiples of any block or chunk, and for iteration counts that leave the result in
each of the three rotating planes.  Shapes with rows of odd length run the column
form in place of the pair form; rows of 6 and 10 cells put every pair, or all but
one, within reach of the clamped edges."""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi
from helpers import band_error, linf

pytestmark = pytest.mark.gpu

PLANS = [("cells", 256, 0), ("columns", 64, 1), ("columns", 64, 4), ("columns", 128, 8), ("columns", 96, 32),
         ("columns", 256, 200), ("sweeps", 32, 1), ("sweeps", 64, 3), ("sweeps", 128, 16), ("sweeps", 256, 64),
         ("sweeps", 64, 500), ("tiled", 128, 1), ("tiled", 128, 5), ("tiled", 128, 8), ("tiled", 128, 100),
         ("pairs", 32, 1), ("pairs", 64, 8), ("pairs", 128, 5), ("pairs", 256, 200),
         ("pairs_tiled", 128, 1), ("pairs_tiled", 128, 3), ("pairs_tiled", 128, 8), ("pairs_tiled", 128, 200)]


def _field(shape, seed):
    """A distorted sphere/circle: |∇φ| far from 1, kinks where two blobs meet."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / max(shape)
    axes = [(np.arange(n) + 0.5) * dx for n in shape]
    grids = np.meshgrid(*axes, indexing="ij")
    c1 = [0.5 * n * dx + rng.uniform(-0.05, 0.05) for n in shape]
    c2 = [0.3 * n * dx for n in shape]
    d1 = np.sqrt(sum((g - c) ** 2 for g, c in zip(grids, c1))) - 0.25 * min(shape) * dx
    d2 = np.sqrt(sum((g - c) ** 2 for g, c in zip(grids, c2))) - 0.15 * min(shape) * dx
    phi = np.minimum(d1, d2) * (1.0 + 2.0 * np.minimum(d1, d2) ** 2 / dx)
    # numpy layout: reversed axes (x fastest)
    return np.ascontiguousarray(np.transpose(phi)), dx


# (72, 20, 24): rows of 16-byte multiples, so the tiled form stages the planes of its interior
# blocks by TMA while its edge blocks walk with global loads
# (36, 11, 13), (8, 5, 7), (4, 9, 6): rows of a multiple of 4 cells, so the tiled pair form stages
# its planes by TMA, with threads beyond the grid and clamped stencils reaching every tile edge
@pytest.mark.parametrize("shape,iters", [((37, 29), 12), ((23, 31, 41), 12), ((45, 6, 9), 7), ((5, 40, 3), 8), ((72, 20, 24), 9),
                                         ((6, 9, 11), 10), ((10, 13, 17), 11), ((36, 11, 13), 9), ((8, 5, 7), 7), ((4, 9, 6), 8)])
def test_plans_match_oracle(oracle_mod, garm_lib, shape, iters):
    phi0, dx = _field(shape, seed=len(shape))
    ref = oracle_mod.reinit(phi0, dx, iters, 0.5)
    try:
        for form, threads, cells in PLANS:
            for prec in (capi.PRECISION_FP64, capi.PRECISION_MIXED):
                capi.reinit_plan_set(shape, prec, form, threads, cells)
                out = capi.reinit_host(phi0, dx, iters, 0.5, prec)
                if prec == capi.PRECISION_FP64:
                    assert linf(out, ref) <= 1e-11 * dx, (form, threads, cells)
                else:
                    assert band_error(out, ref, ref, dx) <= 1e-3 * dx, (form, threads, cells)
    finally:
        for prec in (capi.PRECISION_FP64, capi.PRECISION_MIXED):
            capi.reinit_plan_set(shape, prec, "cells", 0, 0)


def test_autotuned_plan_reported(garm_lib):
    from garm import scenes
    sc = scenes.dam_break(3, 24)
    s = capi.Simulation(sc.grid, capi.default_config())
    plan = s.reinit_plan()
    assert plan["form"] in capi.REINIT_FORMS and 32 <= plan["threads"] <= 256 and plan["ms"] >= 0
    s.close()


def test_plan_set_rejects_bad_arguments(garm_lib):
    with pytest.raises(capi.GarmError):
        capi.reinit_plan_set((8, 8, 8), capi.PRECISION_FP64, "columns", 48, 4)   # not a multiple of 32
    with pytest.raises(capi.GarmError):
        capi.reinit_plan_set((8, 8, 8), capi.PRECISION_FP64, "sweeps", 512, 4)   # above the launch bound
    with pytest.raises(capi.GarmError):
        capi.reinit_plan_set((8, 8, 8), capi.PRECISION_FP64, "sweeps", 64, 0)    # empty walk
    with pytest.raises(capi.GarmError):
        capi.reinit_plan_set((8, 0, 8), capi.PRECISION_FP64, "columns", 64, 4)
