"""GPU parity of the fast-marching configuration (the reference built with _ENABLE_FMM_):
reinitializeLevelSet is FastMarching over a band of 15 cells (LevelSetLiquid.cpp:1151-1152),
and with the Newton configuration the restart ends with a fast-marching sweep
(HybridNewton.cpp:51-64).  Both flags together are the reference's default build.

The GPU solves the fast-marching equations by parallel relaxation instead of a serial heap;
the oracle restates the heap algorithm.  Tolerances (FP64):
  * fast marching of a level set: 1e-12·dx (the two agree to the last bits except where a
    neighbour ties with the root);
  * steps in the fast-marching configuration: φ L∞ <= 1e-6·dx;
  * with the Newton restart, which is ill-conditioned on simulated scenes, the oracle's own
    spread under ulp-level perturbations (as in the Newton tests).
"""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import (STATE_FIELDS, assert_conditioning_parity, conditioning_parity, host_default_config, linf,
                     load_scene, newton_sphere_case, oracle_spread, perturbed_steps)

pytestmark = pytest.mark.gpu


def march_on_gpu(phi, grid, precision=capi.PRECISION_FP64):
    g = capi.Simulation(grid, host_default_config(fast_marching=1, precision=precision))
    g.upload(capi.FIELD_LEVEL_SET, phi.ravel())
    g.stage("reinit")
    return g.download(capi.FIELD_LEVEL_SET)


@pytest.mark.parametrize("dim,n", [(2, 96), (3, 40)])
def test_fast_marching_matches_oracle(oracle_mod, garm_lib, dim, n):
    grid, phi, _, sdf = newton_sphere_case(n, dim)
    dx = 1.0 / n
    phi = phi + 0.05 * dx * np.sin(np.arange(phi.size) * 0.7).reshape(phi.shape)
    out_o = oracle_mod.fast_marching(phi, dx, 15).ravel()
    out_g = march_on_gpu(phi, grid)
    assert linf(out_g, out_o) <= 1e-12 * dx
    assert np.max(np.abs(out_g)) <= 15 * dx
    # the mixed form marches in FP32
    out_m = march_on_gpu(phi, grid, capi.PRECISION_MIXED)
    assert linf(out_m, out_o) <= 1e-4 * dx


def test_fast_marching_plane_and_edge_cases(oracle_mod, garm_lib):
    """An axis-aligned plane marches exactly; a level set with no sign change stays at the
    band width; exact zeros on the interface are seeds at distance 0."""
    n, dx = 40, 1.0 / 40
    grid = capi.grid_desc(3, [n, 8, 8], dx, [0.5, 4 * dx, 4 * dx])
    x = (np.arange(n) + 0.5) * dx
    phi = np.broadcast_to((x - 0.3137)[None, None, :], (8, 8, n)).copy() * 3.0
    out = march_on_gpu(phi, grid)
    assert linf(out, oracle_mod.fast_marching(phi, dx, 15).ravel()) <= 1e-12 * dx
    exact = np.broadcast_to((x - 0.3137)[None, None, :], (8, 8, n)).ravel()
    inband = np.abs(exact) < 14.5 * dx
    assert np.max(np.abs(out - exact)[inband]) < 1e-12
    allpos = np.ones((8, 8, n))
    assert np.array_equal(march_on_gpu(allpos, grid), np.full(allpos.size, 15 * dx))
    zeros = phi.copy()
    zeros[:, :, 12] = 0.0
    assert linf(march_on_gpu(zeros, grid), oracle_mod.fast_marching(zeros, dx, 15).ravel()) <= 1e-12 * dx


SCENES = {"dam3d": lambda: scenes.dam_break(3, 20), "drop3d": lambda: scenes.drop(20, seed=3),
          "dam2d": lambda: scenes.dam_break(2, 40)}


@pytest.mark.parametrize("name", list(SCENES))
def test_fast_marching_configuration_steps(oracle_mod, garm_lib, name):
    sc = SCENES[name]()
    cfg = host_default_config(fast_marching=1)
    g = capi.Simulation(sc.grid, cfg)
    o = oracle_mod.OracleSim(sc.grid, cfg)
    load_scene(g, sc)
    load_scene(o, sc)
    assert g.initialize() == capi.OK and o.initialize() == capi.OK
    dx = sc.grid.spacing
    assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-12 * dx
    g.stage("restart"); o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, 3, 25, 1.0, dx):
        sg, so = g.advance(dt), o.advance(dt)
        assert sg["restarted"] == so["restarted"] and sg["unknowns"] == so["unknowns"]
    err = linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET))
    assert err <= 1e-6 * dx, f"phi err {err / dx:.3e} dx"


def test_default_build_newton_restart_on_a_sphere(oracle_mod, garm_lib):
    """The reference's default build (Newton + fast marching): the restart of a smooth level
    set matches the oracle closely.  It redistances it exactly next to the interface (Newton
    closest points) and to first order beyond (fast marching)."""
    grid, phi, grad, sdf = newton_sphere_case(24, 3)
    cfg = host_default_config(restart_newton=1, fast_marching=1)
    g = capi.Simulation(grid, cfg)
    o = oracle_mod.OracleSim(grid, cfg)
    for s in (g, o):
        s.upload(capi.FIELD_LEVEL_SET, phi.ravel())
        s.upload(capi.FIELD_ORI_LEVEL_SET, phi.ravel())
        s.upload(capi.FIELD_LEVEL_SET_GRAD, grad.ravel())
        s.stage("restart")
    dx = 1.0 / 24
    rg = g.download(capi.FIELD_REF_LEVEL_SET)
    assert linf(rg, o.download(capi.FIELD_REF_LEVEL_SET)) <= 1e-9 * dx
    assert linf(g.download(capi.FIELD_REF_LEVEL_SET_GRAD), o.download(capi.FIELD_REF_LEVEL_SET_GRAD)) <= 1e-8
    err = np.abs(rg - sdf.ravel())
    assert np.max(err[np.abs(sdf.ravel()) <= dx]) < 1e-9 * dx
    assert np.mean(err[np.abs(sdf.ravel()) <= 3 * dx]) < 0.05 * dx
    norms = np.linalg.norm(g.download(capi.FIELD_REF_LEVEL_SET_GRAD).reshape(-1, 3), axis=1)
    assert np.all((np.abs(norms - 1) < 1e-12) | (norms == 0))


@pytest.mark.parametrize("name", ["dam3d", "drop3d"])
def test_default_build_steps_with_restarts(oracle_mod, garm_lib, capsys, name):
    """Newton + fast marching, restart every step: measured against the oracle's own spread."""
    sc = SCENES[name]()
    cfg = host_default_config(restart_newton=1, fast_marching=1, rm_threshold=-1.0)
    dx = sc.grid.spacing
    dts = [0.004, 0.004, 0.004]

    def run(size, seed):
        return perturbed_steps(oracle_mod, sc, cfg, dts, size, seed).download(capi.FIELD_LEVEL_SET)

    base, spread = oracle_spread(run)
    g = capi.Simulation(sc.grid, cfg)
    load_scene(g, sc)
    g.initialize()
    g.stage("restart")
    for dt in dts:
        assert g.advance(dt)["restarted"] == 1
    st = conditioning_parity(g.download(capi.FIELD_LEVEL_SET), base, spread, dx)
    with capsys.disabled():
        print(f"\n[newton + fast marching, restart every step, {name}] " + ", ".join(f"{k} {v:.3e}" for k, v in st.items()))
    assert_conditioning_parity(st, share_slack=0.05)


def test_default_build_auto_steps_equal_host_driven_steps(garm_lib):
    """Graph replay with the gated restart and the cooperative relaxation inside it
    reproduces host-driven steps bit for bit."""
    sc = scenes.dam_break(3, 20)
    cfg = host_default_config(restart_newton=1, fast_marching=1, rm_threshold=-1.0)
    sims = []
    for _ in range(2):
        s = capi.Simulation(sc.grid, cfg)
        load_scene(s, sc)
        s.initialize()
        s.stage("restart")
        sims.append(s)
    host, auto = sims
    for dt in scenes.frame_time_steps(host.max_speed, 4, 25, 1.0, sc.grid.spacing):
        host.advance(dt)
    auto.set_clock(25, 1.0)
    auto.advance_auto(1)
    st = auto.advance_auto(3)
    assert st["status"] == capi.OK and st["restarted"] == 1
    for f in STATE_FIELDS + [capi.FIELD_LEVEL_SET_GRAD]:
        assert np.array_equal(host.download(f), auto.download(f)), capi.FIELD_NAMES[f]
