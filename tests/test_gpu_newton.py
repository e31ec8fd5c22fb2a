"""GPU parity of the Newton configuration (the reference built with _ENABLE_NEWTON_ and
without FMM): compose keeps ∇φ = Πᵀ∇φ₀(ξ), initialize takes ψ0 from the level set's
4th-order gradient, and restart() is HybridNewton's closest-point restart
(LevelSetLiquid.cpp:1290-1308; HybridNewton.h:59-467; HybridNewton.cpp:30-118).

Tolerances (FP64 plain form):
  * the restart of a smooth level set (a sphere): φ0 within 1e-9·dx, ψ0 within 1e-8 (the
    Newton loop stops on a threshold, so a rounding difference can end it one step apart,
    far below the 1e-3·dx³ stopping tolerance); ξ, Π exact;
  * compose and initialize: the stage tolerance of the plain configuration (1e-11);
  * the restart of a simulated scene and steps that restart every time: the reference
    algorithm is ill-conditioned there (a 1e-15 relative change of its input moves some
    cells by a sizeable fraction of dx), so the GPU is held to the oracle's own spread
    under such perturbations (of the inputs of one restart, or entering before every step):
    a 99th percentile and a maximum deviation at most 10x the oracle's, and as large a
    share of cells within 1e-9·dx, less 3 (one restart) or 5 (three steps) points.
"""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import (STATE_FIELDS, assert_conditioning_parity, conditioning_parity, host_default_config, linf,
                     load_scene, newton_sphere_case, oracle_spread, perturbed, perturbed_steps, rel)

pytestmark = pytest.mark.gpu

NEWTON_FIELDS = STATE_FIELDS + [capi.FIELD_LEVEL_SET_GRAD]


def newton_pair(oracle_mod, grid, **kw):
    cfg = host_default_config(restart_newton=1, **kw)
    return capi.Simulation(grid, cfg), oracle_mod.OracleSim(grid, host_default_config(restart_newton=1))


@pytest.mark.parametrize("dim,n", [(3, 24), (2, 48)])
def test_newton_restart_stage_on_a_sphere(oracle_mod, garm_lib, dim, n):
    grid, phi, grad, sdf = newton_sphere_case(n, dim)
    g, o = newton_pair(oracle_mod, grid)
    for s in (g, o):
        s.upload(capi.FIELD_LEVEL_SET, phi.ravel())
        s.upload(capi.FIELD_ORI_LEVEL_SET, phi.ravel())
        s.upload(capi.FIELD_LEVEL_SET_GRAD, grad.ravel())
        s.stage("restart")
    dx = 1.0 / n
    rg, ro = g.download(capi.FIELD_REF_LEVEL_SET), o.download(capi.FIELD_REF_LEVEL_SET)
    assert linf(rg, ro) <= 1e-9 * dx
    assert linf(g.download(capi.FIELD_REF_LEVEL_SET_GRAD), o.download(capi.FIELD_REF_LEVEL_SET_GRAD)) <= 1e-8
    assert linf(g.download(capi.FIELD_LEVEL_SET_GRAD), o.download(capi.FIELD_LEVEL_SET_GRAD)) <= 1e-8
    assert np.array_equal(g.download(capi.FIELD_ORI_LEVEL_SET), rg)
    assert np.array_equal(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP))
    assert np.array_equal(g.download(capi.FIELD_REF_MAP_GRAD), o.download(capi.FIELD_REF_MAP_GRAD))
    band = np.abs(sdf.ravel()) <= 6 * dx
    assert np.max(np.abs(rg - sdf.ravel())[band]) < 1e-3 * dx


def advanced_newton_state(oracle_mod, scene, steps):
    o = oracle_mod.OracleSim(scene.grid, host_default_config(restart_newton=1))
    load_scene(o, scene)
    o.initialize()
    o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, steps, 25, 1.0, scene.grid.spacing):
        o.advance(dt)
    return o


SCENES = {"dam3d": lambda: scenes.dam_break(3, 20), "drop3d": lambda: scenes.drop(20, seed=3),
          "dam2d": lambda: scenes.dam_break(2, 40)}


@pytest.mark.parametrize("name", ["drop3d", "dam2d"])
def test_newton_initialize_compose_and_restart_stages(oracle_mod, garm_lib, capsys, name):
    sc = SCENES[name]()
    g, o = newton_pair(oracle_mod, sc.grid)
    load_scene(g, sc)
    load_scene(o, sc)
    g.initialize()
    o.initialize()
    for f in (capi.FIELD_LEVEL_SET_GRAD, capi.FIELD_REF_LEVEL_SET_GRAD):
        assert rel(g.download(f), o.download(f)) <= 1e-11, capi.FIELD_NAMES[f]
    assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-9 * sc.grid.spacing
    # stages from an advanced oracle state copied to both sides
    adv = advanced_newton_state(oracle_mod, sc, 3)
    snapshot = {f: adv.download(f) for f in NEWTON_FIELDS}

    def load(sim, size=0.0, seed=0):
        for f, v in snapshot.items():
            if size and f in (capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET, capi.FIELD_LEVEL_SET_GRAD):
                v = perturbed(v, size, seed + f)
            sim.upload(f, v)

    load(g); load(o)
    g.stage("compose"); o.stage("compose")
    for f in (capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET, capi.FIELD_LEVEL_SET_GRAD):
        assert rel(g.download(f), o.download(f)) <= 1e-11, f"compose: {capi.FIELD_NAMES[f]}"
    # The restart is ill-conditioned in places (closest-point iterations that end after 20
    # capped steps without converging, and eikonal traces along a vanishing gradient): the
    # comparison is measured against the oracle's own spread under ulp-level perturbations.
    def run(size, seed):
        s = oracle_mod.OracleSim(sc.grid, host_default_config(restart_newton=1))
        load(s, size, seed)
        s.stage("restart")
        return s.download(capi.FIELD_REF_LEVEL_SET)

    base, spread = oracle_spread(run)
    load(g)
    g.stage("restart")
    dx = sc.grid.spacing
    st = conditioning_parity(g.download(capi.FIELD_REF_LEVEL_SET), base, spread, dx)
    with capsys.disabled():
        print(f"\n[newton restart stage, {name}] " + ", ".join(f"{k} {v:.3e}" for k, v in st.items()))
    assert_conditioning_parity(st)
    o.upload(capi.FIELD_LEVEL_SET, snapshot[capi.FIELD_LEVEL_SET])
    load(o)
    o.stage("restart")
    assert np.array_equal(o.download(capi.FIELD_REF_LEVEL_SET), base)  # the unperturbed run is reproducible
    assert np.array_equal(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP))
    norms = np.linalg.norm(g.download(capi.FIELD_REF_LEVEL_SET_GRAD).reshape(-1, sc.grid.dim), axis=1)
    assert np.all((np.abs(norms - 1) < 1e-12) | (norms == 0))


@pytest.mark.parametrize("name", ["dam3d", "drop3d", "dam2d"])
def test_newton_steps_with_restarts_parity_gate(oracle_mod, garm_lib, capsys, name):
    """rm_threshold = -1: the reference-map test fails every step, so every step ends with
    the HybridNewton restart.  After three steps φ is compared against the oracle's own
    spread under ulp-level perturbations entering at every step."""
    sc = SCENES[name]()
    cfg = host_default_config(restart_newton=1, rm_threshold=-1.0)
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
    pg = g.download(capi.FIELD_LEVEL_SET)
    st = conditioning_parity(pg, base, spread, dx)
    band = np.abs(base) <= dx
    with capsys.disabled():
        print(f"\n[newton steps, restart every step, {name}] " + ", ".join(f"{k} {v:.3e}" for k, v in st.items())
              + f", band(1dx) max gpu {np.max(np.abs(pg - base)[band]) / dx:.3e} oracle {np.max(spread[band]) / dx:.3e}")
    assert_conditioning_parity(st, share_slack=0.05)


def test_newton_auto_steps_equal_host_driven_steps(garm_lib):
    """Device-resident steps (graph replay, restart gated on the device) reproduce
    host-driven steps bit for bit in the Newton configuration, restart included."""
    sc = scenes.dam_break(3, 20)
    cfg = host_default_config(restart_newton=1, rm_threshold=-1.0)
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
    assert st["restarted"] == 1
    for f in NEWTON_FIELDS:
        assert np.array_equal(host.download(f), auto.download(f)), capi.FIELD_NAMES[f]


def test_newton_mixed_precision_band(oracle_mod, garm_lib, capsys):
    """Mixed form in the Newton configuration against the FP64 oracle, restart every step:
    FP32 rounding is a far larger perturbation than the ulp-level ones above, so the band
    |φ| <= 3dx is held to its median (1e-4·dx) and 90th-percentile (0.1·dx) deviation."""
    sc = scenes.drop(20, seed=3)
    g = capi.Simulation(sc.grid, host_default_config(restart_newton=1, rm_threshold=-1.0, precision=capi.PRECISION_MIXED))
    o = oracle_mod.OracleSim(sc.grid, host_default_config(restart_newton=1, rm_threshold=-1.0))
    load_scene(g, sc)
    load_scene(o, sc)
    g.initialize(); o.initialize()
    g.stage("restart"); o.stage("restart")
    dx = sc.grid.spacing
    for dt in scenes.frame_time_steps(o.max_speed, 2, 25, 1.0, dx):
        g.advance(dt); o.advance(dt)
    po = o.download(capi.FIELD_LEVEL_SET)
    band = np.abs(po) <= 3 * dx
    d = np.abs(g.download(capi.FIELD_LEVEL_SET) - po)[band] / dx
    q50, q90, q99 = np.quantile(d, [0.5, 0.9, 0.99])
    with capsys.disabled():
        print(f"\n[newton, mixed vs FP64 oracle, drop 20^3] phi band(3dx) median {q50:.3e} dx, q90 {q90:.3e}, "
              f"q99 {q99:.3e}, max {d.max():.3e}")
    assert q50 <= 1e-4 and q90 <= 0.1


def test_newton_save_and_load_keeps_psi0(oracle_mod, garm_lib):
    """loadFrame in the Newton configuration takes ψ0 from the frame (refLevelSetGrad.sav)
    instead of recomputing it (LevelSetLiquid.cpp:500-510); steps after a save/load
    round trip equal uninterrupted steps."""
    sc = scenes.dam_break(3, 16)
    cfg = host_default_config(restart_newton=1)
    a = capi.Simulation(sc.grid, cfg)
    load_scene(a, sc)
    a.initialize()
    a.stage("restart")
    a.advance(0.01)
    saved = {f: a.download(f) for f in (capi.FIELD_VELOCITY, capi.FIELD_REF_MAP, capi.FIELD_REF_LEVEL_SET,
                                         capi.FIELD_ADV_REGION, capi.FIELD_REF_MAP_GRAD, capi.FIELD_REF_LEVEL_SET_GRAD)}
    b = capi.Simulation(sc.grid, cfg)
    b.upload(capi.FIELD_LEVEL_SET, sc.phi.ravel())  # boundary set-up only
    for f, v in saved.items():
        b.upload(f, v)
    b.finish_load()
    assert np.array_equal(b.download(capi.FIELD_REF_LEVEL_SET_GRAD), saved[capi.FIELD_REF_LEVEL_SET_GRAD])
    for s in (a, b):
        s.advance(0.01)
    assert np.array_equal(a.download(capi.FIELD_LEVEL_SET), b.download(capi.FIELD_LEVEL_SET))
