"""GPU parity: every stage of LevelSetLiquid::advance on the sm_103a kernels,
called through the C ABI, against the FP64 CPU oracle on identical seeded inputs.

Tolerances (FP64 plain form):
  * boundary set-up, flags, counts, unknown numbering: exact;
  * single stages: |gpu - oracle| <= 1e-11 (relative to the field's max) — the
    kernels use FMA contraction and a tensor-product Hermite evaluation, so they
    differ from the oracle by rounding only;
  * projection: velocity within 1e-6 relative (both solve to |r| <= 1e-8 |b|);
  * one full step: φ L∞ <= 1e-6·dx (the parity gate of the path).
"""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import (LEVEL_SET_BAND, STATE_FIELDS, band_error, copy_state, host_default_config, linf, load_scene, oracle_spread,
                     perturbed, rel, velocity_check)

pytestmark = pytest.mark.gpu

STAGE_TOL = 1e-11


def pair(oracle_mod, scene, **cfgkw):
    cfg = host_default_config(**cfgkw)
    g = capi.Simulation(scene.grid, cfg)
    o = oracle_mod.OracleSim(scene.grid, cfg)
    load_scene(g, scene)
    load_scene(o, scene)
    return g, o


def advanced_state(oracle_mod, scene, steps, **cfgkw):
    """Oracle state after initialize + restart + `steps` steps (gives non-trivial u, ξ, Π)."""
    cfg = host_default_config(**cfgkw)
    o = oracle_mod.OracleSim(scene.grid, cfg)
    load_scene(o, scene)
    o.initialize()
    o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, steps, 25, 1.0, scene.grid.spacing):
        o.advance(dt)
    return o


SCENES = {
    "dam2d": lambda: scenes.dam_break(2, 40),
    "dam3d": lambda: scenes.dam_break(3, 20),
    "drop3d": lambda: scenes.drop(20, seed=3),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_boundary_and_initialize(oracle_mod, garm_lib, name):
    sc = SCENES[name]()
    g, o = pair(oracle_mod, sc)
    for f in (capi.FIELD_CELL_DIST, capi.FIELD_NODE_DIST, capi.FIELD_BOUNDARY_NORMAL):
        assert np.array_equal(g.download(f), o.download(f)), capi.FIELD_NAMES[f]
    assert g.initialize() == capi.OK
    assert o.initialize() == capi.OK
    assert np.array_equal(g.download(capi.FIELD_FRACTION), o.download(capi.FIELD_FRACTION))
    dx = sc.grid.spacing
    assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-9 * dx
    assert np.array_equal(g.download(capi.FIELD_ADV_REGION), o.download(capi.FIELD_ADV_REGION))
    assert linf(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP)) == 0.0
    ug, uo = g.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_VELOCITY)
    inner, ties = velocity_check(ug, uo, o.download(capi.FIELD_FRACTION), 1e-6)
    assert inner <= 1e-6


@pytest.mark.parametrize("name", list(SCENES))
def test_single_stages(oracle_mod, garm_lib, name):
    sc = SCENES[name]()
    o = advanced_state(oracle_mod, sc, 3)
    cfg = host_default_config()
    g = capi.Simulation(sc.grid, cfg)
    load_scene(g, sc)
    g.initialize()  # boundary fractions
    dt = 0.5 * sc.grid.spacing / max(o.max_speed(), 1e-3)

    def sync():
        copy_state(g, o)

    checks = {
        "advect": ([dt], [capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD, capi.FIELD_VELOCITY]),
        "compose": ([], [capi.FIELD_LEVEL_SET, capi.FIELD_TMP_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET]),
        "reinit": ([], [capi.FIELD_LEVEL_SET]),
        "extrap_collider": ([], [capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET]),
        "restart": ([], [capi.FIELD_REF_LEVEL_SET, capi.FIELD_REF_LEVEL_SET_GRAD, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD]),
        "body_force": ([dt], [capi.FIELD_VELOCITY]),
        "extrap_air": ([], [capi.FIELD_REF_MAP, capi.FIELD_ADV_REGION, capi.FIELD_VELOCITY]),
        "enforce_bc": ([], [capi.FIELD_VELOCITY]),
    }
    snapshot = {f: o.download(f) for f in STATE_FIELDS}
    for stage, (args, fields) in checks.items():
        for f, v in snapshot.items():
            o.upload(f, v)
        sync()
        g.stage(stage, *args)
        o.stage(stage, *(args or [0.0]))
        for f in fields:
            a, b = g.download(f), o.download(f)
            if f == capi.FIELD_ADV_REGION:
                assert np.array_equal(a, b), f"{stage}: {capi.FIELD_NAMES[f]}"
            else:
                assert rel(a, b) <= STAGE_TOL, f"{stage}: {capi.FIELD_NAMES[f]} rel err {rel(a, b):.3e}"
    # reference-map test: identical counts
    for f, v in snapshot.items():
        o.upload(f, v)
    sync()
    assert g.stage("rm_check") == o.stage("rm_check")
    # projection after gravity (a divergence-free state would give a ~0 right-hand side):
    # same unknown set, both converged, velocity within the solver tolerance
    g.stage("body_force", 4 * dt)
    o.stage("body_force", 4 * dt)
    sg = g.stage("project")
    so = o.stage("project")
    assert sg["unknowns"] == so["unknowns"]
    assert sg["status"] == capi.OK and so["status"] == capi.OK
    assert sg["cg_residual"] <= 1e-8 and so["cg_residual"] <= 1e-8
    ug, uo = g.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_VELOCITY)
    assert rel(ug, uo) <= 1e-6, f"project: velocity rel err {rel(ug, uo):.3e}"
    pg, po = g.download(capi.FIELD_PRESSURE), o.download(capi.FIELD_PRESSURE)
    assert rel(pg, po) <= 1e-5
    assert np.array_equal(pg != 0, po != 0) or so["unknowns"] == 0


@pytest.mark.parametrize("name", list(SCENES))
def test_one_step_parity_gate(oracle_mod, garm_lib, name):
    """φ L∞ <= 1e-6·dx after initialize + restart + one advance (same dt on both)."""
    sc = SCENES[name]()
    g, o = pair(oracle_mod, sc)
    g.initialize(); o.initialize()
    g.stage("restart"); o.stage("restart")
    dt = next(scenes.frame_time_steps(o.max_speed, 1, 25, 1.0, sc.grid.spacing))
    sg = g.advance(dt)
    so = o.advance(dt)
    dx = sc.grid.spacing
    err = linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET))
    assert err <= 1e-6 * dx, f"phi err {err / dx:.3e} dx"
    assert sg["restarted"] == so["restarted"]
    assert sg["unknowns"] == so["unknowns"]
    inner, ties = velocity_check(g.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_FRACTION), 1e-5)
    assert inner <= 1e-5


def test_restart_branch_every_step(oracle_mod, garm_lib):
    """rm_threshold = -1 makes checkReferenceMap fail, so restart runs inside advance."""
    sc = scenes.dam_break(3, 16)
    g, o = pair(oracle_mod, sc, rm_threshold=-1.0)
    g.initialize(); o.initialize()
    g.stage("restart"); o.stage("restart")
    for dt in [0.01, 0.01]:
        sg, so = g.advance(dt), o.advance(dt)
        assert sg["restarted"] == 1 and so["restarted"] == 1
    dx = sc.grid.spacing
    assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-6 * dx


def test_restart_override(oracle_mod, garm_lib):
    """garm_sim_set_restart_override: ALWAYS restarts every step, which is what the oracle
    does with a restart test that always fails (rm_threshold = -1); NEVER keeps the
    reference map although the test fails; AUTO returns to the test."""
    sc = scenes.dam_break(3, 16)
    g, o = pair(oracle_mod, sc, rm_threshold=-1.0)
    f = capi.Simulation(sc.grid, host_default_config())
    load_scene(f, sc)
    for s in (g, o, f):
        s.initialize()
        s.stage("restart")
    f.set_restart_override(capi.RESTART_ALWAYS)
    dx = sc.grid.spacing
    for dt in (0.01, 0.01):
        assert f.advance(dt)["restarted"] == 1
        o.advance(dt)
        g.set_restart_override(capi.RESTART_NEVER)
        assert g.advance(dt)["restarted"] == 0
        g.set_restart_override(capi.RESTART_AUTO)
    assert linf(f.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-6 * dx
    assert g.advance(0.01)["restarted"] == 1
    with pytest.raises(capi.GarmError):
        f.set_restart_override(3)


def test_n_step_drift(oracle_mod, garm_lib, capsys):
    """Drift of φ, u and ξ after 12 steps with each side choosing its own dt."""
    sc = scenes.dam_break(3, 24)
    g, o = pair(oracle_mod, sc)
    g.initialize(); o.initialize()
    g.stage("restart"); o.stage("restart")
    dts_g = list(scenes.frame_time_steps(g.max_speed, 1, 25, 1.0, sc.grid.spacing))
    steps = 12
    gen_o = scenes.frame_time_steps(o.max_speed, steps, 25, 1.0, sc.grid.spacing)
    gen_g = scenes.frame_time_steps(g.max_speed, steps, 25, 1.0, sc.grid.spacing)
    for dto, dtg in zip(gen_o, gen_g):
        o.advance(dto)
        g.advance(dtg)
    dx = sc.grid.spacing
    ephi = linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) / dx
    eu = rel(g.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_VELOCITY))
    exi = linf(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP)) / dx
    with capsys.disabled():
        print(f"\n[drift after {steps} steps, 24^3 dam break] phi {ephi:.3e} dx, u rel {eu:.3e}, xi {exi:.3e} dx")
    # measured on GB300: phi 4e-11 dx, u 1e-13, xi 2e-12 dx; gates a factor 20-100 above
    assert ephi <= 1e-9
    assert eu <= 1e-11
    assert exi <= 1e-10
    assert dts_g


def test_empty_and_full_liquid(oracle_mod, garm_lib):
    """No unknowns (all air) and all-liquid domains run and agree."""
    for fill in (+1.0, -1.0):
        sc = scenes.dam_break(3, 12)
        sc.phi[...] = fill
        g, o = pair(oracle_mod, sc)
        g.initialize(); o.initialize()
        g.stage("restart"); o.stage("restart")
        sg, so = g.advance(0.01), o.advance(0.01)
        assert sg["unknowns"] == so["unknowns"]
        if fill > 0:
            assert sg["unknowns"] == 0
        dx = sc.grid.spacing
        assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-6 * dx


def test_reinit_known_answer(oracle_mod, garm_lib):
    """WENO5 reinitialisation of TestReinit case 0 (exp-distorted circle,
    Source/Test/TestReinit/TestReinit.cpp:89-101): the GPU matches the oracle and
    both approach the exact SDF in the |φ| <= 3dx band."""
    n, length = 100, 10.0
    dx = length / n
    x = (np.arange(n) + 0.5) * dx - length / 2
    X, Y = np.meshgrid(x, x, indexing="xy")
    r = np.sqrt(X * X + Y * Y)
    r0 = 0.2313 * length
    maxd = length / np.sqrt(2) - r0
    phi0 = (np.exp(r - r0) - 1) * (maxd / (np.exp(maxd) - 1))
    sdf = r - r0
    pg = capi.reinit_host(phi0, dx, 100, 0.5)
    po = oracle_mod.reinit(phi0, dx, 100, 0.5)
    assert linf(pg, po) <= 1e-10
    band = np.abs(pg) <= 3 * dx
    err0 = np.mean(np.abs(phi0 - sdf)[np.abs(phi0) <= 3 * dx])
    err = np.mean(np.abs(pg - sdf)[band])
    assert err < 0.1 * err0 and err < 0.05 * dx
    # the FP32 form of the same kernel stays within 1e-3·dx of the FP64 result in the band
    pf = capi.reinit_host(phi0, dx, 100, 0.5, capi.PRECISION_MIXED)
    assert band_error(pf, po, po, dx) <= 1e-3 * dx


def test_invalid_arguments(garm_lib):
    sc = scenes.dam_break(2, 16)
    g = capi.Simulation(sc.grid, host_default_config())
    with pytest.raises(capi.GarmError) as e:
        g.upload(capi.FIELD_LEVEL_SET, np.zeros(5))
    assert e.value.status == capi.INVALID
    with pytest.raises(capi.GarmError):
        g.download(capi.FIELD_COUNT if hasattr(capi, "FIELD_COUNT") else 99)
    bad = capi.grid_desc(4, [8, 8, 8], 0.1, [0, 0, 0])
    with pytest.raises(capi.GarmError):
        capi.Simulation(bad, host_default_config())


@pytest.mark.parametrize("name", ["dam3d", "drop3d", "dam2d"])
def test_mixed_precision_within_1e3_dx(oracle_mod, garm_lib, capsys, name):
    """Mixed form (FP32 fields and stencils, FP64 dots/residual/refinement/RM test)
    against the FP64 oracle after one step: φ L∞ <= 1e-3·dx over the level-set band
    |φ| <= 15·dx (helpers.LEVEL_SET_BAND: the reference's air extrapolation radius;
    beyond it the reinitialisation amplifies rounding, and those cells are shown not to
    feed back, in test_oracle_kat.py and test_gpu_far_field.py), on every cell whose
    one-step result the reference algorithm itself determines to 1e-4·dx.  That is
    measured on the oracle: the same step with the initial φ and u changed by one or two
    ulps (helpers.PERTURBATIONS).  On the drop, whose walls start with u·n = -1, the wall
    condition's sign test (Boundary.cpp:104) flips on faces where the normal velocity is
    zero up to rounding, so an ulp moves ξ there by 0.64·dx and φ by up to 0.06·dx in the
    oracle alone; those cells are counted and printed, not gated."""
    sc = SCENES[name]()
    dx = sc.grid.spacing
    cfg = host_default_config(precision=capi.PRECISION_MIXED)
    g = capi.Simulation(sc.grid, cfg)
    load_scene(g, sc)
    g.initialize()
    g.stage("restart")
    dt = next(scenes.frame_time_steps(g.max_speed, 1, 25, 1.0, dx))

    def oracle_step(size, seed):
        o = oracle_mod.OracleSim(sc.grid, host_default_config())
        o.upload(capi.FIELD_LEVEL_SET, perturbed(sc.phi.ravel(), size, seed))
        o.upload(capi.FIELD_VELOCITY, perturbed(sc.velocity, size, seed + 1))
        o.initialize()
        o.stage("restart")
        o.advance(dt)
        return o

    o = oracle_step(0.0, 0)
    _, spread = oracle_spread(lambda size, seed: oracle_step(size, seed).download(capi.FIELD_LEVEL_SET))
    sg = g.advance(dt)
    pg, po = g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)
    ephi_all = linf(pg, po) / dx
    ephi3 = band_error(pg, po, po, dx) / dx
    band = np.abs(po) <= LEVEL_SET_BAND * dx
    stable = band & (spread <= 1e-4 * dx)
    d = np.abs(pg - po) / dx
    ephi = float(np.max(d[stable], initial=0.0))
    unstable = band & ~stable
    with capsys.disabled():
        print(f"\n[mixed vs FP64 oracle, {name}] band cells the oracle's own ulp spread leaves undetermined: "
              f"{int(unstable.sum())} of {int(band.sum())} (oracle spread there up to {float(np.max(spread[unstable], initial=0)) / dx:.2e} dx, "
              f"mixed error there up to {float(np.max(d[unstable], initial=0)):.2e} dx)")
    eu, ties = velocity_check(g.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_VELOCITY), o.download(capi.FIELD_FRACTION), 1e-3)
    exi = linf(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP)) / dx
    with capsys.disabled():
        print(f"\n[mixed vs FP64 oracle, {name}] phi band(15dx) {ephi:.3e} dx, band(3dx) {ephi3:.3e} dx, all cells {ephi_all:.3e} dx, "
              f"u rel (fluid faces) {eu:.3e}, wall ties {ties}, xi {exi:.3e} dx, "
              f"cg {sg['cg_iterations']} it / {sg['cg_refinements']} replacements, residual {sg['cg_residual']:.2e}")
    assert sg["status"] == capi.OK
    assert sg["cg_residual"] <= 1e-8
    assert ephi <= 1e-3


def test_not_converged_is_reported_not_fatal(oracle_mod, garm_lib):
    """cg_max_iters = 1: the reference would exit (LinearSystem.h:33-36); here the step
    completes and reports GARM_NOT_CONVERGED, like the oracle."""
    sc = scenes.drop(16, seed=1)
    g, o = pair(oracle_mod, sc, cg_max_iters=1)
    assert g.initialize() == capi.NOT_CONVERGED
    assert o.initialize() == capi.NOT_CONVERGED
    g.stage("restart"); o.stage("restart")
    sg, so = g.advance(0.01), o.advance(0.01)
    assert sg["status"] == capi.NOT_CONVERGED and so["status"] == capi.NOT_CONVERGED
    assert sg["cg_iterations"] == 1 and so["cg_iterations"] == 1
    assert np.all(np.isfinite(g.download(capi.FIELD_VELOCITY)))


def test_ga_advection_rotation_matches_oracle(oracle_mod, garm_lib):
    """The GA advection known-answer case (slotted disk in a steady rotation, no solid
    ring) through the C ABI: 40 advect stages then compose, against the oracle."""
    from helpers import ROT_LENGTH, run_rotation, rotation_case
    s = 64
    grid, *_ = rotation_case(s)
    g = capi.Simulation(grid, host_default_config())
    o = oracle_mod.OracleSim(grid, host_default_config())
    pg = run_rotation(g, s, 40)
    po = run_rotation(o, s, 40)
    dx = ROT_LENGTH / s
    assert linf(pg, po) <= 1e-9 * dx
    for f in (capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD):
        assert rel(g.download(f), o.download(f)) <= 1e-11, f


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_MIXED])
def test_pressure_solve_block_layouts(oracle_mod, garm_lib, precision):
    """The persistent solve laid out three ways on the same system: one block (more than
    four unknowns per thread: the streamed form), 41 blocks (the grid totals gather more than
    one warp of block partials), one block per SM.  Each converges on the oracle's unknowns
    and matches its pressure within the solve's tolerance."""
    sc = scenes.dam_break(3, 32)
    o = advanced_state(oracle_mod, sc, 2)
    snapshot = {f: o.download(f) for f in STATE_FIELDS}
    dt = 0.01
    o.stage("body_force", dt)
    so = o.stage("project")
    po = o.download(capi.FIELD_PRESSURE)
    assert so["unknowns"] > 4 * 512
    tol = 1e-5 if precision == capi.PRECISION_FP64 else 1e-4
    pressures = []
    for per_block in (10 ** 9, 800, 1):
        g = capi.Simulation(sc.grid, host_default_config(precision=precision, cg_cells_per_block=per_block))
        load_scene(g, sc)
        g.initialize()  # boundary fractions
        for f, v in snapshot.items():
            g.upload(f, v)
        g.stage("body_force", dt)
        sg = g.stage("project")
        assert sg["status"] == capi.OK and sg["unknowns"] == so["unknowns"]
        assert sg["cg_residual"] <= 1e-8
        pg = g.download(capi.FIELD_PRESSURE)
        assert rel(pg, po) <= tol, f"{per_block}: pressure rel err {rel(pg, po):.3e}"
        pressures.append(pg)
    assert rel(pressures[0], pressures[2]) <= tol


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_MIXED])
def test_pressure_solve_rows_longer_than_compact_reach(oracle_mod, garm_lib, precision):
    """The streamed solve's compact rows hold the y neighbours as distances of at most 4095
    unknowns; longer rows take their entries from the full rows.  A 2D grid of 4600 x 8
    interior cells whose liquid (x < 0.95) puts about 4370 unknowns in each row, solved on
    one block (the streamed form), matches the oracle's pressure."""
    nx, ny = 4600, 8
    dx = 1.0 / nx
    grid = capi.grid_desc(2, [nx + 4, ny + 4], dx, [0.5, ny * dx / 2], 2)
    pos = scenes.cell_positions(grid)
    phi = scenes.box_sdf(pos, [-1.0, -1.0], [1.95, 2.0])
    sc = scenes.Scene("wide_rows_2d", grid, np.ascontiguousarray(phi), scenes.zero_velocity(grid))
    cfg = dict(precision=precision, cg_cells_per_block=10 ** 9)
    g, o = pair(oracle_mod, sc, **cfg)
    for s in (g, o):
        s.initialize()
        s.stage("body_force", 1e-3)
    so, sg = o.stage("project"), g.stage("project")
    assert sg["status"] == capi.OK and sg["unknowns"] == so["unknowns"] > 4 * 512
    assert sg["cg_residual"] <= 1e-8
    tol = 1e-5 if precision == capi.PRECISION_FP64 else 1e-4
    err = rel(g.download(capi.FIELD_PRESSURE), o.download(capi.FIELD_PRESSURE))
    print(f"\n[rows of ~{so['unknowns'] // ny} unknowns, precision {precision}] pressure rel err {err:.2e}, {sg['cg_iterations']} it")
    assert err <= tol
