"""The oracle pinned to the reference itself.

oracle/_ref is the reference's own LevelSetLiquid<Dim> (Source/Core, unmodified),
compiled from the reference tree by oracle/build_ref.sh against the project's
Eigen/yaml-cpp subset shim.  These CPU tests drive it and the CPU port
(oracle/garm_oracle.cpp) through the same field/stage vocabulary from the same
scenes and require the two to agree BIT FOR BIT: stage by stage from a shared
evolved state, over whole steps (restarts included), over the 2D dam break
(128^2, 200 steps), and for the standalone WENO5 reinitialisation.  The GPU tests
check the kernels against the port; tests/test_gpu_golden.py checks them against
vectors the reference binary wrote (tests/golden/).

Two differences, neither in the fields: a reporting convention (the port counts the
PCG update that reaches the tolerance, Eigen's iteration counter, and so the
reference's, does not) and the order in which the volume diagnostic adds its cells
(fixed chunks in the port, so that it does not depend on the thread count).

Skipped where the reference binary is neither built nor buildable (no reference
sources on the machine).
"""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import STATE_FIELDS, host_default_config, load_scene

COMPARED = STATE_FIELDS + [capi.FIELD_FRACTION, capi.FIELD_CELL_DIST, capi.FIELD_NODE_DIST,
                           capi.FIELD_BOUNDARY_VELOCITY, capi.FIELD_BOUNDARY_NORMAL]


@pytest.fixture(scope="module")
def ref_mod(oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("reference binary not built and reference sources absent")
    oracle_mod.load_ref()
    return oracle_mod


def _pair(O, sc, **kw):
    p = O.OracleSim(sc.grid, host_default_config(**kw))
    r = O.RefSim(sc.grid, host_default_config(**kw))
    for s in (p, r):
        load_scene(s, sc)
    return p, r


def _same(p, r, fields=COMPARED, tag=""):
    for f in fields:
        a, b = p.download(f), r.download(f)
        assert np.array_equal(a, b), f"{tag}: {capi.FIELD_NAMES[f]} differs by {np.max(np.abs(a.astype(float) - b.astype(float))):.3e}"


SCENES = {
    "dam3d": lambda: scenes.dam_break(3, 16),
    "drop3d": lambda: scenes.drop(20, seed=3),
    "dam2d": lambda: scenes.dam_break(2, 40),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_port_equals_reference_over_steps(ref_mod, name):
    sc = SCENES[name]()
    p, r = _pair(ref_mod, sc)
    assert p.initialize() == capi.OK and r.initialize() == capi.OK
    _same(p, r, tag="initialize")
    p.stage("restart")
    r.stage("restart")
    _same(p, r, tag="restart")
    for k, dt in enumerate(scenes.frame_time_steps(r.max_speed, 4, 25, 1.0, sc.grid.spacing)):
        sp, sr = p.advance(dt), r.advance(dt)
        assert sp["restarted"] == sr["restarted"]
        assert sp["unknowns"] == sr["unknowns"]
        assert sp["cg_iterations"] == sr["cg_iterations"] + 1  # counting convention, see the module docstring
        _same(p, r, tag=f"step {k + 1}")
    assert p.max_speed() == r.max_speed()
    # the volume is a sum over cells; the port adds it in fixed chunks (independent of the
    # thread count), the reference in its own order
    assert abs(p.volume() - r.volume()) <= 1e-13 * abs(r.volume())


@pytest.mark.parametrize("name", ["dam3d", "drop3d"])
def test_port_equals_reference_stage_by_stage(ref_mod, name):
    """Each protected stage method of LevelSetLiquid<Dim> (LevelSetLiquid.h:145-169) from the same
    evolved state, on the port and on the reference."""
    sc = SCENES[name]()
    p, r = _pair(ref_mod, sc)
    for s in (p, r):
        s.initialize()
        s.stage("restart")
    for dt in scenes.frame_time_steps(r.max_speed, 2, 25, 1.0, sc.grid.spacing):
        p.advance(dt)
        r.advance(dt)
    snapshot = {f: r.download(f) for f in STATE_FIELDS}
    dt = 0.5 * sc.grid.spacing / max(r.max_speed(), 1e-3)
    for stage, arg in (("advect", dt), ("compose", 0.0), ("reinit", 0.0), ("extrap_collider", 0.0), ("restart", 0.0),
                       ("body_force", dt), ("project", 0.0), ("extrap_air", 0.0), ("enforce_bc", 0.0),
                       ("enforce_boundary_level_set", 3 * sc.grid.spacing)):
        for s in (p, r):
            for f, v in snapshot.items():
                s.upload(f, v)
            s.stage(stage, arg)
        _same(p, r, STATE_FIELDS, tag=stage)
    for s in (p, r):
        for f, v in snapshot.items():
            s.upload(f, v)
    assert p.stage("rm_check")[0] == r.stage("rm_check")[0]


def test_port_equals_reference_2d_dam_break_200_steps(ref_mod, capsys):
    """The 2D dam break on a 128^2 MAC grid for 200 steps at CFL 1 (a configuration of the
    benchmark suite), restarts included: identical bits at every step."""
    sc = scenes.dam_break(2, 128)
    p, r = _pair(ref_mod, sc)
    for s in (p, r):
        s.initialize()
        s.stage("restart")
    restarts = 0
    for k, dt in enumerate(scenes.frame_time_steps(r.max_speed, 200, 25, 1.0, sc.grid.spacing)):
        sp, sr = p.advance(dt), r.advance(dt)
        assert sp["restarted"] == sr["restarted"], k
        restarts += sr["restarted"]
        if k % 25 == 24 or k == 199:
            _same(p, r, [capi.FIELD_LEVEL_SET, capi.FIELD_VELOCITY, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD], tag=f"step {k + 1}")
    with capsys.disabled():
        print(f"\n[port vs reference binary, 2D dam break 128^2] 200 steps, {restarts} restarts, identical bits")
    assert restarts > 0


def test_reinit_equals_reference(ref_mod):
    """Reinitialization::solve<5> on TestReinit's distorted circle (TestReinit.cpp:89-101)."""
    n, length = 100, 10.0
    dx = length / n
    x = (np.arange(n) + 0.5) * dx - length / 2
    X, Y = np.meshgrid(x, x, indexing="xy")
    r = np.sqrt(X * X + Y * Y)
    r0 = 0.2313 * length
    phi0 = (np.exp(r - r0) - 1) * 0.05
    assert np.array_equal(ref_mod.reinit(phi0, dx, 100, 0.5), ref_mod.ref_reinit(phi0, dx, 100, 0.5))
    z = np.linspace(-1, 1, 24)
    phi3 = np.sqrt(sum(g * g for g in np.meshgrid(z, z, z, indexing="ij"))) - 0.5
    assert np.array_equal(ref_mod.reinit(phi3, 2 / 23, 30, 0.9), ref_mod.ref_reinit(phi3, 2 / 23, 30, 0.9))


def test_reference_refuses_other_constants(ref_mod):
    sc = scenes.dam_break(3, 8)
    for kw in ({"reinit_iters": 10}, {"rm_threshold": -1.0}, {"precision": capi.PRECISION_MIXED}, {"restart_newton": 1}):
        with pytest.raises(ValueError):
            ref_mod.RefSim(sc.grid, host_default_config(**kw))
