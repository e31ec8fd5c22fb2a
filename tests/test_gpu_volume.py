"""Volume diagnostic (LevelSetLiquid::calculateVolume, LevelSetLiquid.cpp:1162-1190) on
the GPU against the oracle, on the tmp level set of real scenes, in both corner orders."""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import host_default_config, load_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_MIXED])
@pytest.mark.parametrize("name", ["dam3d", "drop3d", "dam2d", "pool3d"])
def test_volume_matches_oracle(oracle_mod, garm_lib, name, precision):
    sc = {"dam3d": lambda: scenes.dam_break(3, 40), "drop3d": lambda: scenes.drop(36, seed=5),
          "dam2d": lambda: scenes.dam_break(2, 96), "pool3d": lambda: scenes.random_pool_scene(44, seed=9)}[name]()
    g = capi.Simulation(sc.grid, host_default_config(precision=precision))
    load_scene(g, sc)
    g.initialize()
    g.stage("restart")
    g.stage("compose")
    tmp = g.download(capi.FIELD_TMP_LEVEL_SET).astype(np.float64).reshape(tuple(reversed(
        [sc.grid.resolution[a] for a in range(sc.grid.dim)])))
    dx = sc.grid.spacing
    for order in (False, True):
        vg = g.volume(evaluator_order=order)
        vo = oracle_mod.field_volume(tmp, dx, evaluator_order=order)
        assert abs(vg - vo) <= 1e-12 * abs(vo), (order, vg, vo)
    if precision == capi.PRECISION_FP64:
        o = oracle_mod.OracleSim(sc.grid, host_default_config())
        load_scene(o, sc)
        o.initialize()
        o.stage("restart")
        o.stage("compose")
        assert abs(g.volume() - o.volume()) <= 1e-10 * abs(o.volume())
        o.close()
    g.close()


def test_volume_rejects_bad_order(garm_lib):
    sc = scenes.dam_break(3, 16)
    g = capi.Simulation(sc.grid, host_default_config())
    v = capi.C.c_double()
    assert g.lib.garm_sim_volume(g.handle, 2, capi.C.byref(v)) == capi.INVALID
    assert g.lib.garm_sim_volume(g.handle, 0, None) == capi.INVALID
    g.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_volume_recorded_per_step(oracle_mod, garm_lib, dim):
    """record_volume: every step's statistics carry the volume of tmp, computed on the
    device inside the step (also inside replayed step graphs) and equal to the volume
    the synchronous call gives for the same state."""
    sc = scenes.dam_break(dim, 32 if dim == 3 else 64)
    cfg = host_default_config(record_volume=1)
    g = capi.Simulation(sc.grid, cfg)
    load_scene(g, sc)
    g.initialize()
    g.stage("restart")
    g.set_clock(25, 1.0)
    vols = []
    for _ in range(4):
        st = g.advance_auto(1)
        vols.append(st["volume"])
        assert st["volume"] == g.volume()
    assert all(v > 0 for v in vols)
    assert g.graph_active()
    g.close()
