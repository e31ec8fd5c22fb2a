"""Device-resident stepping (garm_sim_advance_auto): dt from max|u| and the frame
clock on the device, the restart decision as a device flag, one synchronisation
per call, captured step graphs when available.  It must reproduce the host-driven
loop (Simulator::advanceTimeBySteps around advance, Common/Util/Simulator.cpp:102-128)."""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import host_default_config, linf, load_scene

pytestmark = pytest.mark.gpu


def _make(scene, **cfg):
    s = capi.Simulation(scene.grid, host_default_config(**cfg))
    load_scene(s, scene)
    s.initialize()
    s.stage("restart")
    return s


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_MIXED])
def test_auto_steps_equal_host_driven_steps(garm_lib, capsys, precision):
    sc = scenes.dam_break(3, 24)
    host = _make(sc, precision=precision)
    auto = _make(sc, precision=precision)
    steps = 7
    for dt in scenes.frame_time_steps(host.max_speed, steps, 25, 1.0, sc.grid.spacing):
        host.advance(dt)
    auto.set_clock(25, 1.0)
    st = auto.advance_auto(3)
    st = auto.advance_auto(steps - 3)  # two calls: the frame clock and buffer roles carry over
    assert st["status"] == capi.OK
    for f in (capi.FIELD_LEVEL_SET, capi.FIELD_VELOCITY, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD, capi.FIELD_ADV_REGION):
        assert np.array_equal(host.download(f), auto.download(f)), capi.FIELD_NAMES[f]
    with capsys.disabled():
        print(f"\n[auto stepping, precision {precision}] graph replay: {auto.graph_active()}, last step cg {st['cg_iterations']} it")


def test_auto_steps_match_oracle_and_restart(oracle_mod, garm_lib):
    """rm_threshold = -1 fails checkReferenceMap every step, so the device-gated
    restart branch runs each step; the dam break has no wall-condition ties, so
    both sides choose the same dt sequence."""
    sc = scenes.dam_break(3, 20)
    cfg = dict(rm_threshold=-1.0)
    g = _make(sc, **cfg)
    o = oracle_mod.OracleSim(sc.grid, host_default_config(**cfg))
    load_scene(o, sc)
    o.initialize()
    o.stage("restart")
    restarts_o = 0
    for dt in scenes.frame_time_steps(o.max_speed, 5, 25, 1.0, sc.grid.spacing):
        restarts_o += o.advance(dt)["restarted"]
    g.set_clock(25, 1.0)
    st = g.advance_auto(5)
    dx = sc.grid.spacing
    assert restarts_o == 5 and st["restarted"] == 1
    assert linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) <= 1e-6 * dx
    assert linf(g.download(capi.FIELD_REF_MAP), o.download(capi.FIELD_REF_MAP)) <= 1e-9


def test_interleaving_auto_and_single_stages(garm_lib):
    """Host-dt steps and single stages between graph replays keep the buffer roles right."""
    sc = scenes.dam_break(3, 16)
    a = _make(sc)
    b = _make(sc)
    a.set_clock(25, 1.0)
    b.set_clock(25, 1.0)
    a.advance_auto(2)
    b.advance_auto(2)
    for s in (a, b):
        s.advance(0.004)
    a.advance_auto(3)
    b.advance_auto(1); b.advance_auto(2)
    assert np.array_equal(a.download(capi.FIELD_LEVEL_SET), b.download(capi.FIELD_LEVEL_SET))
    assert np.array_equal(a.download(capi.FIELD_VELOCITY), b.download(capi.FIELD_VELOCITY))
