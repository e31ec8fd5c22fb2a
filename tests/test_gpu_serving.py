"""Batched scenes and the serving loop: several scenes advance concurrently on
their own streams, and each scene's result is the same alone and in the mix
(bit-identical: a scene's kernels touch only its own state and its solver grid
depends only on its own size)."""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes, serving
from helpers import host_default_config, load_scene

pytestmark = pytest.mark.gpu


def _sim(scene, precision, cfg=None):
    s = capi.Simulation(scene.grid, cfg if cfg is not None else host_default_config(precision=precision))
    load_scene(s, scene)
    s.initialize()
    s.stage("restart")
    s.set_clock(25, 1.0)
    return s


@pytest.mark.parametrize("precision", [capi.PRECISION_FP64, capi.PRECISION_MIXED])
def test_batch_equals_alone(garm_lib, precision):
    scs = [scenes.dam_break(3, 16), scenes.drop(20, seed=2), scenes.random_pool_scene(24, seed=7)]
    alone = []
    for sc in scs:
        s = _sim(sc, precision)
        s.advance_auto(6)
        alone.append(s.download(capi.FIELD_LEVEL_SET))
        s.close()
    sims = [_sim(sc, precision) for sc in scs]
    stats = capi.batch_advance_auto(sims, 6)
    assert len(stats) == 3
    for s, ref in zip(sims, alone):
        assert np.array_equal(s.download(capi.FIELD_LEVEL_SET), ref)


def test_serving_results_equal_alone_and_budget_respected(garm_lib, capsys):
    reqs = serving.make_requests(6, rate=200.0, seed=3, n_range=(16, 28), steps_range=(4, 9))
    # a budget that fits about three of these scenes at once forces queueing and reuse of memory
    cfg = capi.default_config(precision=capi.PRECISION_MIXED)
    one = max(capi.estimate_bytes(scenes.unit_grid(3, r.n), cfg) for r in reqs)
    server = serving.Server(budget_bytes=3.2 * one, keep_phi=True, chunk=2)
    out = server.run(reqs)
    assert out["requests"] == 6
    assert out["peak_resident_bytes"] <= server.budget
    assert out["peak_active"] >= 2  # requests overlapped on the device
    for res in out["results"]:
        req = next(r for r in reqs if r.rid == res.rid)
        sc = serving.build_scene(req)
        s = _sim(sc, capi.PRECISION_MIXED, server.cfg)  # the same solver partition as in the mix
        s.advance_auto(req.steps)
        assert np.array_equal(s.download(capi.FIELD_LEVEL_SET), res.phi), f"request {req.rid}"
        s.close()
    with capsys.disabled():
        print(f"\n[serving] {out['requests']} requests, peak {out['peak_active']} resident, "
              f"p50/p99 step {out['p50_step_ms']:.2f}/{out['p99_step_ms']:.2f} ms, "
              f"p50/p99 e2e {out['p50_e2e_s']:.3f}/{out['p99_e2e_s']:.3f} s")
