"""The grid barrier of the persistent kernels (the pressure solve, the fast-marching
relaxation) through garm_barrier_selftest: its cost per barrier across all SMs, and its
bounded wait.  The wait is made to run out with a count that no block ever completes (no
fault, no trap); the call returns GARM_TIMEOUT and the context stays usable."""
from __future__ import annotations

import time

import numpy as np
import pytest

from garm import capi, scenes
from helpers import host_default_config, load_scene

pytestmark = pytest.mark.gpu


def test_barrier_rounds_complete(garm_lib, capsys):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for blocks in (1, sms):
        st, ms = capi.barrier_selftest(blocks, 20000)
        assert st == capi.OK
        assert 0 < ms < 0.05
        with capsys.disabled():
            print(f"\n[grid barrier, {blocks} blocks] {ms * 1e3:.2f} us per barrier")
    assert capi.barrier_selftest(sms * 64, 10)[0] == capi.INVALID  # beyond co-residency


def test_barrier_wait_is_bounded_and_the_context_survives(garm_lib):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    t0 = time.perf_counter()
    st, _ = capi.barrier_selftest(sms, 5, never_complete=True)
    wall = time.perf_counter() - t0
    assert st == capi.TIMEOUT
    assert 1.0 < wall < 20.0
    # the device still runs work: a step of a small scene
    sc = scenes.dam_break(3, 16)
    g = capi.Simulation(sc.grid, host_default_config())
    load_scene(g, sc)
    assert g.initialize() == capi.OK
    assert g.advance(0.005)["status"] == capi.OK
    assert np.all(np.isfinite(g.download(capi.FIELD_LEVEL_SET)))
    assert capi.barrier_selftest(sms, 100)[0] == capi.OK


def test_fp64_peak_selftest(garm_lib, capsys):
    """The FP64 FMA throughput the plain form's stencils are measured against: positive and
    below the nominal 1.25 TFLOP/s of a GB300 by no more than a timing margin."""
    tf = capi.fp64_peak_tflops()
    with capsys.disabled():
        print(f"\n[FP64 FMA peak] {tf:.3f} TFLOP/s")
    assert 0.1 < tf < 5.0
