"""GPU kernels against vectors written by the reference itself.

tests/golden/*.npz come from the reference binary (the reference's own LevelSetLiquid,
built from its sources by oracle/build_ref.sh; see tests/golden/make_golden.py).  Here
the plain FP64 GPU form runs the same scenes with the same dt sequence through the C
ABI and is compared with them: the parity gate φ L∞ <= 1e-6·dx on every cell, the
velocity on the fluid faces and ξ to 1e-9, the advection flags exactly, and the same
restart decisions at every step.  Over the 200 steps of the 2D dam break the gate on
the level-set band (|φ| <= 15·dx) is 1e-9·dx; beyond the band the file's record of the
reference's own spread under ulp changes of its initial state is printed beside the GPU
difference (the reinitialisation amplifies rounding there, see test_oracle_kat.py).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from garm import capi, scenes
from helpers import LEVEL_SET_BAND, host_default_config, load_scene, velocity_check

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _run(sc, gold, check):
    """Initialize, restart and the recorded steps on the GPU; check(step, sim, stats) after each."""
    assert np.float64(np.sum(sc.phi)) == gold["phi0_sum"], "scene generator changed since the golden vectors were written"
    g = capi.Simulation(sc.grid, host_default_config(record_volume=1))
    load_scene(g, sc)
    assert g.initialize() == capi.OK
    g.stage("restart")
    for k, dt in enumerate(gold["dts"], 1):
        st = g.advance(float(dt))
        assert st["restarted"] == gold["restarted"][k - 1], f"step {k}: restart decision"
        assert st["unknowns"] == gold["unknowns"][k - 1], f"step {k}: unknowns"
        check(k, g, st)
    g.close()


@pytest.mark.parametrize("name,make", [("dam3d_12", lambda: scenes.dam_break(3, 12)),
                                       ("drop3d_12_seed3", lambda: scenes.drop(12, seed=3))])
def test_fp64_matches_reference_vectors(garm_lib, capsys, name, make):
    gold = np.load(GOLDEN / f"{name}.npz")
    sc = make()
    dx = sc.grid.spacing
    worst = {"phi": 0.0, "u": 0.0, "xi": 0.0}

    def check(k, g, st):
        if f"phi_{k}" in gold:
            e = float(np.max(np.abs(g.download(capi.FIELD_LEVEL_SET) - gold[f"phi_{k}"]))) / dx
            worst["phi"] = max(worst["phi"], e)
            assert e <= 1e-6, f"step {k}: phi {e:.3e} dx"
        if f"u_{k}" in gold:
            inner, _ = velocity_check(g.download(capi.FIELD_VELOCITY), gold[f"u_{k}"], g.download(capi.FIELD_FRACTION), 1e-9)
            worst["u"] = max(worst["u"], inner)
            assert inner <= 1e-9, f"step {k}: u {inner:.3e}"
        if f"xi_{k}" in gold:
            e = float(np.max(np.abs(g.download(capi.FIELD_REF_MAP) - gold[f"xi_{k}"]))) / dx
            worst["xi"] = max(worst["xi"], e)
            assert e <= 1e-9, f"step {k}: xi {e:.3e} dx"
        if f"adv_{k}" in gold:
            assert np.array_equal(g.download(capi.FIELD_ADV_REGION), gold[f"adv_{k}"])
        assert abs(st["volume"] - gold["volume"][k - 1]) <= 1e-9 * abs(gold["volume"][k - 1])

    _run(sc, gold, check)
    with capsys.disabled():
        print(f"\n[GPU FP64 vs reference binary, {name}] phi {worst['phi']:.2e} dx, u {worst['u']:.2e}, xi {worst['xi']:.2e} dx")


def test_fp64_2d_dam_break_200_steps_against_reference(garm_lib, capsys):
    """The 2D dam break, 128^2 MAC grid, 200 steps at CFL 1, against the reference binary:
    drift of φ, u and ξ at steps 1, 10, 50 and 200, restart decisions at every step, and the
    volume diagnostic of every step (the reference records it inside advance,
    LevelSetLiquid.cpp:663)."""
    gold = np.load(GOLDEN / "dam2d_128_200.npz")
    sc = scenes.dam_break(2, 128)
    dx = sc.grid.spacing
    rows, vols = [], []

    def check(k, g, st):
        vols.append(st["volume"])
        if f"phi_{k}" not in gold:
            return
        pr = gold[f"phi_{k}"]
        d = np.abs(g.download(capi.FIELD_LEVEL_SET) - pr) / dx
        band = np.abs(pr) <= LEVEL_SET_BAND * dx
        row = {"step": k, "phi_band": float(d[band].max()), "phi_all": float(d.max()),
               "ref_spread_all": float(gold[f"spread_phi_{k}"].max()) / dx}
        if f"u_{k}" in gold:
            row["u"], _ = velocity_check(g.download(capi.FIELD_VELOCITY), gold[f"u_{k}"], g.download(capi.FIELD_FRACTION), 1e-9)
            row["xi"] = float(np.max(np.abs(g.download(capi.FIELD_REF_MAP) - gold[f"xi_{k}"]))) / dx
        rows.append(row)
        assert row["phi_band"] <= 1e-9, row
        assert row.get("u", 0) <= 1e-9 and row.get("xi", 0) <= 1e-9, row

    _run(sc, gold, check)
    vref = gold["volume"]
    dv = np.abs(np.array(vols) - vref) / np.abs(vref)
    with capsys.disabled():
        print(f"\n[GPU FP64 vs reference binary, 2D dam break 128^2, 200 steps, {int(gold['restarted'].sum())} restarts]")
        for r in rows:
            print("  " + ", ".join(f"{k} {v:.2e}" if isinstance(v, float) else f"{k} {v}" for k, v in r.items()))
        print(f"  volume: max relative difference {dv.max():.2e}; drift over the run {(vref[-1] - vref[0]) / vref[0]:+.3%} "
              f"(reference) vs {(vols[-1] - vols[0]) / vols[0]:+.3%} (GPU)")
    assert dv.max() <= 1e-9
