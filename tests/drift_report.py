"""Drift of the plain FP64 GPU form against the CPU oracle over a whole run.

    python tests/drift_report.py [--dim 3] [--n 128] [--steps 100] [--spread]

The FP64 form and the oracle (which gives the same bits as the reference's own code,
tests/test_ref_pin.py) advance the same dam break with one dt sequence, the Simulator's
CFL-1 policy on the GPU's velocity.  At steps 1, 10, 50 and the last, it prints the
per-field differences (bench.field_errors: φ over the band |φ| <= 15·dx, over |φ| <= 3·dx,
by |φ| bin and over all cells; u on the fluid faces; ξ), the restart counts and the volume
diagnostic of both.  With --spread, the oracle also runs from a state one or two ulps away
(every value times 1 + U(-1e-15, 1e-15)), and its distance from the unperturbed oracle is
printed beside the GPU's: the reference algorithm's own conditioning.  It prints one JSON
line.  A report, not a pytest test: at 128^3 the oracle takes minutes.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
sys.path.insert(0, str(REPO))

import bench  # noqa: E402
from garm import capi, scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--dim", type=int, default=3)
    p.add_argument("--n", type=int, default=128)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--spread", action="store_true")
    args = p.parse_args()
    capi.load()
    sc = scenes.dam_break(args.dim, args.n)
    dx = sc.grid.spacing
    g = capi.Simulation(sc.grid, capi.default_config(precision=capi.PRECISION_FP64, record_volume=1))
    o = O.OracleSim(sc.grid, g.cfg)
    sims = [g, o]
    q = None
    if args.spread:
        q = O.OracleSim(sc.grid, g.cfg)
        sims.append(q)
    for s in sims:
        phi0, u0 = sc.phi.ravel(), sc.velocity
        if s is q:
            rng = np.random.default_rng(11)
            phi0 = phi0 * (1 + 1e-15 * rng.uniform(-1, 1, phi0.shape))
            u0 = u0 * (1 + 1e-15 * rng.uniform(-1, 1, u0.shape))
        s.upload(capi.FIELD_LEVEL_SET, phi0)
        s.upload(capi.FIELD_VELOCITY, u0)
        s.initialize()
        s.stage("restart")
    K = args.steps
    marks = {m for m in (1, 10, 50, K) if 1 <= m <= K}
    rows, vg, vo, rg, ro = {}, [], [], 0, 0
    t_cpu = 0.0
    for k, dt in enumerate(scenes.frame_time_steps(g.max_speed, K, 25, 1.0, dx), 1):
        sg = g.advance(dt)
        t0 = time.perf_counter()
        so = o.advance(dt)
        t_cpu += time.perf_counter() - t0
        if q is not None:
            q.advance(dt)
        rg += sg["restarted"]
        ro += so["restarted"]
        vg.append(sg["volume"])
        vo.append(o.volume())
        if k in marks:
            rows[str(k)] = {"restarts_gpu": rg, "restarts_oracle": ro, **bench.field_errors(g, o, dx),
                            "volume_rel_diff": abs(vg[-1] - vo[-1]) / abs(vo[-1])}
            if q is not None:
                rows[str(k)]["oracle_ulp_spread"] = bench.field_errors(q, o, dx)
    for s in sims:
        s.close()
    print(json.dumps({"workload": f"{args.dim}D dam break {args.n}^{args.dim}, plain FP64 GPU form against the CPU oracle, {K} steps",
                      "drift": rows, "volume_drift_gpu": (vg[-1] - vg[0]) / vg[0], "volume_drift_oracle": (vo[-1] - vo[0]) / vo[0],
                      "cpu_s_per_step": t_cpu / K}), flush=True)


if __name__ == "__main__":
    main()
