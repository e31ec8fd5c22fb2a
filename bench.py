#!/usr/bin/env python
"""Benchmark of the GB300 GARM-LS per-timestep pipeline.

Workload: the 3D dam break on a 128^3 MAC grid (unit cube, solid walls, liquid
{x<0.4, y<0.5, z<0.6} at rest, gravity -9.8, CFL 1.0, frame rate 25, WENO5 x30
reinitialisation every step, Jacobi-PCG to rel tol 1e-8).  A step is one
LevelSetLiquid::advance(dt) of the whole scene.  `value` is interior cell-steps
per second of the plain FP64 form measured with CUDA events over exactly K
steps; the state (> 1 GB) is larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl garm|reference]
                  [--workload dam|batch|serve|drop]

The default line also carries the mixed form, the reference's default build, the 48-scene
batch, the end-to-end figure through the C ABI, per-stage times, the roofline of the
reinitialisation sub-stage, and the CPU oracle: its speed and, at full size, the per-field
differences between the FP64 form and it after one step.

Under torchrun each rank advances its own replica of the scene (replicas
only: the path does not shard), `value` = all ranks' cell-steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
sys.path.insert(0, str(REPO))

METRIC = "cell-steps/s mixed vs FP64 on 1 GB300 at φ err≤1e-3·dx; p50/p99 step latency"
UNIT = "cell-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["garm", "reference"], default="garm")
    p.add_argument("--n", type=int, default=None, help="interior cells per axis (128; 256 for the drop workload)")
    p.add_argument("--precision", choices=["fp64", "mixed"], default="fp64", help="form timed as `value`")
    p.add_argument("--no-mixed", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--no-default-build", action="store_true",
                   help="skip the same workload in the reference's default build (Newton restart + fast marching)")
    p.add_argument("--seed", type=int, default=0, help="drop: seed of the sphere's centre")
    p.add_argument("--workload", choices=["dam", "dam2d", "batch", "serve", "drop", "reinit"], default="dam",
                   help="dam: the 128^3 dam break (default line, with mixed and batch sub-objects); "
                        "dam2d: the 2D dam break on a 128^2 grid, FP64 and mixed, with the CPU oracle beside them; "
                        "batch: 48 uneven pool scenes only; serve: the Poisson request stream only; "
                        "drop: the 256^3 drop into a pool, mixed against FP64 over K steps with per-field errors; "
                        "reinit: the dam break's reinitialisation stage alone, K times after W (for profiling one kernel)")
    p.add_argument("--spread", action="store_true",
                   help="drop: also run the FP64 form from an initial state changed by one ulp and report its "
                        "deviation at the same steps (the algorithm's own conditioning)")
    p.add_argument("--batch-scenes", type=int, default=48)
    p.add_argument("--batch-cg-cells", type=int, default=None,
                   help="batch: interior cells per pressure-solve block (default: the measured best)")
    p.add_argument("--batch-streams", type=int, default=None,
                   help="batch: streams the scenes share, round robin (default: one per scene)")
    p.add_argument("--reinit-plan", default=None, metavar="FORM,THREADS,CELLS",
                   help="pin the reinitialisation launch plan of the dam-break grid instead of autotuning it")
    p.add_argument("--requests", type=int, default=48, help="serve: number of requests")
    p.add_argument("--serve-requests", type=int, default=12, help="requests of the serving leg of the default line")
    p.add_argument("--no-serve", action="store_true")
    args = p.parse_args()
    if args.n is None:
        args.n = 256 if args.workload == "drop" else 128
    return args


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dam_config(n: int, precision: str, world: int) -> dict:
    """The workload description both arms print (the repo arm and --impl reference)."""
    return {"workload": f"3D dam break {n}^3 MAC grid, {'plain FP64' if precision == 'fp64' else 'mixed FP32/FP64'} form",
            "n": n, "interior_cells": n ** 3, "storage_cells": (n + 4) ** 3, "cfl": 1.0, "frame_rate": 25,
            "reinit": "WENO5 x30 every step", "pcg_tol": 1e-8, "replicas": world,
            "l2": "no flush: device state > 1 GB, larger than L2"}


def reduce_max(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, interior_cells: int, steps: int, max_elapsed_ms: float) -> float:
    """Whole-job cell-steps/s: every rank advances its own replica of the scene."""
    return world * interior_cells * steps / (max_elapsed_ms * 1e-3)


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def state_fields():
    from garm import capi
    return [capi.FIELD_VELOCITY, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD, capi.FIELD_REF_LEVEL_SET,
            capi.FIELD_REF_LEVEL_SET_GRAD, capi.FIELD_ADV_REGION]


PROFILED_PLANS = {  # (form, precision) -> ncu summary of that WENO5 sub-stage at 128^3
    ("sweeps", "fp64"): "weno_sweeps_fp64_dam_break_128.txt",
    ("columns", "mixed"): "weno_columns_f32_dam_break_128.txt",
    ("pairs", "mixed"): "weno_pairs_f32_dam_break_128.txt",
}


def profiled_pipe(plan: dict, precision: str, n: int):
    """The compute pipe that bounds the profiled WENO5 sub-stage and its busy fraction
    (mean over the captured launches of the ncu pipe metric), from the summary under profiles/."""
    name = PROFILED_PLANS.get((plan["form"], precision))
    p = REPO / "profiles" / name if name else None
    if n != 128 or p is None or not p.exists():
        return None
    metric = "sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active" if precision == "fp64" \
        else "smsp__issue_active.avg.pct_of_peak_sustained_active"
    text = p.read_text().splitlines()
    frac = [float(ln.split(":")[1]) for ln in text if ln.startswith("issue_active_frac:")]
    if frac and precision != "fp64":
        vals = [100 * frac[0]]
    else:
        vals = []
        for ln in text:
            parts = ln.split()
            if ln.startswith(metric) and len(parts) > 1:
                try:
                    vals.append(float(parts[1]))
                except ValueError:
                    pass
    if not vals:
        return None
    return {"pipe": "fp64" if precision == "fp64" else "issue", "metric": metric,
            "frac": round(sum(vals) / len(vals) / 100, 3), "source": f"profiles/{name}"}


def profiled_traffic(plan: dict, precision: str, n: int):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the ncu
    capture summarised under profiles/, when it was taken on this workload size and for
    the launch form the autotuner picked here (None otherwise)."""
    name = PROFILED_PLANS.get((plan["form"], precision))
    p = REPO / "profiles" / name if name else None
    if n != 128 or p is None or not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("traffic_bytes_per_launch:"):
            return int(ln.split(":")[1])
    return None


def profiled_fp64_ops(plan: dict):
    """FP64 operations per storage cell and sub-stage (2·DFMA + DADD + DMUL executed, from
    the ncu capture summarised under profiles/) of the FP64 plan the autotuner picked."""
    name = PROFILED_PLANS.get((plan["form"], "fp64"))
    p = REPO / "profiles" / name if name else None
    if p is None or not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("fp64_ops_per_cell_substage:"):
            return float(ln.split(":")[1])
    return None


def profiled_fp64_inst(plan: dict):
    """FP64 instructions per storage cell and sub-stage (DFMA + DADD + DMUL executed, each
    one issue slot of the FP64 pipe) from the same ncu summary as profiled_fp64_ops."""
    name = PROFILED_PLANS.get((plan["form"], "fp64"))
    p = REPO / "profiles" / name if name else None
    if p is None or not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("fp64_inst_per_cell_substage:"):
            return float(ln.split(":")[1])
    return None


def reinit_roofline(sim, torch, stream, n_cells: int, esz: int, iters: int, peaks: dict) -> dict:
    """Time the WENO5 reinitialisation stage alone with CUDA events on the sim's stream
    and express its algorithmic bytes per launch against the measured HBM peak.  In the
    FP64 form the sub-stage is bound by the FP64 pipe, not by HBM: there the line's
    roofline is its FP64 operations per second against the FP64 FMA peak measured on
    this device (garm_fp64_peak_selftest), and the HBM figures ride along."""
    launches = 3 * iters
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.stage("reinit")  # warm
    reps = 2
    ev0.record(stream)
    for _ in range(reps):
        sim.stage("reinit")
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_per_launch = ev0.elapsed_time(ev1) / (reps * launches)
    # per launch: read the input plane, write the output plane; 2 of 3 sub-stages also read φ
    bytes_per_launch = (2.0 + 2.0 / 3.0) * n_cells * esz
    achieved = bytes_per_launch / (ms_per_launch * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs")
    src = "measured"
    if not peak:
        peak, src = 6800.0, "fallback"
    plan = sim.reinit_plan()
    name = {"cells": "kReinitCells", "columns": "kReinitColumns", "sweeps": "kWenoSweep x3",
            "tiled": "kReinitColumnsTiled (TMA-staged plane tiles)", "pairs": "kReinitPairs"}[plan["form"]]
    hbm = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "peak_source": src, "unit": "GB/s",
           "frac": round(achieved / peak, 4), "traffic": None, "algorithmic_bytes_per_launch": int(bytes_per_launch)}
    out = {"kernel": f"{name} (WENO5 TVD-RK3 sub-stage)", "plan": plan, **hbm, "ms_per_launch": round(ms_per_launch, 4)}
    ops = profiled_fp64_ops(plan) if esz == 8 else None
    if ops:
        from garm import capi
        fp64_peak = capi.fp64_peak_tflops()
        tflops = ops * n_cells / (ms_per_launch * 1e-3) / 1e12
        out.update({"bound": "fp64", "achieved": round(tflops, 4), "peak": round(fp64_peak, 4),
                    "peak_source": "measured: garm_fp64_peak_selftest (FP64 FMA chains, CUDA events) on this device",
                    "unit": "TFLOP/s", "frac": round(tflops / fp64_peak, 4),
                    "fp64_ops_per_launch": int(ops * n_cells), "fp64_ops_per_cell": ops, "hbm": hbm})
        inst = profiled_fp64_inst(plan)
        if inst:
            # the same peak as FP64 instructions: an FMA chain issues one DFMA per 2 operations
            rate = inst * n_cells / (ms_per_launch * 1e-3) / 1e12
            out["fp64_issue"] = {"inst_per_cell": inst, "achieved": round(rate, 4), "peak": round(fp64_peak / 2, 4),
                                 "unit": "T inst/s", "frac": round(rate / (fp64_peak / 2), 4)}
    return out


# The level-set band φ is gated on: |φ| <= 15·dx, the reference's air extrapolation radius
# (_airExtrapolationRadius, LevelSetLiquid.h:93).  Beyond it the reinitialisation amplifies
# rounding along 3D diagonals, so forms that round differently differ there by more, and
# those cells do not feed back into the band (tests/test_oracle_kat.py, test_gpu_far_field.py).
LEVEL_SET_BAND = 15.0
PHI_BINS = ((0, 3), (3, 10), (10, 15), (15, 20), (20, 30), (30, 1e9))


def phi_profile(d, pr, dx: float) -> dict:
    """L∞ of |Δφ| (in dx) by |φ_ref|/dx bin."""
    import numpy as np
    a = np.abs(pr) / dx
    return {f"[{lo},{hi if hi < 1e9 else 'inf'})": float(np.max(d[(a >= lo) & (a < hi)], initial=0.0)) / dx
            for lo, hi in PHI_BINS}


def field_errors(test, ref, dx: float) -> dict:
    """Per-field L∞ and RMS of simulation `test` against simulation `ref` on the same grid:
    φ and ξ in units of dx (φ also over the level-set band |φ| <= 15 dx, which the gates
    use, over |φ| <= 3 dx, and by |φ| bin), u relative to max|u| over the faces of the
    fluid domain (fraction < 1; solid-ring faces hold the wall condition's sign ties)."""
    import numpy as np
    from garm import capi

    def linf_rms(d):
        return (float(np.max(d)) if d.size else 0.0), (float(np.sqrt(np.mean(d * d))) if d.size else 0.0)

    pr = ref.download(capi.FIELD_LEVEL_SET)
    d = np.abs(test.download(capi.FIELD_LEVEL_SET) - pr)
    band = np.abs(pr) <= 3 * dx
    out = {"phi_linf_band15dx_dx": float(np.max(d[np.abs(pr) <= LEVEL_SET_BAND * dx], initial=0.0)) / dx,
           "phi_linf_band3dx_dx": float(np.max(d[band], initial=0.0)) / dx,
           "phi_linf_by_abs_phi_dx": phi_profile(d, pr, dx)}
    a, b = linf_rms(d)
    out.update({"phi_linf_dx": a / dx, "phi_rms_dx": b / dx})
    # where the largest φ difference sits: storage cell (x, y, z), φ there, distance from the
    # nearest face of the storage grid in cells
    shape = tuple(reversed([int(ref.grid.resolution[q]) for q in range(ref.grid.dim)]))
    at = np.unravel_index(int(np.argmax(d)), shape)[::-1]
    out["phi_linf_at"] = {"cell": [int(q) for q in at], "phi_ref_dx": float(pr[int(np.argmax(d))]) / dx,
                          "cells_from_grid_face": int(min(min(q, s - 1 - q) for q, s in zip(at, reversed(shape))))}
    ur = ref.download(capi.FIELD_VELOCITY)
    scale = max(float(np.max(np.abs(ur))), 1e-300)
    fluid = ref.download(capi.FIELD_FRACTION) < 1
    a, b = linf_rms(np.abs(test.download(capi.FIELD_VELOCITY) - ur)[fluid])
    out.update({"u_linf_rel_fluid_faces": a / scale, "u_rms_rel_fluid_faces": b / scale})
    a, b = linf_rms(np.abs(test.download(capi.FIELD_REF_MAP) - ref.download(capi.FIELD_REF_MAP)))
    out.update({"xi_linf_dx": a / dx, "xi_rms_dx": b / dx})
    return out


def stage_ms(sim, dx: float, steps: int = 3) -> dict:
    """Median device time of each stage of LevelSetLiquid::advance over `steps`
    host-driven steps (CUDA events between the stages; garm_step_stats.ms_stage)."""
    from garm import capi, scenes
    rows = [sim.advance(dt)["ms_stage"] for dt in scenes.frame_time_steps(sim.max_speed, steps, 25, 1.0, dx)]
    return {name: round(statistics.median(r[i] for r in rows), 4) for i, name in enumerate(capi.STAGE_NAMES)}


BATCH_CG_CELLS_PER_BLOCK = 131072  # measured best for the 48-scene batch (65536: 268M, 131072: 277M, 262144: 257M cell-steps/s)


def batch_scenes(count: int, seed: int = 0):
    """`count` independent pool scenes: n drawn uniformly from {64, 96, 128, 160},
    1-3 seed-placed spheres of radius 0.05-0.15 over a pool of depth 0.1-0.4."""
    import numpy as np
    from garm import scenes
    rng = np.random.default_rng(seed)
    sizes = rng.choice([64, 96, 128, 160], size=count)
    return [scenes.random_pool_scene(int(n), seed=1000 + i) for i, n in enumerate(sizes)]


def run_batch(args, torch, world: int, W: int, K: int) -> dict:
    """Mixed-precision steps of a batch of uneven scenes, one stream per scene, each
    batch step one replay of every scene's captured step graph (garm_batch_advance_auto).
    Timed with events on one stream joined to every scene stream on both sides."""
    from garm import capi
    scs = batch_scenes(args.batch_scenes)
    cfg = capi.default_config(precision=capi.PRECISION_MIXED)
    # each scene's pressure solve takes one SM per 131072 interior cells (2-32 SMs here), so the
    # solves of different scenes run side by side instead of each taking the whole GPU
    cfg.cg_cells_per_block = args.batch_cg_cells or BATCH_CG_CELLS_PER_BLOCK
    streams = [torch.cuda.Stream() for _ in range(min(args.batch_streams or len(scs), len(scs)))]
    sims = []
    for i, sc in enumerate(scs):
        st = streams[i % len(streams)]
        sim = capi.Simulation(sc.grid, cfg, stream=st.cuda_stream)
        sim.upload(capi.FIELD_LEVEL_SET, sc.phi.ravel())
        sim.upload(capi.FIELD_VELOCITY, sc.velocity)
        sim.initialize()
        sim.stage("restart")
        sim.set_clock(25, 1.0)
        sims.append(sim)
    cells = sum(sc.interior_cells for sc in scs)
    resident = sum(s.device_bytes() for s in sims)
    capi.batch_advance_auto(sims, W)  # warm-up, captures every scene's step graphs
    l0 = sum(s.launch_count() for s in sims)
    main = torch.cuda.current_stream()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(main)
    for st in streams:
        st.wait_event(e0)
    stats = capi.batch_advance_auto(sims, K)
    for st in streams:
        ev = torch.cuda.Event()
        ev.record(st)
        main.wait_event(ev)
    e1.record(main)
    torch.cuda.synchronize()
    ms = reduce_max(e0.elapsed_time(e1), world)
    launches = sum(s.launch_count() for s in sims) - l0
    per_step = [st["ms_total"] / K for st in stats]
    graphs = all(s.graph_active() for s in sims)
    for s in sims:
        s.close()
    # the same scenes one after another, each alone on the GPU with the single-scene
    # configuration (its pressure solve may take every SM): what batching is measured against
    seq_ms = 0.0
    for sc in scs:
        s1 = capi.Simulation(sc.grid, capi.default_config(precision=capi.PRECISION_MIXED), stream=main.cuda_stream)
        s1.upload(capi.FIELD_LEVEL_SET, sc.phi.ravel())
        s1.upload(capi.FIELD_VELOCITY, sc.velocity)
        s1.initialize()
        s1.stage("restart")
        s1.set_clock(25, 1.0)
        s1.advance_auto(W)
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(main)
        s1.advance_auto(K)
        q1.record(main)
        torch.cuda.synchronize()
        seq_ms += q0.elapsed_time(q1)
        s1.close()
    seq_ms = reduce_max(seq_ms, world)
    import numpy as np
    value = world * cells * K / (ms * 1e-3)
    seq_value = world * cells * K / (seq_ms * 1e-3)
    return {"value": value, "unit": UNIT, "ms_per_batch_step": ms / K, "scenes": len(scs),
            "sequential": {"value": seq_value, "ms_per_round": seq_ms / K,
                           "what": "the same scenes one at a time, each alone with the single-scene configuration"},
            "speedup_vs_sequential": value / seq_value,
            "interior_cells": cells, "sizes": sorted({int(round(sc.interior_cells ** (1 / 3))) for sc in scs}),
            "resident_bytes": resident, "graph_replay": graphs, "gpu_launches": launches,
            "cg_cells_per_block": cfg.cg_cells_per_block, "streams": len(streams),
            "p50_scene_step_ms": float(np.percentile(per_step, 50)), "p99_scene_step_ms": float(np.percentile(per_step, 99)),
            "dtype": "f32 storage+math, f64 dots/residual/refinement/RM test",
            "workload": f"{len(scs)} pool scenes, n uniform in {{64,96,128,160}}, 1-3 spheres, mixed, "
                        f"one stream and one step graph per scene, {K} steps each"}


def run_serve(args, world: int, count: int | None = None) -> dict:
    """The Poisson request stream served with HBM-budget admission and continuous batching."""
    from garm import serving
    reqs = serving.make_requests(count or args.requests, rate=20.0, seed=11)
    out = serving.Server(budget_bytes=150e9).run(reqs)
    res = out.pop("results")
    out.update({"unit": UNIT, "value": world * out["cell_steps_per_s"],
                "workload": f"{len(reqs)} requests, Poisson 20/s, n log-uniform in [48,192], 20-200 steps, "
                            "dam break or drop, mixed, 150 GB budget",
                "restarts": sum(r.restarts for r in res)})
    return out


def run_drop(args, torch, stream, world: int, W: int, K: int) -> dict:
    """The 3D drop into a pool, mixed against FP64: a pool of depth 0.3 and a sphere of
    radius 0.12 at a seeded centre in [0.3,0.7]^2 x [0.6,0.8], every face at u_y = -1.
    Both forms take the same dt sequence (the Simulator's CFL-1 policy on the FP64
    form's velocity) from the same scene, one host-driven step at a time.  The mixed
    form's per-field errors against the FP64 form are taken at steps 1, 10, 50 and K;
    each step is timed with CUDA events, and steps after the first W make the figures."""
    import numpy as np
    from garm import capi, scenes
    n = args.n
    sc = scenes.drop(n, seed=args.seed)
    dx = sc.grid.spacing
    sims = {}
    # mixed_fixed: the mixed form held to the FP64 form's restart schedule
    # (garm_sim_set_restart_override before each step), which separates the drift of the
    # fields from the restart decisions that the two roundings may take differently
    # fp64_ulp: the FP64 form started from a state one or two ulps away (every value scaled by
    # 1 + U(-1e-15, 1e-15)), the algorithm's own spread to read the mixed form's errors against
    forms = [("fp64", capi.PRECISION_FP64), ("mixed", capi.PRECISION_MIXED), ("mixed_fixed", capi.PRECISION_MIXED)]
    if args.spread:
        forms.append(("fp64_ulp", capi.PRECISION_FP64))
    for name, prec in forms:
        s = capi.Simulation(sc.grid, capi.default_config(precision=prec), stream=stream.cuda_stream)
        phi0, u0 = sc.phi.ravel(), sc.velocity
        if name == "fp64_ulp":
            rng = np.random.default_rng(11)
            phi0 = phi0 * (1 + 1e-15 * rng.uniform(-1, 1, phi0.shape))
            u0 = u0 * (1 + 1e-15 * rng.uniform(-1, 1, u0.shape))
        s.upload(capi.FIELD_LEVEL_SET, phi0)
        s.upload(capi.FIELD_VELOCITY, u0)
        s.initialize()
        s.stage("restart")
        sims[name] = s
    marks = {m for m in (1, 10, 50, K) if 1 <= m <= K}
    times = {k: [] for k in sims}
    cg = {k: [] for k in sims}
    launches = {k: 0 for k in sims}
    restarts = {k: 0 for k in sims}
    errors, errors_fixed, errors_ulp = {}, {}, {}
    last_fp64_restart = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    for step, dt in enumerate(scenes.frame_time_steps(sims["fp64"].max_speed, K, 25, 1.0, dx), 1):
        for name, s in sims.items():
            if name == "mixed_fixed":
                s.set_restart_override(capi.RESTART_ALWAYS if last_fp64_restart else capi.RESTART_NEVER)
            l0 = s.launch_count()
            e0.record(stream)
            st = s.advance(dt)
            e1.record(stream)
            torch.cuda.synchronize()
            restarts[name] += st["restarted"]
            if name == "fp64":
                last_fp64_restart = st["restarted"]
            if step > W:
                times[name].append(e0.elapsed_time(e1))
                cg[name].append(st["cg_iterations"])
                launches[name] += s.launch_count() - l0
        if step in marks:
            errors[str(step)] = field_errors(sims["mixed"], sims["fp64"], dx)
            errors_fixed[str(step)] = field_errors(sims["mixed_fixed"], sims["fp64"], dx)
            if "fp64_ulp" in sims:
                errors_ulp[str(step)] = field_errors(sims["fp64_ulp"], sims["fp64"], dx)
    clk = clocks.stop()
    timed = max(K - W, 1)
    legs = {}
    for name in sims:
        total = reduce_max(sum(times[name]), world)
        legs[name] = {"value": world * n ** 3 * len(times[name]) / max(total * 1e-3, 1e-30), "unit": UNIT,
                      "ms_per_step": total / timed, "p50_step_ms": statistics.median(times[name]) if times[name] else None,
                      "p99_step_ms": float(np.percentile(times[name], 99)) if times[name] else None,
                      "cg_iterations_mean": statistics.mean(cg[name]) if cg[name] else None,
                      "restarts": restarts[name], "resident_bytes": sims[name].device_bytes()}
        sims[name].close()
    legs["mixed"]["dtype"] = "f32 storage+math, f64 dots/residual/refinement/RM test"
    return {"value": legs["mixed"]["value"], "ms_per_step": legs["mixed"]["ms_per_step"], "clocks": clk,
            "gpu_launches": launches["mixed"],
            "workload": f"3D drop into a pool {n}^3 (seed {args.seed}), mixed and FP64 on one dt sequence, "
                        f"{K} steps, the first {W} untimed",
            "drop": {"fp64": legs["fp64"], "mixed": legs["mixed"],
                     "mixed_on_fp64_restart_schedule": {"restarts": legs["mixed_fixed"]["restarts"],
                                                        "errors_vs_fp64": errors_fixed},
                     "fp64_one_ulp_away": ({"restarts": legs["fp64_ulp"]["restarts"], "errors_vs_fp64": errors_ulp}
                                           if "fp64_ulp" in legs else None),
                     "speedup_vs_fp64": legs["mixed"]["value"] / legs["fp64"]["value"],
                     "sphere": {"center": [float(c) for c in sc.meta["center"]], "radius": sc.meta["radius"]},
                     "errors_mixed_vs_fp64": errors}}


def run_dam2d(args, torch, stream, world: int, W: int, K: int) -> dict:
    """The 2D dam break {x < 0.4, y < 0.6} on an n^2 MAC grid (the reference's CPU-runnable
    workload), plain FP64 and mixed, K device-resident steps each after W (graph replay, dt
    on the device), timed with CUDA events; beside them the CPU oracle (the reference's FP64
    path, bit-identical to it) on the same K steps with all host threads."""
    from garm import capi, scenes
    n = args.n
    sc = scenes.dam_break(2, n)
    dx = sc.grid.spacing
    legs = {}
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    launches = 0
    for name, prec in (("fp64", capi.PRECISION_FP64), ("mixed", capi.PRECISION_MIXED)):
        s = capi.Simulation(sc.grid, capi.default_config(precision=prec), stream=stream.cuda_stream)
        s.upload(capi.FIELD_LEVEL_SET, sc.phi.ravel())
        s.upload(capi.FIELD_VELOCITY, sc.velocity)
        s.initialize()
        s.stage("restart")
        s.set_clock(25, 1.0)
        s.advance_auto(W)
        barrier(world)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = s.launch_count()
        e0.record(stream)
        st = s.advance_auto(K)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = reduce_max(e0.elapsed_time(e1), world)
        if name == "fp64":
            launches = s.launch_count() - l0
        legs[name] = {"value": world * n * n * K / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / K,
                      "cg_iterations_last_step": st["cg_iterations"], "graph_replay": s.graph_active()}
        s.close()
    clk = clocks.stop()
    legs["mixed"]["speedup_vs_fp64"] = legs["mixed"]["value"] / legs["fp64"]["value"]
    out = {"value": legs["fp64"]["value"], "ms_per_step": legs["fp64"]["ms_per_step"], "clocks": clk,
           "gpu_launches": launches, "mixed": legs["mixed"],
           "workload": f"2D dam break {n}^2 MAC grid, plain FP64 form, {K} steps after {W}"}
    if int(os.environ.get("RANK", 0)) == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        sys.path.insert(0, str(REPO / "tests"))
        from helpers import host_default_config, load_scene
        o = O.OracleSim(sc.grid, host_default_config())
        load_scene(o, sc)
        o.initialize()
        o.stage("restart")
        gen = scenes.frame_time_steps(o.max_speed, W + K, 25, 1.0, dx)
        for _ in range(W):
            o.advance(next(gen))
        t0 = time.perf_counter()
        for _ in range(K):
            o.advance(next(gen))
        secs = time.perf_counter() - t0
        o.close()
        out["cpu_baseline"] = {"value": n * n * K / secs, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                               "sample": f"{K} oracle steps of the {n}^2 dam break after {W} ({secs:.2f} s)",
                               "build": O.BUILD_FLAGS}
    return out


def run_garm(args) -> None:
    import numpy as np
    import torch
    from garm import capi, scenes

    rank, local, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    capi.load()
    n, K, W = args.n, args.steps, args.warmup
    if args.workload == "drop":
        sub = run_drop(args, torch, stream, world, W, K)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": sub["value"], "unit": UNIT, "n_gpus": world, "steps": K,
                              "warmup": W, "ms_per_step": sub["ms_per_step"], "higher_is_better": True,
                              "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                              "config": {"workload": sub["workload"], "n": n, "replicas": world,
                                         "l2": "no flush: device state larger than L2"},
                              "clocks": sub["clocks"], "gpu_launches": sub["gpu_launches"], "drop": sub["drop"]}),
                  flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload == "dam2d":
        sub = run_dam2d(args, torch, stream, world, W, K)
        if rank == 0:
            line = {"metric": METRIC, "value": sub["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                    "ms_per_step": sub["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "f64", "data": "synthetic",
                    "config": {"workload": sub["workload"], "n": n, "dim": 2, "cfl": 1.0, "frame_rate": 25,
                               "reinit": "WENO5 x30 every step", "pcg_tol": 1e-08, "replicas": world,
                               "l2": "no flush: the 2D state fits in L2; each step re-reads it"},
                    "clocks": sub["clocks"], "gpu_launches": sub["gpu_launches"], "mixed": sub["mixed"]}
            if "cpu_baseline" in sub:
                line["cpu_baseline"] = sub["cpu_baseline"]
            print(json.dumps(line), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload in ("batch", "serve"):
        clocks = Clocks(local)
        clocks.start()
        sub = run_batch(args, torch, world, W, K) if args.workload == "batch" else run_serve(args, world)
        clk = clocks.stop()
        if rank == 0:
            line = {"metric": METRIC, "value": sub.pop("value"), "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                    "data": "synthetic", "config": {"workload": sub.pop("workload"), "replicas": world,
                                                    "l2": "no flush: device state larger than L2"},
                    "clocks": clk}
            if "ms_per_batch_step" in sub:
                line["ms_per_step"] = sub["ms_per_batch_step"]
                line["gpu_launches"] = sub["gpu_launches"]
            line[args.workload] = sub
            print(json.dumps(line), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    scene = scenes.dam_break(3, n)
    dx = scene.grid.spacing
    interior = n ** 3
    if args.workload == "reinit" and not args.reinit_plan:
        args.reinit_plan = "sweeps,32,44" if args.precision == "fp64" else "columns,128,8"
    if args.reinit_plan:
        form, threads, cells = args.reinit_plan.split(",")
        for prec in (capi.PRECISION_FP64, capi.PRECISION_MIXED):
            capi.reinit_plan_set([scene.grid.resolution[a] for a in range(3)], prec, form, int(threads), int(cells))

    def make(precision, **flags):
        cfg = capi.default_config(precision=precision)
        for k, v in flags.items():
            setattr(cfg, k, v)
        sim = capi.Simulation(scene.grid, cfg, stream=stream.cuda_stream)
        sim.upload(capi.FIELD_LEVEL_SET, scene.phi.ravel())
        sim.upload(capi.FIELD_VELOCITY, scene.velocity)
        sim.initialize()
        sim.stage("restart")
        return sim

    main_prec = capi.PRECISION_MIXED if args.precision == "mixed" else capi.PRECISION_FP64
    sim = make(main_prec)
    if args.workload == "reinit":
        # the reinitialisation stage alone on the scene's level set, with a pinned plan, so that
        # an ncu capture sees only the sub-stage kernels after the scene's set-up
        for _ in range(W):
            sim.stage("reinit")
        torch.cuda.synchronize()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = sim.launch_count()
        r0.record(stream)
        for _ in range(K):
            sim.stage("reinit")
        r1.record(stream)
        torch.cuda.synchronize()
        ms = r0.elapsed_time(r1)
        if rank == 0:
            print(json.dumps({"metric": "reinitialisation stages/s", "value": K / (ms * 1e-3), "unit": "stages/s", "n_gpus": world,
                              "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic",
                              "config": {"workload": f"WENO5 x30 reinitialisation of the {n}^3 dam break, plan {args.reinit_plan}",
                                         "n": n}, "gpu_launches": sim.launch_count() - l0, "plan": sim.reinit_plan()}), flush=True)
        sim.close()
        return
    sim.set_clock(25, 1.0)  # Simulator dt policy on the device: CFL 1, 25 frames/s
    sim.advance_auto(W)     # warm-up (also captures the step graphs)
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    l0 = sim.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.advance_auto(K)     # K steps, dt from max|u| on the device, one synchronisation
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = sim.launch_count() - l0
    elapsed_ms = reduce_max(ev0.elapsed_time(ev1), world)
    # per-step latency: the same loop one step per call (each call synchronises)
    step_ms, cg_it, restarts = [], [], 0
    for _ in range(K):
        st = sim.advance_auto(1)
        step_ms.append(st["ms_total"])
        cg_it.append(st["cg_iterations"])
        restarts += st["restarted"]
    stages = stage_ms(sim, dx)
    barrier(world)
    value = replica_value(world, interior, K, elapsed_ms)
    peaks = measured_peaks()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": elapsed_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": dam_config(n, args.precision, world),
        "p50_step_ms": statistics.median(step_ms), "p99_step_ms": float(np.percentile(step_ms, 99)),
        "cg_iterations_mean": statistics.mean(cg_it), "restarts": restarts, "graph_replay": sim.graph_active(),
        "stage_ms": stages,
        "clocks": clk, "gpu_launches": launches,
    }
    if rank == 0:
        out["roofline"] = reinit_roofline(sim, torch, stream, int(scene.phi.size), 8 if args.precision == "fp64" else 4, 30, peaks)
        out["roofline"]["traffic"] = profiled_traffic(out["roofline"]["plan"], args.precision, n)
        if "hbm" in out["roofline"]:
            out["roofline"]["hbm"]["traffic"] = out["roofline"]["traffic"]
        out["roofline"]["compute"] = profiled_pipe(out["roofline"]["plan"], args.precision, n)

    # end to end through the C ABI with host buffers: upload the step's input state
    # from pinned memory, advance, download the state and the level set
    if not args.no_e2e:
        fields = state_fields()
        pinned_in = {f: torch.from_numpy(sim.download(f)).pin_memory().numpy() for f in fields}
        pinned_out = {f: torch.from_numpy(sim.download(f)).pin_memory().numpy() for f in fields + [capi.FIELD_LEVEL_SET]}
        h2d = sum(a.nbytes for a in pinned_in.values())
        d2h = sum(a.nbytes for a in pinned_out.values())
        barrier(world)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(K):
            for f in fields:
                sim.upload(f, pinned_in[f])
            sim.advance(next(scenes.frame_time_steps(sim.max_speed, 1, 25, 1.0, dx)))
            for f, buf in pinned_out.items():
                sim.download(f, buf)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        e2e_ms = reduce_max(e0.elapsed_time(e1), world)
        out["e2e"] = {"value": world * interior * K / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms / K, "host_wall_ms_per_step": 1e3 * wall / K,
                      "api": "garm_sim_upload x6 (.sav state) + garm_sim_advance + garm_sim_download x7"}

    # mixed precision on the same workload: throughput and φ error against the FP64 form
    if not args.no_mixed and args.precision == "fp64":
        ref = make(capi.PRECISION_FP64)
        mix = make(capi.PRECISION_MIXED)
        dt0 = next(scenes.frame_time_steps(ref.max_speed, 1, 25, 1.0, dx))
        ref.advance(dt0)
        mix.advance(dt0)
        pr, pm = ref.download(capi.FIELD_LEVEL_SET), mix.download(capi.FIELD_LEVEL_SET)
        dphi = np.abs(pr - pm)
        phi_err = float(np.max(dphi)) / dx
        phi_err_band = float(np.max(dphi[np.abs(pr) <= 3 * dx])) / dx
        phi_err_band15 = float(np.max(dphi[np.abs(pr) <= LEVEL_SET_BAND * dx])) / dx
        phi_prof = phi_profile(dphi, pr, dx)
        ref.close()
        mix.set_clock(25, 1.0)
        mix.advance_auto(W)
        barrier(world)
        torch.cuda.synchronize()
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0.record(stream)
        mix.advance_auto(K)
        m1.record(stream)
        torch.cuda.synchronize()
        mix_ms = reduce_max(m0.elapsed_time(m1), world)
        mms, mcg = [], []
        for _ in range(K):
            st = mix.advance_auto(1)
            mms.append(st["ms_total"])
            mcg.append(st["cg_iterations"])
        mval = world * interior * K / (mix_ms * 1e-3)
        mstages = stage_ms(mix, dx)
        out["mixed"] = {"value": mval, "unit": UNIT, "ms_per_step": mix_ms / K, "p50_step_ms": statistics.median(mms),
                        "p99_step_ms": float(np.percentile(mms, 99)),
                        "phi_gate": {"metric": "φ L∞ after 1 step vs the FP64 form over |φ_fp64| <= 15·dx", "limit_dx": 1e-3,
                                     "value_dx": phi_err_band15, "pass": bool(phi_err_band15 <= 1e-3)},
                        "phi_err_dx_band15dx_after_1_step_vs_fp64": phi_err_band15,
                        "phi_err_dx_band3dx_after_1_step_vs_fp64": phi_err_band, "phi_err_dx_all_cells_after_1_step_vs_fp64": phi_err,
                        "phi_err_dx_by_abs_phi_after_1_step_vs_fp64": phi_prof,
                        "speedup_vs_fp64": mval / value, "cg_iterations_mean": statistics.mean(mcg), "stage_ms": mstages,
                        "dtype": "f32 storage+math, f64 dots/residual/refinement/RM test"}
        if rank == 0:
            out["mixed"]["roofline"] = reinit_roofline(mix, torch, stream, int(scene.phi.size), 4, 30, peaks)
            out["mixed"]["roofline"]["traffic"] = profiled_traffic(out["mixed"]["roofline"]["plan"], "mixed", n)
            out["mixed"]["roofline"]["compute"] = profiled_pipe(out["mixed"]["roofline"]["plan"], "mixed", n)
        mix.close()

    # the same workload in the reference's default build: HybridNewton restart and fast
    # marching in place of WENO5 (restart_newton = fast_marching = 1)
    if not args.no_default_build and args.precision == "fp64":
        legs = {}
        for name, prec in (("fp64", capi.PRECISION_FP64), ("mixed", capi.PRECISION_MIXED)):
            d = make(prec, restart_newton=1, fast_marching=1)
            d.set_clock(25, 1.0)
            d.advance_auto(W)
            barrier(world)
            torch.cuda.synchronize()
            d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            d0.record(stream)
            st = d.advance_auto(K)
            d1.record(stream)
            torch.cuda.synchronize()
            dms = reduce_max(d0.elapsed_time(d1), world)
            legs[name] = {"value": world * interior * K / (dms * 1e-3), "unit": UNIT, "ms_per_step": dms / K,
                          "restarted_last_step": st["restarted"]}
            d.close()
        out["default_build"] = {"config": "restart_newton=1, fast_marching=1 (the reference's default xmake options)", **legs}

    # many uneven scenes at once (mixed): the batched form of the same pipeline
    if not args.no_batch:
        out["batch"] = run_batch(args, torch, world, W, K)
        out["batch"]["speedup_vs_fp64"] = out["batch"]["value"] / value if args.precision == "fp64" else None

    # the Poisson request stream (a short one) with HBM-budget admission, so that the line
    # carries serving throughput and p50/p99 step and end-to-end latency
    if not args.no_serve:
        out["serve"] = run_serve(args, world, args.serve_requests)

    # CPU baseline: the oracle (a CPU port of the reference's FP64 path) on this host,
    # one step of the same 128^3 workload started from the GPU's state.  The GPU then
    # takes the same step from the same state, and the two are compared field by field.
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        o = O.OracleSim(scene.grid, sim.cfg)
        for f in state_fields() + [capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET, capi.FIELD_TMP_LEVEL_SET, capi.FIELD_FRACTION]:
            o.upload(f, sim.download(f))
        dt = next(scenes.frame_time_steps(o.max_speed, 1, 25, 1.0, dx))
        t0 = time.perf_counter()
        o.advance(dt)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": interior / secs, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                               "sample": f"1 oracle advance of the {n}^3 dam break from the GPU state ({secs:.1f} s)",
                               "build": O.BUILD_FLAGS,
                               "solver": "Jacobi-PCG to |r| <= 1e-8 |b| (the workload's tolerance; the reference's "
                                         "Eigen IC-PCG stops at 1e-5)"}
        sim.advance(dt)
        out["parity_vs_oracle_1_step"] = {"form": args.precision, "from": f"the GPU state after {2 * K + W + 3} steps",
                                          **field_errors(sim, o, dx)}
        # the reference's own thread policy, omp_set_num_threads(nprocs / 3) (Source/Demo/Demo.cpp:27)
        all_threads = O.max_threads()
        third = max(1, (os.cpu_count() or 3) // 3)
        O.set_threads(third)
        dt = next(scenes.frame_time_steps(o.max_speed, 1, 25, 1.0, dx))
        t0 = time.perf_counter()
        o.advance(dt)
        secs3 = time.perf_counter() - t0
        O.set_threads(all_threads)
        out["cpu_baseline"]["nprocs_div_3"] = {"value": interior / secs3, "threads": third,
                                               "sample": f"the next oracle step at nprocs/3 threads ({secs3:.1f} s)"}
        o.close()
        # the gate as the path states it: initialize, restart and one step of the scene
        g0 = make(main_prec)
        o0 = O.OracleSim(scene.grid, g0.cfg)
        o0.upload(capi.FIELD_LEVEL_SET, scene.phi.ravel())
        o0.upload(capi.FIELD_VELOCITY, scene.velocity)
        o0.initialize()
        o0.stage("restart")
        dt0 = next(scenes.frame_time_steps(o0.max_speed, 1, 25, 1.0, dx))
        o0.advance(dt0)
        g0.advance(dt0)
        out["parity_vs_oracle_first_step"] = {"form": args.precision, "from": "the scene (initialize, restart, one step)",
                                              **field_errors(g0, o0, dx)}
        o0.close()
        g0.close()
    sim.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args) -> None:
    """The reference's FP64 CPU path on the same workload, all host threads: the oracle port,
    which gives the same bits as the reference's own code compiled from its sources
    (tests/test_ref_pin.py); those sources are not on the GPU machine, the port is."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    from garm import scenes
    from garm.build import build_oracle
    build_oracle()
    from oracle import oracle as O
    sys.path.insert(0, str(REPO / "tests"))
    from helpers import host_default_config, load_scene

    n, K, W = args.n, args.steps, args.warmup
    scene = scenes.dam_break(3, n)
    dx = scene.grid.spacing
    o = O.OracleSim(scene.grid, host_default_config())
    load_scene(o, scene)
    o.initialize()
    o.stage("restart")
    gen = scenes.frame_time_steps(o.max_speed, min(W, 1) + K, 25, 1.0, dx)
    for _ in range(min(W, 1)):
        o.advance(next(gen))
    times = []
    for _ in range(K):
        t0 = time.perf_counter()
        o.advance(next(gen))
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n ** 3 * K / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": dam_config(n, "fp64", world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                         "sample": f"{K} full oracle steps of the {n}^3 dam break; warm-up capped at 1 step; "
                                   "the oracle equals the reference's own code bit for bit (2D 128^2, 200 steps)",
                         "build": O.BUILD_FLAGS},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_garm(args)


if __name__ == "__main__":
    main()
