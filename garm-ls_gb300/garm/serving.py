"""Serving loop: simulation requests admitted by an HBM budget, state resident
on the device, continuous batching.

Each request is one scene (a dam break or a drop) of n^3 cells that must be
advanced `steps` times.  Requests arrive as a Poisson stream.  The server admits
a request as soon as it has arrived and its device footprint
(garm_sim_estimate_bytes) fits in the remaining budget; every admitted scene owns
a stream, and each round the server enqueues the next chunk of steps of every
idle scene (garm_sim_enqueue_auto), so work of different requests overlaps on
the GPU; finished requests free their memory and make room for queued ones.

Per-step latency is the device time of each enqueued chunk divided by its
steps (events on the scene's stream, so it includes contention from the other
scenes); end-to-end latency is completion minus arrival on the host clock.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import capi, scenes


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    n: int                  # interior cells per axis
    steps: int
    kind: str               # "dam" | "drop"
    seed: int


@dataclass
class Result:
    rid: int
    n: int
    steps: int
    arrival: float
    admitted: float
    completed: float
    step_ms: list = field(default_factory=list)
    restarts: int = 0
    phi: np.ndarray | None = None

    @property
    def e2e(self) -> float:
        return self.completed - self.arrival


def make_requests(count: int, rate: float = 20.0, seed: int = 0, n_range=(48, 192), steps_range=(20, 200)) -> list[Request]:
    """Poisson arrivals at `rate`/s; n log-uniform in n_range; steps uniform in steps_range;
    dam break or drop chosen at random; every draw from one seeded generator."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        n = int(round(math.exp(rng.uniform(lo, hi))))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        kind = "dam" if rng.random() < 0.5 else "drop"
        out.append(Request(rid, t, n, steps, kind, int(rng.integers(0, 2**31 - 1))))
    return out


def build_scene(req: Request) -> scenes.Scene:
    if req.kind == "dam":
        rng = np.random.default_rng(req.seed)
        ext = (rng.uniform(0.3, 0.5), rng.uniform(0.4, 0.6), rng.uniform(0.4, 0.7))
        return scenes.dam_break(3, req.n, ext)
    return scenes.drop(req.n, seed=req.seed)


class Server:
    def __init__(self, budget_bytes: float = 150e9, precision: int = capi.PRECISION_MIXED, frame_rate: int = 25,
                 cfl: float = 1.0, chunk: int = 1, keep_phi: bool = False, cg_cells_per_block: int = 65536):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.frame_rate = frame_rate
        self.cfl = cfl
        self.chunk = chunk
        self.keep_phi = keep_phi
        # one SM per 65536 interior cells for each pressure solve: resident scenes' solves run
        # side by side instead of each taking the whole GPU (measured on the default stream:
        # 262144 cells per block 133M, 131072 189M, 65536 206M cell-steps/s)
        self.cfg = capi.default_config(precision=precision, cg_cells_per_block=cg_cells_per_block)

    def _admit(self, req: Request, t0: float):
        sc = build_scene(req)
        sim = capi.Simulation(sc.grid, self.cfg)  # own stream
        sim.upload(capi.FIELD_LEVEL_SET, sc.phi.ravel())
        sim.upload(capi.FIELD_VELOCITY, sc.velocity)
        sim.initialize()
        sim.stage("restart")
        sim.set_clock(self.frame_rate, self.cfl)
        res = Result(req.rid, req.n, req.steps, req.arrival, time.perf_counter() - t0, 0.0)
        return {"req": req, "sim": sim, "res": res, "done": 0, "busy": False, "cells": sc.interior_cells}

    def run(self, requests: list[Request], time_scale: float = 1.0) -> dict:
        """Serve `requests` (arrival times scaled by time_scale) and return statistics."""
        pending = sorted(requests, key=lambda r: r.arrival)
        sizes = {r.rid: capi.estimate_bytes(scenes.unit_grid(3, r.n), self.cfg) for r in pending}
        for r in pending:
            if sizes[r.rid] > self.budget:
                raise ValueError(f"request {r.rid} ({r.n}^3) does not fit the budget on its own")
        active, results = [], []
        used = 0.0
        peak_used, peak_active = 0.0, 0
        cell_steps = 0
        t0 = time.perf_counter()
        while pending or active:
            now = time.perf_counter() - t0
            # admission: arrived requests, in order, while the budget allows
            while pending and pending[0].arrival * time_scale <= now and used + sizes[pending[0].rid] <= self.budget:
                req = pending.pop(0)
                used += sizes[req.rid]
                active.append(self._admit(req, t0))
            peak_used = max(peak_used, used)
            peak_active = max(peak_active, len(active))
            # continuous batching: every idle scene gets its next chunk
            for a in active:
                if not a["busy"]:
                    k = min(self.chunk, a["req"].steps - a["done"])
                    a["sim"].enqueue_auto(k)
                    a["busy"], a["k"] = True, k
            progressed = False
            for a in list(active):
                if a["busy"] and a["sim"].poll():
                    st = a["sim"].collect()
                    a["busy"] = False
                    a["done"] += a["k"]
                    a["res"].step_ms.extend([st["ms_total"] / a["k"]] * a["k"])
                    a["res"].restarts += st["restarted"]
                    cell_steps += a["cells"] * a["k"]
                    progressed = True
                    if a["done"] >= a["req"].steps:
                        a["res"].completed = time.perf_counter() - t0
                        if self.keep_phi:
                            a["res"].phi = a["sim"].download(capi.FIELD_LEVEL_SET)
                        a["sim"].close()
                        used -= sizes[a["req"].rid]
                        active.remove(a)
                        results.append(a["res"])
            if not progressed:
                time.sleep(0.0002)
        wall = time.perf_counter() - t0
        step_ms = np.concatenate([np.asarray(r.step_ms) for r in results]) if results else np.zeros(1)
        e2e = np.asarray([r.e2e for r in results])
        return {
            "requests": len(results), "wall_s": wall, "cell_steps": cell_steps, "cell_steps_per_s": cell_steps / wall,
            "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "p50_e2e_s": float(np.percentile(e2e, 50)), "p99_e2e_s": float(np.percentile(e2e, 99)),
            "peak_resident_bytes": peak_used, "peak_active": peak_active, "budget_bytes": self.budget,
            "results": results,
        }
