"""Writes the golden vectors of tests/golden/ from the reference binary.

The reference binary is the reference's own LevelSetLiquid<Dim> (oracle/_ref, built
from the reference's Source/Core by oracle/build_ref.sh); it cannot travel to a GPU
machine, so the GPU tests (tests/test_gpu_golden.py) compare the kernels with the
vectors it wrote here.  Scenes come from garm.scenes with fixed sizes and seeds; the
files record a checksum of the initial level set so a changed scene generator is
caught.  For the 2D dam break the file also holds the reference's own spread under
ulp-sized changes of its initial state (the largest difference over two perturbed
runs), the yardstick for drift over 200 steps.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

from garm import capi, scenes  # noqa: E402
from helpers import host_default_config, perturbed  # noqa: E402
from oracle import oracle as O  # noqa: E402

F = {"phi": capi.FIELD_LEVEL_SET, "u": capi.FIELD_VELOCITY, "xi": capi.FIELD_REF_MAP, "adv": capi.FIELD_ADV_REGION}


def run(sc, steps, keep, size=0.0, seed=0, dts=None):
    """Reference run: initialize, restart, `steps` steps (dt from the Simulator's CFL-1 policy
    on the reference's own velocity unless `dts` is given).  Returns the dts, per-step records
    and the requested fields after the requested steps."""
    r = O.RefSim(sc.grid, host_default_config())
    r.upload(capi.FIELD_LEVEL_SET, perturbed(sc.phi.ravel(), size, seed) if size else sc.phi.ravel())
    r.upload(capi.FIELD_VELOCITY, perturbed(sc.velocity, size, seed + 1) if size else sc.velocity)
    assert r.initialize() == capi.OK
    r.stage("restart")
    gen = iter(dts) if dts is not None else scenes.frame_time_steps(r.max_speed, steps, 25, 1.0, sc.grid.spacing)
    out, used, rec = {}, [], []
    for k in range(1, steps + 1):
        dt = next(gen)
        st = r.advance(dt)
        assert st["status"] == capi.OK
        used.append(dt)
        rec.append((st["restarted"], st["unknowns"], st["volume"]))
        for name, at in keep.items():
            if k in at:
                out[f"{name}_{k}"] = r.download(F[name])
    r.close()
    return np.array(used), np.array(rec, dtype=np.float64), out


def write(name, sc, steps, keep, spread_runs=0):
    dts, rec, out = run(sc, steps, keep)
    extra = {}
    for q in range(spread_runs):
        _, _, o2 = run(sc, steps, keep, size=(1e-15, 2e-15)[q], seed=11 + q, dts=dts)
        for k, v in o2.items():
            extra[f"spread_{k}"] = np.maximum(extra.get(f"spread_{k}", 0), np.abs(v.astype(np.float64) - out[k].astype(np.float64)))
    np.savez_compressed(HERE / f"{name}.npz", dts=dts, restarted=rec[:, 0].astype(np.int8), unknowns=rec[:, 1].astype(np.int32),
                        volume=rec[:, 2], phi0_sum=np.float64(np.sum(sc.phi)), **out, **extra)
    print(f"{name}: {steps} steps, {int(rec[:, 0].sum())} restarts, {(HERE / f'{name}.npz').stat().st_size // 1024} KB")


def main():
    write("dam3d_12", scenes.dam_break(3, 12), 3, {"phi": (1, 3), "u": (1, 3), "xi": (1, 3), "adv": (3,)})
    write("drop3d_12_seed3", scenes.drop(12, seed=3), 2, {"phi": (1, 2), "u": (2,), "xi": (2,)})
    write("dam2d_128_200", scenes.dam_break(2, 128), 200, {"phi": (1, 10, 50, 200), "u": (200,), "xi": (200,)}, spread_runs=2)


if __name__ == "__main__":
    main()
