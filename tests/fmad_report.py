"""FMA contraction as a diagnostic of the FP64 form's parity with the oracle.

    python tests/fmad_report.py

Builds the library a second time with nvcc -fmad=false (separate products and sums are no
longer contracted into FMAs; the kernels' explicit fma() calls stay fused) into
garm-ls_gb300/_build_nofmad/ and libgarm_nofmad.so.  Then, with each library, it runs the
per-stage comparison of tests/test_gpu_parity.py (every stage from the same oracle state
after three steps) and the one-step gate (initialize, restart, one advance), on the 2D dam
break, the 3D dam break and the 3D drop.  It prints one JSON line: per scene and library, the
largest relative difference of each stage's fields from the oracle and the one-step φ L∞ in
units of dx.  A report, not a pytest test: it needs a GPU and builds a second library.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

from garm import build, capi, scenes  # noqa: E402
from helpers import STATE_FIELDS, copy_state, host_default_config, linf, load_scene, rel  # noqa: E402
from oracle import oracle as O  # noqa: E402

SCENES = {
    "dam2d": lambda: scenes.dam_break(2, 40),
    "dam3d": lambda: scenes.dam_break(3, 20),
    "drop3d": lambda: scenes.drop(20, seed=3),
}
STAGES = {
    "advect": (True, [capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD, capi.FIELD_VELOCITY]),
    "compose": (False, [capi.FIELD_LEVEL_SET, capi.FIELD_TMP_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET]),
    "reinit": (False, [capi.FIELD_LEVEL_SET]),
    "extrap_collider": (False, [capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET]),
    "restart": (False, [capi.FIELD_REF_LEVEL_SET, capi.FIELD_REF_LEVEL_SET_GRAD, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD]),
    "extrap_air": (False, [capi.FIELD_REF_MAP, capi.FIELD_VELOCITY]),
    "enforce_bc": (False, [capi.FIELD_VELOCITY]),
}


def stage_errors(sc) -> dict:
    cfg = host_default_config()
    o = O.OracleSim(sc.grid, cfg)
    load_scene(o, sc)
    o.initialize()
    o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, 3, 25, 1.0, sc.grid.spacing):
        o.advance(dt)
    g = capi.Simulation(sc.grid, cfg)
    load_scene(g, sc)
    g.initialize()
    dt = 0.5 * sc.grid.spacing / max(o.max_speed(), 1e-3)
    snapshot = {f: o.download(f) for f in STATE_FIELDS}
    out = {}
    for stage, (takes_dt, fields) in STAGES.items():
        for f, v in snapshot.items():
            o.upload(f, v)
        copy_state(g, o)
        g.stage(stage, *([dt] if takes_dt else []))
        o.stage(stage, dt if takes_dt else 0.0)
        out[stage] = float(max(rel(g.download(f), o.download(f)) for f in fields))
    g.close()
    return out


def one_step(sc) -> float:
    cfg = host_default_config()
    g, o = capi.Simulation(sc.grid, cfg), O.OracleSim(sc.grid, cfg)
    for s in (g, o):
        load_scene(s, sc)
        s.initialize()
        s.stage("restart")
    dt = next(scenes.frame_time_steps(o.max_speed, 1, 25, 1.0, sc.grid.spacing))
    g.advance(dt)
    o.advance(dt)
    err = linf(g.download(capi.FIELD_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET)) / sc.grid.spacing
    g.close()
    return float(err)


def main() -> None:
    libs = {"default": build.build_library(),
            "fmad_false": build.build_library(extra_flags=("-fmad=false",), tag="nofmad")}
    report = {}
    for name, make in SCENES.items():
        report[name] = {}
        for label, path in libs.items():
            capi._LIB = capi.load(path)
            sc = make()
            row = stage_errors(sc)
            row["one_step_phi_dx"] = one_step(sc)
            report[name][label] = {k: float(np.format_float_scientific(v, 2)) for k, v in row.items()}
    print(json.dumps(report))


if __name__ == "__main__":
    main()
