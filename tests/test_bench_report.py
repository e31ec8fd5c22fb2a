"""The benchmark's parity report (bench.field_errors), checked on the CPU with two oracle
simulations: zero for identical states, and a planted difference in φ, u and ξ found with
its size and its cell."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

from garm import capi, scenes
from helpers import host_default_config, load_scene

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


def _pair(oracle_mod):
    sc = scenes.dam_break(3, 12)
    sims = []
    for _ in range(2):
        o = oracle_mod.OracleSim(sc.grid, host_default_config())
        load_scene(o, sc)
        o.initialize()
        sims.append(o)
    return sc, sims


def test_identical_states_report_zero(oracle_mod):
    sc, (a, b) = _pair(oracle_mod)
    e = bench.field_errors(a, b, sc.grid.spacing)
    for k in ("phi_linf_band3dx_dx", "phi_linf_dx", "phi_rms_dx", "u_linf_rel_fluid_faces", "xi_linf_dx"):
        assert e[k] == 0.0, k


def test_planted_differences_are_found(oracle_mod):
    sc, (a, b) = _pair(oracle_mod)
    dx = sc.grid.spacing
    n = [int(sc.grid.resolution[q]) for q in range(3)]
    phi = b.download(capi.FIELD_LEVEL_SET)
    cell = (5, 7, 6)                                  # (x, y, z) of the planted change
    flat = cell[0] + n[0] * (cell[1] + n[1] * cell[2])
    phi[flat] += 0.25 * dx
    b.upload(capi.FIELD_LEVEL_SET, phi)
    xi = b.download(capi.FIELD_REF_MAP)
    xi[3] += 0.5 * dx
    b.upload(capi.FIELD_REF_MAP, xi)
    e = bench.field_errors(a, b, dx)
    assert np.isclose(e["phi_linf_dx"], 0.25, rtol=1e-9)
    assert e["phi_linf_at"]["cell"] == list(cell)
    assert e["phi_linf_at"]["cells_from_grid_face"] == min(min(c, m - 1 - c) for c, m in zip(cell, n))
    assert np.isclose(e["phi_rms_dx"], 0.25 / np.sqrt(phi.size), rtol=1e-9)
    assert np.isclose(e["xi_linf_dx"], 0.5, rtol=1e-9)
    assert e["u_linf_rel_fluid_faces"] == 0.0


def test_profiles_named_by_the_bench_parse():
    """Every ncu summary the bench reads for its roofline (bench.PROFILED_PLANS) yields the
    compute fraction and the DRAM traffic per launch, and the FP64 one its operation count."""
    for (form, precision) in bench.PROFILED_PLANS:
        plan = {"form": form}
        pipe = bench.profiled_pipe(plan, precision, 128)
        assert pipe is not None and 0 < pipe["frac"] <= 1, (form, precision)
        traffic = bench.profiled_traffic(plan, precision, 128)
        assert traffic is not None and traffic > 0, (form, precision)
    ops = bench.profiled_fp64_ops({"form": "sweeps"})
    assert ops is not None and 100 < ops < 1000
    inst = bench.profiled_fp64_inst({"form": "sweeps"})
    assert inst is not None and ops / 2 < inst < ops  # an FMA is one instruction, two operations
