"""The C ABI library loads and exports every entry point declared in include/garm.h,
and its struct layouts and defaults agree with the host-side restatements
(no GPU call is made)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from garm import capi
from helpers import host_default_config

REPO = Path(__file__).resolve().parents[1]
HEADER = REPO / "include" / "garm.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(garm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(garm_lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(garm_lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(names) <= set(capi._SIGS), set(names) - set(capi._SIGS)


def test_nm_lists_symbols_as_extern_c(garm_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (garm_\w+)", out))
    assert set(declared_functions()) <= exported


def test_struct_layout_matches_header(tmp_path):
    probe = tmp_path / "probe.c"
    probe.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "garm.h"\n'
                     'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(garm_grid_desc), sizeof(garm_config),'
                     ' sizeof(garm_step_stats), offsetof(garm_config, fast_marching), offsetof(garm_step_stats, volume));return 0;}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(REPO / "include"), str(probe), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals == [C.sizeof(capi.GridDesc), C.sizeof(capi.Config), C.sizeof(capi.StepStats),
                    capi.Config.fast_marching.offset, capi.StepStats.volume.offset]


def test_config_defaults_equal_reference_constants(garm_lib):
    lib_cfg = capi.default_config()
    host = host_default_config()
    for name, _ in capi.Config._fields_:
        assert getattr(lib_cfg, name) == getattr(host, name), name
    assert lib_cfg.rm_threshold == 0.883022221559489  # LevelSetLiquid.cpp:631
    assert lib_cfg.reinit_iters == 30 and lib_cfg.reinit_cfl == 0.9  # LevelSetLiquid.cpp:1156
    assert lib_cfg.cg_max_iters == 2000  # Projector.cpp:161


def test_status_strings_and_abi_version(garm_lib):
    assert garm_lib.garm_abi_version() == 5
    assert garm_lib.garm_status_string(capi.NOT_CONVERGED) == b"pressure solve did not converge"


def test_null_arguments_are_rejected_without_a_gpu(garm_lib):
    # argument validation happens before any CUDA call
    assert garm_lib.garm_sim_create(None, None, None, None) == capi.INVALID
    assert garm_lib.garm_sim_advance(None, 0.01, None) == capi.INVALID
    assert garm_lib.garm_sim_upload(None, 0, None, 0) == capi.INVALID
    assert garm_lib.garm_config_default(None) == capi.INVALID
    bad = capi.grid_desc(3, [3, 3, 3], 0.1, [0, 0, 0])  # smaller than the solid ring
    h = C.c_void_p()
    assert garm_lib.garm_sim_create(C.byref(bad), None, None, C.byref(h)) == capi.INVALID


def test_header_constants_match_the_binding():
    """Field ids and reinitialisation forms of include/garm.h against the ctypes binding."""
    text = HEADER.read_text()
    fields = {m.group(1): int(m.group(2)) for m in re.finditer(r"GARM_FIELD_([A-Z_]+)\s*=\s*(\d+)", text)}
    count = fields.pop("COUNT")
    assert count == len(fields) == len(capi.FIELD_NAMES)
    for name, value in fields.items():
        assert getattr(capi, "FIELD_" + name) == value, name
    forms = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define GARM_REINIT_([A-Z_]+) (\d+)", text)}
    assert forms == {f: i for i, f in enumerate(capi.REINIT_FORMS)}


def test_new_config_fields_are_validated_without_a_gpu(garm_lib):
    g = capi.grid_desc(3, [12, 12, 12], 0.1, [0.6, 0.6, 0.6])
    h = C.c_void_p()
    for field, bad in (("restart_newton", 2), ("fast_marching", -1), ("record_volume", 3), ("air_extrap_radius", 1000.0),
                       ("boundary_extrap_radius", float("nan")), ("cg_cells_per_block", -5)):
        cfg = host_default_config(**{field: bad})
        assert garm_lib.garm_sim_create(C.byref(g), C.byref(cfg), None, C.byref(h)) == capi.INVALID, field
    size = (C.c_int * 3)(20, 20, 20)
    assert garm_lib.garm_reinit_plan_set(3, capi.PRECISION_MIXED, size, 7, 128, 8) == capi.INVALID
    assert garm_lib.garm_reinit_plan_set(3, capi.PRECISION_MIXED, size, 3, 100, 8) == capi.INVALID


def test_estimate_bytes_validates_like_create(garm_lib):
    """garm_sim_estimate_bytes applies the grid and configuration checks of garm_sim_create
    before sizing anything, and sizes a valid request without a GPU."""
    n = C.c_size_t()
    est = garm_lib.garm_sim_estimate_bytes
    ok = capi.grid_desc(3, [32, 32, 32], 1 / 32, [1.0, 1.0, 1.0])
    assert est(C.byref(ok), None, C.byref(n)) == capi.OK and n.value > 0
    small = n.value
    big = capi.grid_desc(3, [64, 64, 64], 1 / 64, [1.0, 1.0, 1.0])
    assert est(C.byref(big), None, C.byref(n)) == capi.OK and 6 * small < n.value < 10 * small
    for grid in (capi.grid_desc(3, [0, 8, 8], 0.1, [0, 0, 0]), capi.grid_desc(3, [-4, 8, 8], 0.1, [0, 0, 0]),
                 capi.grid_desc(3, [3, 3, 3], 0.1, [0, 0, 0]), capi.grid_desc(3, [1300, 1300, 1300], 1e-3, [0, 0, 0]),
                 capi.grid_desc(3, [20000, 8, 8], 0.1, [0, 0, 0]), capi.grid_desc(3, [8, 8, 8], 0.0, [0, 0, 0]),
                 capi.grid_desc(4, [8, 8, 8], 0.1, [0, 0, 0])):
        assert est(C.byref(grid), None, C.byref(n)) == capi.INVALID, list(grid.resolution)
    for field, bad in (("precision", 7), ("fast_marching", 2), ("cg_tolerance", 0.0), ("air_extrap_radius", 300.0)):
        cfg = host_default_config(**{field: bad})
        assert est(C.byref(ok), C.byref(cfg), C.byref(n)) == capi.INVALID, field
    assert est(None, None, C.byref(n)) == capi.INVALID and est(C.byref(ok), None, None) == capi.INVALID


def test_barrier_selftest_validates_without_a_gpu(garm_lib):
    ms = C.c_double()
    for blocks, rounds, never in ((0, 10, 0), (4, 0, 0), (4, 10, 2), (-1, 10, 1)):
        assert garm_lib.garm_barrier_selftest(blocks, rounds, never, C.byref(ms)) == capi.INVALID


def test_fp64_peak_selftest_validates_without_a_gpu(garm_lib):
    out = C.c_double()
    for per_sm, iters in ((0, 100), (17, 100), (4, 0), (4, (1 << 22) + 1)):
        assert garm_lib.garm_fp64_peak_selftest(per_sm, iters, C.byref(out)) == capi.INVALID
    assert garm_lib.garm_fp64_peak_selftest(4, 100, None) == capi.INVALID
