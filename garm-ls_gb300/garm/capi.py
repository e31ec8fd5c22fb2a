"""ctypes binding of libgarm.so (include/garm.h).

The library is the product: every call goes to CUDA kernels for sm_103a.  If
the shared library is missing or fails to load, `load()` raises — there is no
CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parents[1]
LIB_PATH = PKG_DIR / "libgarm.so"

# garm_status
OK, INVALID, OOM, NOT_CONVERGED, NUMERIC, CUDA_ERROR, TIMEOUT, UNSUPPORTED = range(8)
STATUS_NAMES = {OK: "ok", INVALID: "invalid", OOM: "oom", NOT_CONVERGED: "not_converged", NUMERIC: "numeric",
                CUDA_ERROR: "cuda_error", TIMEOUT: "timeout", UNSUPPORTED: "unsupported"}

PRECISION_FP64, PRECISION_MIXED = 0, 1
REINIT_FORMS = ["cells", "columns", "sweeps", "tiled", "pairs", "pairs_tiled"]  # GARM_REINIT_CELLS, _COLUMNS, _SWEEPS, _TILED, _PAIRS, _PAIRS_TILED

# garm_field
(FIELD_VELOCITY, FIELD_LEVEL_SET, FIELD_REF_MAP, FIELD_REF_MAP_GRAD, FIELD_REF_LEVEL_SET, FIELD_REF_LEVEL_SET_GRAD,
 FIELD_ADV_REGION, FIELD_ORI_LEVEL_SET, FIELD_TMP_LEVEL_SET, FIELD_CELL_DIST, FIELD_NODE_DIST, FIELD_FRACTION,
 FIELD_BOUNDARY_VELOCITY, FIELD_BOUNDARY_NORMAL, FIELD_PRESSURE, FIELD_LEVEL_SET_GRAD) = range(16)
FIELD_NAMES = {
    FIELD_VELOCITY: "velocity", FIELD_LEVEL_SET: "levelSet", FIELD_REF_MAP: "refMap", FIELD_REF_MAP_GRAD: "refMapGrad",
    FIELD_REF_LEVEL_SET: "refLevelSet", FIELD_REF_LEVEL_SET_GRAD: "refLevelSetGrad", FIELD_ADV_REGION: "advRegion",
    FIELD_ORI_LEVEL_SET: "oriLevelSet", FIELD_TMP_LEVEL_SET: "tmpLevelSet", FIELD_CELL_DIST: "cellDist",
    FIELD_NODE_DIST: "nodeDist", FIELD_FRACTION: "fraction", FIELD_BOUNDARY_VELOCITY: "boundaryVelocity",
    FIELD_BOUNDARY_NORMAL: "boundaryNormal", FIELD_PRESSURE: "pressure", FIELD_LEVEL_SET_GRAD: "levelSetGrad",
}


class GarmError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("resolution", C.c_int * 3), ("boundary_width", C.c_int),
                ("spacing", C.c_double), ("center", C.c_double * 3)]


class Config(C.Structure):
    _fields_ = [("precision", C.c_int), ("reinit_iters", C.c_int), ("reinit_cfl", C.c_double),
                ("reinit_interval", C.c_int), ("cg_tolerance", C.c_double), ("cg_max_iters", C.c_int),
                ("boundary_extrap_radius", C.c_double), ("air_extrap_radius", C.c_double),
                ("rm_threshold", C.c_double), ("rm_band", C.c_double), ("rm_ratio", C.c_double),
                ("enable_gravity", C.c_int), ("mixed_residual_drop", C.c_double),
                ("mixed_replace_interval", C.c_int), ("cg_cells_per_block", C.c_int), ("record_volume", C.c_int), ("restart_newton", C.c_int),
                ("fast_marching", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("restarted", C.c_int), ("cg_iterations", C.c_int), ("cg_refinements", C.c_int),
                ("unknowns", C.c_int), ("cg_residual", C.c_double), ("rm_total", C.c_int), ("rm_bad", C.c_int),
                ("ms_total", C.c_double), ("ms_stage", C.c_double * 8), ("volume", C.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "ms_stage"}
        d["ms_stage"] = list(self.ms_stage)
        return d


STAGE_NAMES = ["advect", "compose", "reinit", "extrap_collider", "rm_check_restart", "body_force", "project",
               "extrap_air_enforce_bc"]

# Every exported entry point with its ctypes signature (the header's declarations).
_SIGS = {
    "garm_abi_version": (C.c_int, []),
    "garm_status_string": (C.c_char_p, [C.c_int]),
    "garm_config_default": (C.c_int, [C.POINTER(Config)]),
    "garm_sim_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(Config), C.c_void_p, C.POINTER(C.c_void_p)]),
    "garm_sim_destroy": (C.c_int, [C.c_void_p]),
    "garm_sim_estimate_bytes": (C.c_int, [C.POINTER(GridDesc), C.POINTER(Config), C.POINTER(C.c_size_t)]),
    "garm_sim_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "garm_sim_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "garm_sim_field_bytes": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "garm_sim_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "garm_sim_download": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "garm_sim_initialize": (C.c_int, [C.c_void_p]),
    "garm_sim_finish_load": (C.c_int, [C.c_void_p]),
    "garm_sim_advance": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(StepStats)]),
    "garm_sim_set_clock": (C.c_int, [C.c_void_p, C.c_uint, C.c_double]),
    "garm_sim_set_restart_override": (C.c_int, [C.c_void_p, C.c_int]),
    "garm_sim_advance_auto": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(StepStats)]),
    "garm_sim_graph_active": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "garm_reinit_plan_set": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int]),
    "garm_sim_volume": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "garm_sim_reinit_plan": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_float)]),
    "garm_sim_enqueue_auto": (C.c_int, [C.c_void_p, C.c_int]),
    "garm_sim_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "garm_sim_collect": (C.c_int, [C.c_void_p, C.POINTER(StepStats)]),
    "garm_batch_advance_auto": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(StepStats)]),
    "garm_sim_max_speed": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "garm_sim_time_step": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_double)]),
    "garm_stage_advect": (C.c_int, [C.c_void_p, C.c_double]),
    "garm_stage_compose": (C.c_int, [C.c_void_p]),
    "garm_stage_reinit": (C.c_int, [C.c_void_p]),
    "garm_stage_extrap_collider": (C.c_int, [C.c_void_p]),
    "garm_stage_rm_check": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "garm_stage_restart": (C.c_int, [C.c_void_p]),
    "garm_stage_body_force": (C.c_int, [C.c_void_p, C.c_double]),
    "garm_stage_project": (C.c_int, [C.c_void_p, C.POINTER(StepStats)]),
    "garm_stage_extrap_air": (C.c_int, [C.c_void_p]),
    "garm_stage_enforce_bc": (C.c_int, [C.c_void_p]),
    "garm_stage_enforce_boundary_level_set": (C.c_int, [C.c_void_p, C.c_double]),
    "garm_reinit_host": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int, C.c_double, C.c_int]),
    "garm_reinit_device_noalloc": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.c_double, C.c_void_p, C.c_int, C.c_double, C.c_void_p]),
    "garm_barrier_selftest": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "garm_fp64_peak_selftest": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
}

NOALLOC_MAX_CELLS = 1 << 19

_LIB = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libgarm.so and declare its signatures.  Raises if it is absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(status: int, what: str) -> None:
    if status != OK:
        raise GarmError(status, what)


RESTART_AUTO, RESTART_NEVER, RESTART_ALWAYS = 0, 1, 2


def default_config(**overrides) -> Config:
    cfg = Config()
    check(load().garm_config_default(C.byref(cfg)), "garm_config_default")
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def grid_desc(dim: int, resolution, spacing: float, center, boundary_width: int = 2) -> GridDesc:
    g = GridDesc()
    g.dim = dim
    for a in range(3):
        g.resolution[a] = int(resolution[a]) if a < dim else 1
        g.center[a] = float(center[a]) if a < dim else 0.0
    g.boundary_width = boundary_width
    g.spacing = float(spacing)
    return g


def field_shapes(grid: GridDesc) -> dict:
    """Per-field numpy shapes of the .sav layout (x-fastest: numpy order reversed)."""
    d = grid.dim
    n = [grid.resolution[a] for a in range(d)]
    cell = tuple(reversed(n))
    faces = [tuple(reversed([n[b] + (1 if b == a else 0) for b in range(d)])) for a in range(d)]
    node = tuple(reversed([x + 1 for x in n]))
    return {"cell": cell, "faces": faces, "node": node}


class Simulation:
    """One device-resident scene behind the C ABI (garm_sim*)."""

    def __init__(self, grid: GridDesc, cfg: Config | None = None, stream: int | None = None):
        self.lib = load()
        self.grid = grid
        self.cfg = cfg if cfg is not None else default_config()
        self.handle = C.c_void_p()
        check(self.lib.garm_sim_create(C.byref(grid), C.byref(self.cfg), C.c_void_p(stream) if stream else None,
                                       C.byref(self.handle)), "garm_sim_create")
        self.shapes = field_shapes(grid)

    # -- lifetime
    def close(self) -> None:
        if self.handle:
            self.lib.garm_sim_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- transfer
    def field_bytes(self, field: int) -> int:
        n = C.c_size_t()
        check(self.lib.garm_sim_field_bytes(self.handle, field, C.byref(n)), "garm_sim_field_bytes")
        return n.value

    def launch_count(self) -> int:
        n = C.c_longlong()
        check(self.lib.garm_sim_launch_count(self.handle, C.byref(n)), "garm_sim_launch_count")
        return n.value

    def device_bytes(self) -> int:
        n = C.c_size_t()
        check(self.lib.garm_sim_device_bytes(self.handle, C.byref(n)), "garm_sim_device_bytes")
        return n.value

    def upload(self, field: int, data: np.ndarray) -> None:
        dtype = np.uint8 if field == FIELD_ADV_REGION else np.float64
        arr = np.ascontiguousarray(data, dtype=dtype)
        check(self.lib.garm_sim_upload(self.handle, field, arr.ctypes.data, arr.nbytes), f"upload {FIELD_NAMES[field]}")

    def download(self, field: int, out: np.ndarray | None = None) -> np.ndarray:
        nbytes = self.field_bytes(field)
        dtype = np.uint8 if field == FIELD_ADV_REGION else np.float64
        if out is None:
            out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        check(self.lib.garm_sim_download(self.handle, field, out.ctypes.data, out.nbytes), f"download {FIELD_NAMES[field]}")
        return out

    # -- Simulation interface (Common/Util/Simulation.h:10-34)
    def dimension(self) -> int:
        return self.grid.dim

    def initialize(self) -> int:
        st = self.lib.garm_sim_initialize(self.handle)
        if st not in (OK, NOT_CONVERGED):
            check(st, "garm_sim_initialize")
        return st

    def finish_load(self) -> None:
        check(self.lib.garm_sim_finish_load(self.handle), "garm_sim_finish_load")

    def advance(self, dt: float, allow_not_converged: bool = True) -> dict:
        stats = StepStats()
        st = self.lib.garm_sim_advance(self.handle, float(dt), C.byref(stats))
        if st != OK and not (allow_not_converged and st == NOT_CONVERGED):
            check(st, "garm_sim_advance")
        d = stats.as_dict()
        d["status"] = st
        return d

    def set_restart_override(self, mode: int) -> None:
        """garm_sim_set_restart_override: RESTART_AUTO, RESTART_NEVER or RESTART_ALWAYS."""
        check(self.lib.garm_sim_set_restart_override(self.handle, int(mode)), "garm_sim_set_restart_override")

    def set_clock(self, frame_rate: int = 25, cfl: float = 1.0) -> None:
        check(self.lib.garm_sim_set_clock(self.handle, int(frame_rate), float(cfl)), "garm_sim_set_clock")

    def advance_auto(self, steps: int, allow_not_converged: bool = True) -> dict:
        stats = StepStats()
        st = self.lib.garm_sim_advance_auto(self.handle, int(steps), C.byref(stats))
        if st != OK and not (allow_not_converged and st == NOT_CONVERGED):
            check(st, "garm_sim_advance_auto")
        d = stats.as_dict()
        d["status"] = st
        return d

    def enqueue_auto(self, steps: int) -> None:
        check(self.lib.garm_sim_enqueue_auto(self.handle, int(steps)), "garm_sim_enqueue_auto")

    def poll(self) -> bool:
        v = C.c_int()
        check(self.lib.garm_sim_poll(self.handle, C.byref(v)), "garm_sim_poll")
        return bool(v.value)

    def collect(self, allow_not_converged: bool = True) -> dict:
        stats = StepStats()
        st = self.lib.garm_sim_collect(self.handle, C.byref(stats))
        if st != OK and not (allow_not_converged and st == NOT_CONVERGED):
            check(st, "garm_sim_collect")
        d = stats.as_dict()
        d["status"] = st
        return d

    def graph_active(self) -> bool:
        v = C.c_int()
        check(self.lib.garm_sim_graph_active(self.handle, C.byref(v)), "garm_sim_graph_active")
        return bool(v.value)

    def reinit_plan(self) -> dict:
        f, b, c, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        check(self.lib.garm_sim_reinit_plan(self.handle, C.byref(f), C.byref(b), C.byref(c), C.byref(ms)),
              "garm_sim_reinit_plan")
        return {"form": REINIT_FORMS[f.value], "threads": b.value, "cells_per_thread": c.value, "ms": ms.value}

    def volume(self, evaluator_order: bool = False) -> float:
        """calculateVolume of the current tmp level set (garm_sim_volume)."""
        v = C.c_double()
        check(self.lib.garm_sim_volume(self.handle, int(evaluator_order), C.byref(v)), "garm_sim_volume")
        return v.value

    def max_speed(self) -> float:
        v = C.c_double()
        check(self.lib.garm_sim_max_speed(self.handle, C.byref(v)), "garm_sim_max_speed")
        return v.value

    def time_step(self, cfl: float) -> float:
        v = C.c_double()
        check(self.lib.garm_sim_time_step(self.handle, float(cfl), C.byref(v)), "garm_sim_time_step")
        return v.value

    # -- single stages
    def stage(self, name: str, *args):
        lib, h = self.lib, self.handle
        if name == "advect":
            check(lib.garm_stage_advect(h, float(args[0])), name)
        elif name == "compose":
            check(lib.garm_stage_compose(h), name)
        elif name == "reinit":
            check(lib.garm_stage_reinit(h), name)
        elif name == "extrap_collider":
            check(lib.garm_stage_extrap_collider(h), name)
        elif name == "rm_check":
            keep, tot, bad = C.c_int(), C.c_int(), C.c_int()
            check(lib.garm_stage_rm_check(h, C.byref(keep), C.byref(tot), C.byref(bad)), name)
            return keep.value, tot.value, bad.value
        elif name == "restart":
            check(lib.garm_stage_restart(h), name)
        elif name == "body_force":
            check(lib.garm_stage_body_force(h, float(args[0])), name)
        elif name == "project":
            stats = StepStats()
            st = lib.garm_stage_project(h, C.byref(stats))
            if st not in (OK, NOT_CONVERGED):
                check(st, name)
            d = stats.as_dict()
            d["status"] = st
            return d
        elif name == "extrap_air":
            check(lib.garm_stage_extrap_air(h), name)
        elif name == "enforce_bc":
            check(lib.garm_stage_enforce_bc(h), name)
        elif name == "enforce_boundary_level_set":
            check(lib.garm_stage_enforce_boundary_level_set(h, float(args[0])), name)
        else:
            raise ValueError(name)
        return None


def fp64_peak_tflops(blocks_per_sm: int = 4, iters: int = 4096) -> float:
    """garm_fp64_peak_selftest: measured FP64 FMA throughput of the current device (TFLOP/s)."""
    out = C.c_double(0)
    check(load().garm_fp64_peak_selftest(int(blocks_per_sm), int(iters), C.byref(out)), "garm_fp64_peak_selftest")
    return out.value


def barrier_selftest(blocks: int, rounds: int, never_complete: bool = False) -> tuple[int, float]:
    """garm_barrier_selftest: (status, ms per barrier passed) of one cooperative launch."""
    ms = C.c_double()
    st = load().garm_barrier_selftest(int(blocks), int(rounds), int(bool(never_complete)), C.byref(ms))
    return st, ms.value


def estimate_bytes(grid: GridDesc, cfg: Config) -> int:
    n = C.c_size_t()
    check(load().garm_sim_estimate_bytes(C.byref(grid), C.byref(cfg), C.byref(n)), "garm_sim_estimate_bytes")
    return n.value


def reinit_host(phi: np.ndarray, spacing: float, iters: int, cfl: float, precision: int = PRECISION_FP64) -> np.ndarray:
    """WENO5 reinitialisation of a numpy cell field on the GPU (TestReinit usage)."""
    lib = load()
    a = np.ascontiguousarray(phi, dtype=np.float64).copy()
    dim = a.ndim
    size = (C.c_int * 3)(*([int(x) for x in reversed(a.shape)] + [1] * (3 - dim)))
    check(lib.garm_reinit_host(dim, size, float(spacing), a.ctypes.data_as(C.POINTER(C.c_double)), int(iters), float(cfl),
                               int(precision)), "garm_reinit_host")
    return a


def reinit_plan_set(shape_xyz, precision: int, form: str, threads: int, cells_per_thread: int) -> None:
    """Pin the reinitialisation launch plan of one grid shape (cells per axis, x first):
    form "cells" | "columns" | "sweeps" | "tiled"; threads=0 returns the shape to the autotuner."""
    size = (C.c_int * 3)(*([int(x) for x in shape_xyz] + [1] * (3 - len(shape_xyz))))
    check(load().garm_reinit_plan_set(len(shape_xyz), int(precision), size, REINIT_FORMS.index(form), int(threads),
                                      int(cells_per_thread)), "garm_reinit_plan_set")


def batch_advance_auto(sims: list, steps: int) -> list:
    """garm_batch_advance_auto over `sims` (each created with its own stream)."""
    lib = load()
    arr = (C.c_void_p * len(sims))(*[s.handle.value for s in sims])
    stats = (StepStats * len(sims))()
    st = lib.garm_batch_advance_auto(arr, len(sims), int(steps), stats)
    if st not in (OK, NOT_CONVERGED):
        check(st, "garm_batch_advance_auto")
    return [s.as_dict() for s in stats]
