"""ctypes binding of the CPU oracle (oracle/garm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py as the checker — never by the library.  The oracle is
a restatement of the reference's FP64 algorithm; see the header of
garm_oracle.cpp for what it is pinned against.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
from garm.capi import (Config, GridDesc, StepStats, FIELD_ADV_REGION, FIELD_NAMES, OK, NOT_CONVERGED,  # noqa: E402
                       field_shapes)

LIB_PATH = REPO / "oracle" / "liboracle.so"
from garm.build import ORACLE_FLAGS  # noqa: E402
BUILD_FLAGS = "g++ -std=c++20 " + " ".join(ORACLE_FLAGS)

STAGES = {"advect": 0, "compose": 1, "reinit": 2, "extrap_collider": 3, "rm_check": 4, "restart": 5,
          "body_force": 6, "project": 7, "extrap_air": 8, "enforce_bc": 9, "enforce_boundary_level_set": 10}

_LIB = None


def load() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        from garm.build import build_oracle
        build_oracle()
    lib = C.CDLL(str(LIB_PATH))
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.POINTER(GridDesc), C.POINTER(Config)]
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_field_bytes.restype = C.c_size_t
    lib.orc_field_bytes.argtypes = [C.c_void_p, C.c_int]
    lib.orc_upload.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.orc_download.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.orc_initialize.argtypes = [C.c_void_p]
    lib.orc_restart.argtypes = [C.c_void_p]
    lib.orc_advance.argtypes = [C.c_void_p, C.c_double, C.POINTER(StepStats)]
    lib.orc_stage.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(StepStats), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.orc_max_speed.restype = C.c_double
    lib.orc_max_speed.argtypes = [C.c_void_p]
    lib.orc_volume.restype = C.c_double
    lib.orc_volume.argtypes = [C.c_void_p]
    lib.orc_mc_cube_volume.restype = C.c_double
    lib.orc_mc_cube_volume.argtypes = [C.POINTER(C.c_double)]
    lib.orc_ms_square_area.restype = C.c_double
    lib.orc_ms_square_area.argtypes = [C.POINTER(C.c_double)]
    lib.orc_mc_tables_ok.restype = C.c_int
    lib.orc_field_volume.restype = C.c_double
    lib.orc_field_volume.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int]
    lib.orc_set_threads.argtypes = [C.c_int]
    lib.orc_max_threads.restype = C.c_int
    lib.orc_reinit.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int, C.c_double]
    lib.orc_fast_marching.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int, C.c_void_p]
    lib.orc_hermite_eval.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.orc_cubic_eval.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    _LIB = lib
    return lib


REF_LIB_PATH = REPO / "oracle" / "_ref" / "libgarmref.so"
REF_BUILD = REPO / "oracle" / "build_ref.sh"
_REF = None


def ref_available() -> bool:
    """True when the reference binary (oracle/_ref, built from the reference's own sources by
    oracle/build_ref.sh) exists or can be built here."""
    if REF_LIB_PATH.exists():
        return True
    return Path("/root/reference/Source/Core/LevelSetLiquid.cpp").exists()


def load_ref() -> C.CDLL:
    """The reference binary: the unmodified LevelSetLiquid<Dim> driven by oracle/ref_harness.cpp."""
    global _REF
    if _REF is not None:
        return _REF
    if not REF_LIB_PATH.exists():
        import subprocess
        subprocess.run(["sh", str(REF_BUILD)], check=True, stdout=subprocess.DEVNULL)
    lib = C.CDLL(str(REF_LIB_PATH))
    lib.ref_create.restype = C.c_void_p
    lib.ref_create.argtypes = [C.POINTER(GridDesc), C.POINTER(Config)]
    lib.ref_destroy.argtypes = [C.c_void_p]
    lib.ref_field_bytes.restype = C.c_size_t
    lib.ref_field_bytes.argtypes = [C.c_void_p, C.c_int]
    lib.ref_upload.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.ref_download.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.ref_initialize.argtypes = [C.c_void_p]
    lib.ref_restart.argtypes = [C.c_void_p]
    lib.ref_advance.argtypes = [C.c_void_p, C.c_double, C.POINTER(StepStats)]
    lib.ref_stage.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(StepStats), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.ref_max_speed.restype = C.c_double
    lib.ref_max_speed.argtypes = [C.c_void_p]
    lib.ref_volume.restype = C.c_double
    lib.ref_volume.argtypes = [C.c_void_p]
    lib.ref_profile.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.ref_set_threads.argtypes = [C.c_int]
    lib.ref_max_threads.restype = C.c_int
    lib.ref_reinit.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_double, C.POINTER(C.c_double), C.c_int, C.c_double]
    _REF = lib
    return lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleSim:
    """CPU FP64 LevelSetLiquid<Dim> with the same field/stage vocabulary as garm.capi.Simulation:
    the port (garm_oracle.cpp)."""

    PREFIX = "orc_"

    def _lib(self) -> C.CDLL:
        return load()

    def _fn(self, name: str):
        return getattr(self.lib, self.PREFIX + name)

    def __init__(self, grid: GridDesc, cfg: Config):
        self.lib = self._lib()
        self.grid = grid
        self.cfg = cfg
        self.h = self._fn("create")(C.byref(grid), C.byref(cfg))
        if not self.h:
            raise ValueError(f"{self.PREFIX}create failed")
        self.shapes = field_shapes(grid)

    def close(self):
        if self.h:
            self._fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, field: int, data: np.ndarray) -> None:
        dtype = np.uint8 if field == FIELD_ADV_REGION else np.float64
        a = np.ascontiguousarray(data, dtype=dtype)
        if self._fn("upload")(self.h, field, a.ctypes.data, a.nbytes) != OK:
            raise ValueError(f"orc_upload {FIELD_NAMES[field]}")

    def download(self, field: int) -> np.ndarray:
        n = self._fn("field_bytes")(self.h, field)
        dtype = np.uint8 if field == FIELD_ADV_REGION else np.float64
        out = np.empty(n // np.dtype(dtype).itemsize, dtype=dtype)
        if self._fn("download")(self.h, field, out.ctypes.data, out.nbytes) != OK:
            raise ValueError(f"orc_download {FIELD_NAMES[field]}")
        return out

    def initialize(self) -> int:
        return self._fn("initialize")(self.h)

    def advance(self, dt: float) -> dict:
        st = StepStats()
        rc = self._fn("advance")(self.h, float(dt), C.byref(st))
        d = st.as_dict()
        d["status"] = rc
        return d

    def max_speed(self) -> float:
        return self._fn("max_speed")(self.h)

    def volume(self) -> float:
        """calculateVolume (LevelSetLiquid.cpp:1162-1190) of the current tmp level set."""
        return self._fn("volume")(self.h)

    def stage(self, name: str, arg: float = 0.0):
        st = StepStats()
        keep, tot, bad = C.c_int(), C.c_int(), C.c_int()
        rc = self._fn("stage")(self.h, STAGES[name], float(arg), C.byref(st), C.byref(keep), C.byref(tot), C.byref(bad))
        if rc not in (OK, NOT_CONVERGED):
            raise ValueError(f"orc_stage {name}: {rc}")
        if name == "rm_check":
            return keep.value, tot.value, bad.value
        if name == "project":
            d = st.as_dict()
            d["status"] = rc
            return d
        return None


class RefSim(OracleSim):
    """The reference itself: LevelSetLiquid<Dim> from the reference's own sources
    (oracle/_ref), with the port's field/stage vocabulary.  Only the reference's constants
    (30 WENO5 iterations at 0.9, its restart test, 2000 solver iterations, FP64) are
    accepted; rm_check returns (keep, -1, -1), the reference not exposing its counts."""

    PREFIX = "ref_"

    def _lib(self) -> C.CDLL:
        return load_ref()

    def profile(self) -> dict:
        """The reference's own stage timers of the last step (LevelSetLiquid.cpp:601-606), seconds."""
        out = (C.c_double * 4)()
        self.lib.ref_profile(self.h, out)
        return {"tadvect": out[0], "tproject": out[1], "trestart": out[2], "textrap": out[3]}


def ref_reinit(phi: np.ndarray, spacing: float, iters: int, cfl: float) -> np.ndarray:
    """Reinitialization::solve<5> of the reference binary on a bare cell field."""
    a = np.ascontiguousarray(phi, dtype=np.float64).copy()
    size = (C.c_int * 3)(*([int(x) for x in reversed(a.shape)] + [1] * (3 - a.ndim)))
    if load_ref().ref_reinit(a.ndim, size, float(spacing), _dp(a), int(iters), float(cfl)) != OK:
        raise ValueError("ref_reinit")
    return a


def ref_set_threads(n: int) -> None:
    load_ref().ref_set_threads(int(n))


def set_threads(n: int) -> None:
    load().orc_set_threads(int(n))


def max_threads() -> int:
    return load().orc_max_threads()


def reinit(phi: np.ndarray, spacing: float, iters: int, cfl: float) -> np.ndarray:
    a = np.ascontiguousarray(phi, dtype=np.float64).copy()
    size = (C.c_int * 3)(*([int(x) for x in reversed(a.shape)] + [1] * (3 - a.ndim)))
    if load().orc_reinit(a.ndim, size, float(spacing), _dp(a), int(iters), float(cfl)) != OK:
        raise ValueError("orc_reinit")
    return a


def fast_marching(phi: np.ndarray, spacing: float, max_steps: int, mark: np.ndarray | None = None) -> np.ndarray:
    """FastMarching::perform on a cell field (numpy order, x fastest): seeds from the sign
    changes, or the cells where `mark` is non-zero keep |φ|."""
    a = np.ascontiguousarray(phi, dtype=np.float64).copy()
    size = (C.c_int * 3)(*([int(x) for x in reversed(a.shape)] + [1] * (3 - a.ndim)))
    m = None if mark is None else np.ascontiguousarray(mark, dtype=np.uint8)
    if load().orc_fast_marching(a.ndim, size, float(spacing), _dp(a), int(max_steps), None if m is None else m.ctypes.data) != OK:
        raise ValueError("orc_fast_marching")
    return a


def hermite_eval(val: np.ndarray, grad: np.ndarray, spacing: float, origin, pts: np.ndarray):
    """Scalar Hermite interpolation; grad has a trailing axis of size dim."""
    dim = val.ndim
    v = np.ascontiguousarray(val, dtype=np.float64)
    g = np.ascontiguousarray(grad, dtype=np.float64)
    size = (C.c_int * 3)(*([int(x) for x in reversed(v.shape)] + [1] * (3 - dim)))
    o = np.ascontiguousarray(origin, dtype=np.float64)
    p = np.ascontiguousarray(pts, dtype=np.float64)
    ov = np.empty(len(p))
    og = np.empty((len(p), dim))
    load().orc_hermite_eval(dim, size, float(spacing), _dp(o), _dp(v), _dp(g), len(p), _dp(p), _dp(ov), _dp(og))
    return ov, og


def cubic_eval(val: np.ndarray, spacing: float, origin, pts: np.ndarray) -> np.ndarray:
    dim = val.ndim
    v = np.ascontiguousarray(val, dtype=np.float64)
    size = (C.c_int * 3)(*([int(x) for x in reversed(v.shape)] + [1] * (3 - dim)))
    o = np.ascontiguousarray(origin, dtype=np.float64)
    p = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.empty(len(p))
    load().orc_cubic_eval(dim, size, float(spacing), _dp(o), _dp(v), len(p), _dp(p), _dp(out))
    return out


def mc_cube_volume(v8) -> float:
    """MC-style volume of one unit cube, corners in the evaluator's order."""
    a = np.ascontiguousarray(v8, dtype=np.float64)
    return load().orc_mc_cube_volume(_dp(a))


def ms_square_area(v4) -> float:
    """Filled marching-squares area of one unit square, corners (0,0), (1,0), (0,1), (1,1)."""
    a = np.ascontiguousarray(v4, dtype=np.float64)
    return load().orc_ms_square_area(_dp(a))


def field_volume(phi: np.ndarray, spacing: float, evaluator_order: bool = False) -> float:
    """calculateVolume of a bare cell field (numpy shape reversed(size)); evaluator_order
    passes each cube's corners in the MC-style evaluator's own order (3D) instead of the
    reference's x-fastest stencil order."""
    a = np.ascontiguousarray(phi, dtype=np.float64)
    size = (C.c_int * 3)(*([int(x) for x in reversed(a.shape)] + [1] * (3 - a.ndim)))
    return load().orc_field_volume(a.ndim, size, float(spacing), _dp(a), int(evaluator_order))


def mc_tables_ok() -> bool:
    return bool(load().orc_mc_tables_ok())
