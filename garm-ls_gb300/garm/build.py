"""Build the GB300 GARM-LS library (and, for tests, the CPU oracle).

`build_library()` compiles garm-ls_gb300/csrc/*.cu for sm_103a with nvcc, one
translation unit per process, and links garm-ls_gb300/libgarm.so in-tree.
`build_oracle()` compiles oracle/garm_oracle.cpp with g++ into oracle/liboracle.so;
the oracle is test infrastructure and is never loaded by the library itself.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parents[1]          # garm-ls_gb300/
REPO = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "libgarm.so"
ORACLE_SRC = REPO / "oracle" / "garm_oracle.cpp"
ORACLE_LIB = REPO / "oracle" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The oracle keeps the reference's evaluation order (no FMA contraction, no fast-math);
# -O3 as the reference's release build.
ORACLE_FLAGS = ["-O3", "-fopenmp", "-ffp-contract=off"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + res.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False, extra_flags: tuple[str, ...] = (), tag: str = "") -> Path:
    """libgarm.so, or with a tag a variant built with extra nvcc flags into _build_<tag>/ and
    libgarm_<tag>.so beside it (diagnostic builds; the library the package loads is untagged)."""
    nvcc = _nvcc()
    build_dir = BUILD_DIR.with_name(f"_build_{tag}") if tag else BUILD_DIR
    lib_path = LIB_PATH.with_name(f"libgarm_{tag}.so") if tag else LIB_PATH
    build_dir.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [REPO / "include" / "garm.h"]
    objs = []
    jobs = []
    for src in sources:
        obj = build_dir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", str(REPO / "include"), "-c", str(src), "-o", str(obj)])
    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if force or jobs or _stale(lib_path, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib_path), *map(str, objs), "-lcudart"])
    if verbose:
        print(f"built {lib_path}", file=sys.stderr)
    return lib_path


DEMO_SRC = PKG_DIR / "host" / "garm_demo.cpp"
DEMO_BIN = PKG_DIR / "garm_demo"


def build_demo(force: bool = False) -> Path:
    """The C++ host drop-in (host/GpuLevelSetLiquid.h) exercised by a demo driver."""
    deps = [DEMO_SRC, PKG_DIR / "host" / "GpuLevelSetLiquid.h", REPO / "include" / "garm.h", LIB_PATH]
    if force or _stale(DEMO_BIN, deps):
        _run(["g++", "-std=c++17", "-O2", "-Wall", "-I", str(REPO / "include"), "-I", str(PKG_DIR / "host"),
              str(DEMO_SRC), "-o", str(DEMO_BIN), "-L", str(PKG_DIR), "-lgarm", "-Wl,-rpath,$ORIGIN"])
    return DEMO_BIN


def build_oracle(force: bool = False) -> Path:
    if force or _stale(ORACLE_LIB, [ORACLE_SRC, REPO / "include" / "garm.h"]):
        _run(["g++", "-std=c++20", *ORACLE_FLAGS, "-fPIC", "-shared", "-o", str(ORACLE_LIB), str(ORACLE_SRC)])
    return ORACLE_LIB


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_demo(force="--force" in sys.argv)
    build_oracle(force="--force" in sys.argv)
