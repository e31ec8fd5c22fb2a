"""Shared test set-up: import paths, the `gpu` marker, and oracle/GPU pairs."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "garm-ls_gb300"))
sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels through the C ABI")


def gpu_available() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def pytest_collection_modifyitems(config, items):
    # A GPU test on a machine without a GPU is an error of the run, not a skip:
    # only deselect them when the user did not ask for them explicitly.
    pass


@pytest.fixture(scope="session")
def oracle_mod():
    from garm.build import build_oracle
    build_oracle()
    from oracle import oracle as O
    return O


@pytest.fixture(scope="session")
def garm_lib():
    from garm.build import build_library
    build_library()
    from garm import capi
    return capi.load()
