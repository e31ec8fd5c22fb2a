"""The entry point that allocates nothing: garm_reinit_device_noalloc.

It serves callers that may not allocate device memory themselves — a plug-in
whose host application owns all GPU memory, or a real-time loop that cannot take
cudaMalloc's implicit synchronisation.  The caller hands over a device field;
the stage planes come from one fixed array inside the library.

Checked through the C ABI against the allocating entry point garm_reinit_host
(same tolerance as the other reinitialisation tests, 1e-10) on two calls in a
row, so the second call runs on scratch that still holds the first call's data;
the 3D call is also checked against the CPU oracle.  Further checks: repeated
calls of an already-seen shape leave the device's free memory unchanged, and a
host pointer is refused before any kernel could dereference it.
This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from garm import capi

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _field(dim: int, n: int, length: float = 10.0):
    dx = length / n
    x = (np.arange(n) + 0.5) * dx - length / 2
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    r = np.sqrt(sum(g * g for g in grids))
    r0 = 0.2313 * length
    phi = (np.exp(r - r0) - 1) * 0.05  # a non-SDF with the circle/sphere r0 as zero set
    return np.ascontiguousarray(phi), dx


def _size(phi: np.ndarray):
    return (C.c_int * 3)(*([int(s) for s in reversed(phi.shape)] + [1] * (3 - phi.ndim)))


def _noalloc_on(lib, dev, phi: np.ndarray, dx: float, iters: int, cfl: float) -> None:
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.garm_reinit_device_noalloc(phi.ndim, _size(phi), dx, C.c_void_p(dev.data_ptr()), iters, cfl, C.c_void_p(stream))
    assert st == capi.OK, capi.STATUS_NAMES.get(st, st)


def _noalloc(lib, phi: np.ndarray, dx: float, iters: int, cfl: float) -> np.ndarray:
    import torch
    dev = torch.tensor(phi, dtype=torch.float64, device="cuda")
    _noalloc_on(lib, dev, phi, dx, iters, cfl)
    torch.cuda.synchronize()
    return dev.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_two_calls(garm_lib, oracle_mod):
    pytest.importorskip("torch")
    first, dx1 = _field(3, 48)     # 110592 cells
    second, dx2 = _field(2, 300)   # 90000 cells: smaller, so stale scratch from call 1 remains beyond it
    out1 = _noalloc(garm_lib, first, dx1, 12, 0.5)
    out2 = _noalloc(garm_lib, second, dx2, 20, 0.5)
    ref1 = capi.reinit_host(first, dx1, 12, 0.5)
    ref2 = capi.reinit_host(second, dx2, 20, 0.5)
    assert np.max(np.abs(out1 - ref1)) <= TOL
    assert np.max(np.abs(out2 - ref2)) <= TOL
    assert np.max(np.abs(out2 - second)) > 1e-3  # the call did change the field
    # the 3D call against the CPU oracle directly, not only against the other GPU entry point
    assert np.max(np.abs(out1 - oracle_mod.reinit(first, dx1, 12, 0.5))) <= TOL


def test_noalloc_repeated_calls_allocate_nothing(garm_lib):
    """After one call of a shape (which loads the kernels and looks up the scratch
    address), further calls must not change the device's free memory."""
    torch = pytest.importorskip("torch")
    phi, dx = _field(3, 40)
    dev = torch.tensor(phi, dtype=torch.float64, device="cuda")
    _noalloc_on(garm_lib, dev, phi, dx, 4, 0.5)  # warm-up: 12 sub-stages, then one copy back
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        _noalloc_on(garm_lib, dev, phi, dx, 4, 0.5)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # five more calls of 4 iterations each continue from the warmed-up field
    assert np.all(np.isfinite(dev.cpu().numpy()))


def test_noalloc_refuses_a_host_pointer(garm_lib):
    """A host array (the mistake its near-twin garm_reinit_host invites) returns
    GARM_INVALID; cudaPointerGetAttributes reports it as not device memory."""
    pytest.importorskip("torch")
    phi, dx = _field(2, 64)
    host = np.ascontiguousarray(phi)
    before = host.copy()
    st = garm_lib.garm_reinit_device_noalloc(2, _size(phi), dx, host.ctypes.data_as(C.c_void_p), 3, 0.5, None)
    assert st == capi.INVALID
    assert np.array_equal(host, before)


def test_noalloc_rejects_grids_beyond_the_fixed_scratch(garm_lib):
    too_big = (C.c_int * 3)(128, 128, 33)  # 540672 cells > 2^19
    assert capi.NOALLOC_MAX_CELLS == 1 << 19
    st = garm_lib.garm_reinit_device_noalloc(3, too_big, 0.1, C.c_void_p(16), 1, 0.5, None)
    assert st == capi.INVALID
