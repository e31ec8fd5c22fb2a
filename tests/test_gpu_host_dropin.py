"""The C++ drop-in (garm-ls_gb300/host/GpuLevelSetLiquid.h) driven like the
reference demo: build the scene on the host, initialize, run frames with the
Simulator dt policy, saveFrame, loadFrame into a fresh instance, and check the
two continue bit-identically (LevelSetLiquid.cpp:425-526 round trip)."""
from __future__ import annotations

import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,n", [(2, 48), (3, 24)])
def test_demo_frames_and_resume(garm_lib, tmp_path, dim, n):
    from garm.build import build_demo
    exe = build_demo()
    res = subprocess.run([str(exe), str(dim), str(n), "2", str(tmp_path / "frame")], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "resume check" in res.stdout
    for name in ("velocity.sav", "refMap.sav", "refLevelSet.sav", "advRegion.sav", "refMapGrad.sav", "levelSet.bin"):
        assert (tmp_path / "frame" / name).stat().st_size > 0
    # .sav sizes follow the reference layout
    cells = (n + 4) ** dim
    assert (tmp_path / "frame" / "refMap.sav").stat().st_size == cells * 8 * dim
    assert (tmp_path / "frame" / "refMapGrad.sav").stat().st_size == cells * 8 * dim * dim
    assert (tmp_path / "frame" / "advRegion.sav").stat().st_size == cells
