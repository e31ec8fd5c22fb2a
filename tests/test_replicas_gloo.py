"""Multi-process host logic of bench.py on CPU (gloo, world_size 2): each rank
times its own replica, the job time is the max over ranks and `value` is all
ranks' cell-steps over that time.  No GPU is touched."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 + 50.0 * rank          # rank 1 is slower
    m = bench.reduce_max(local_ms, world)
    bench.barrier(world)
    out[rank] = (m, bench.replica_value(world, 128 ** 3, 10, m))
    dist.destroy_process_group()


def test_max_over_ranks_and_weak_scaling_value():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of this (threaded) process
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        m, v = out[r]
        assert m == 150.0
        assert v == pytest.approx(2 * 128 ** 3 * 10 / 0.150)
