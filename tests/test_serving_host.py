"""Host logic of the serving loop (garm/serving.py) on the CPU, with the simulations
replaced by a fake that only tracks device memory and enqueued steps: admission waits
for arrival and for budget, the budget is never exceeded, every request completes with
its steps, and a request larger than the budget is refused."""
from __future__ import annotations

import time

import pytest

from garm import serving


class FakeSim:
    live = 0          # simulations alive at once
    peak = 0

    def __init__(self, grid, cfg, stream=None):
        self.n = int(grid.resolution[0])
        self.k = 0
        self.ready_at = 0.0
        self.closed = False
        FakeSim.live += 1
        FakeSim.peak = max(FakeSim.peak, FakeSim.live)

    def upload(self, *a):
        pass

    def initialize(self):
        return 0

    def stage(self, *a):
        return None

    def set_clock(self, *a):
        pass

    def enqueue_auto(self, k):
        assert not self.closed and k >= 1
        self.k = k
        self.ready_at = time.perf_counter() + 0.0005 * k

    def poll(self):
        return time.perf_counter() >= self.ready_at

    def collect(self):
        return {"ms_total": 0.5 * self.k, "restarted": 0}

    def download(self, field):
        return None

    def close(self):
        assert not self.closed
        self.closed = True
        FakeSim.live -= 1


def fake_bytes(grid, cfg):
    return int(grid.resolution[0]) ** 3 * 1000


@pytest.fixture
def fake_capi(monkeypatch):
    FakeSim.live = FakeSim.peak = 0
    monkeypatch.setattr(serving.capi, "Simulation", FakeSim)
    monkeypatch.setattr(serving.capi, "estimate_bytes", fake_bytes)


def test_requests_are_seeded_and_in_range():
    a = serving.make_requests(200, rate=20.0, seed=4, n_range=(48, 192), steps_range=(20, 200))
    b = serving.make_requests(200, rate=20.0, seed=4, n_range=(48, 192), steps_range=(20, 200))
    assert [(r.arrival, r.n, r.steps, r.kind, r.seed) for r in a] == [(r.arrival, r.n, r.steps, r.kind, r.seed) for r in b]
    assert all(48 <= r.n <= 192 and 20 <= r.steps <= 200 for r in a)
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert {r.kind for r in a} == {"dam", "drop"}
    mean_gap = a[-1].arrival / len(a)
    assert 0.035 < mean_gap < 0.065  # Poisson at 20/s


def test_budget_arrival_and_completion(fake_capi):
    reqs = serving.make_requests(12, rate=200.0, seed=2, n_range=(8, 14), steps_range=(3, 9))
    sizes = {r.rid: fake_bytes(serving.scenes.unit_grid(3, r.n), None) for r in reqs}
    budget = 2.5 * max(sizes.values())
    out = serving.Server(budget_bytes=budget, chunk=2).run(reqs, time_scale=0.2)
    res = out.pop("results")
    assert out["requests"] == len(reqs) and len(res) == len(reqs)
    assert out["peak_resident_bytes"] <= budget
    assert 2 <= out["peak_active"] == FakeSim.peak
    assert FakeSim.live == 0  # every simulation was closed
    by_id = {r.rid: r for r in reqs}
    for r in res:
        q = by_id[r.rid]
        assert r.admitted >= q.arrival * 0.2 - 1e-6   # not before it arrived
        assert r.completed >= r.admitted
        assert len(r.step_ms) == q.steps               # every step accounted
    cells = sum(serving.build_scene(q).interior_cells * q.steps for q in reqs)
    assert out["cell_steps"] == cells


def test_request_larger_than_the_budget_is_refused(fake_capi):
    reqs = serving.make_requests(3, seed=1, n_range=(10, 12), steps_range=(2, 3))
    with pytest.raises(ValueError):
        serving.Server(budget_bytes=100.0).run(reqs)
