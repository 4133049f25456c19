"""Host logic of the request loop, with the device stage replaced by a fake
(no GPU): admission in arrival order by slots and memory budget, overlap of
admitted units, multi-wavelength requests, refusal of a unit larger than
the budget, and the latency statistics."""
import threading
import time

import numpy as np
import pytest

from at3d_gb300 import serving


class FakePlan:
    def __init__(self, problem):
        self.problem = problem
        self.sizes = {"device_bytes": problem["bytes"]}
        self._p = object()

    def release(self):
        self._p = None


class FakeRTE:
    lock = threading.Lock()
    live = 0
    peak = 0
    order = []

    @classmethod
    def from_plan(cls, plan, device=0):
        r = cls()
        r.pb = plan.problem
        with cls.lock:
            cls.live += 1
            cls.peak = max(cls.peak, cls.live)
            cls.order.append(r.pb["id"])
        return r

    def set_sweep_mode(self, m):
        assert m == "graph"

    def set_transform_mode(self, m):
        pass

    def solve(self, maxiter, verbose=False):
        time.sleep(self.pb["t"])
        return 7, 1e-5

    def render(self, x, y, z, mu, phi):
        return np.full(len(x), float(self.pb["id"]), np.float32)

    def close(self):
        with FakeRTE.lock:
            FakeRTE.live -= 1


class FakeServer(serving.SolveServer):
    def _free_bytes(self):
        return 10_000

    def _bind_device(self):
        pass


@pytest.fixture(autouse=True)
def fakes(monkeypatch):
    monkeypatch.setattr(serving, "HostPlan", FakePlan)
    monkeypatch.setattr(serving, "RTE", FakeRTE)
    FakeRTE.live = FakeRTE.peak = 0
    FakeRTE.order = []


RAYS = tuple(np.zeros(5) for _ in range(5))


def test_overlap_and_results():
    with FakeServer(slots=3, hbm_budget=1000, planners=2) as srv:
        futs = [srv.submit({"id": i, "bytes": 100, "t": 0.05}, RAYS) for i in range(9)]
        res = [f.result(timeout=30) for f in futs]
        st = srv.stats()
    for i, r in enumerate(res):
        assert np.all(r.radiance == i) and r.iterations == [7]
    assert FakeRTE.peak == 3 and st["peak_in_flight"] == 3
    assert FakeRTE.order == list(range(9))          # admitted in arrival order
    assert st["completed"] == 9 and st["units"] == 9 and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0 and st["solves_per_s"] > 0


def test_budget_limits_concurrency():
    with FakeServer(slots=4, hbm_budget=250, planners=2) as srv:
        futs = [srv.submit({"id": i, "bytes": 100, "t": 0.03}, RAYS) for i in range(8)]
        [f.result(timeout=30) for f in futs]
        st = srv.stats()
    assert FakeRTE.peak == 2 and st["peak_device_bytes"] <= 250


def test_multi_wavelength_request():
    with FakeServer(slots=2, hbm_budget=1000) as srv:
        f = srv.submit([{"id": 10 + w, "bytes": 100, "t": 0.02} for w in range(4)], RAYS)
        r = f.result(timeout=30)
    assert [float(a[0]) for a in r.radiances] == [10, 11, 12, 13]
    assert r.device_bytes == 100


def test_too_large_unit_fails_alone():
    with FakeServer(slots=2, hbm_budget=300) as srv:
        bad = srv.submit({"id": 0, "bytes": 400, "t": 0.0}, RAYS)
        good = srv.submit({"id": 1, "bytes": 100, "t": 0.0}, RAYS)
        with pytest.raises(MemoryError):
            bad.result(timeout=30)
        assert good.result(timeout=30).radiance[0] == 1
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1


def test_poisson_arrivals():
    t = serving.poisson_arrivals(10.0, 2000, seed=1)
    assert np.all(np.diff(t) > 0)
    assert abs(2000 / t[-1] - 10.0) < 1.0
