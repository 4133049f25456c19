"""Host logic of SolversDict (at3d/containers.py:674-742) with fake solvers
(no GPU): which solvers are solved, the threaded path, the sweep mode set
for concurrent solves and restored, errors re-raised; and deferred RTE
creation, whose planning errors surface at the first use of the solver."""
import threading
import time

import pytest

from at3d_gb300.containers import SolversDict
from at3d_gb300.solver import RTE, SHDOMError


class FakeRTE(RTE):
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, solved=False, fail=False):
        self._solved, self._fail, self.calls, self.modes = solved, fail, 0, []
        self._sweep_mode = "persistent"

    def check_solved(self, verbose=True):
        return self._solved

    def set_sweep_mode(self, mode):
        self.modes.append(mode)
        self._sweep_mode = mode

    def solve(self, maxiter, init_solution=True, setup_grid=True, verbose=True, solve=True):
        with FakeRTE.lock:
            FakeRTE.live += 1
            FakeRTE.peak = max(FakeRTE.peak, FakeRTE.live)
        time.sleep(0.05)
        with FakeRTE.lock:
            FakeRTE.live -= 1
        if self._fail:
            raise SHDOMError("planted failure")
        self.calls += 1
        self._solved = True

    def close(self):
        pass


@pytest.fixture(autouse=True)
def reset():
    FakeRTE.live = FakeRTE.peak = 0


def test_only_unsolved_and_sequential():
    sd = SolversDict()
    a, b = FakeRTE(solved=True), FakeRTE()
    sd.add_solver(0.66, a)
    sd.add_solver(0.86, b)
    assert sd.to_solve(False)[0] == [0.86]
    sd.solve(n_jobs=1)
    assert (a.calls, b.calls) == (0, 1) and FakeRTE.peak == 1
    sd.solve(n_jobs=1, overwrite_solver=True)
    assert (a.calls, b.calls) == (1, 2)


def test_threaded_concurrency_and_mode_restored():
    sd = SolversDict()
    ss = [FakeRTE() for _ in range(6)]
    for k, s in enumerate(ss):
        sd.add_solver(k, s)
    sd.solve(n_jobs=3)
    assert all(s.calls == 1 for s in ss)
    assert FakeRTE.peak == 3
    assert all(s.modes == ["graph", "persistent"] for s in ss)


def test_error_reraised_after_all_threads():
    sd = SolversDict()
    ss = [FakeRTE(), FakeRTE(fail=True), FakeRTE()]
    for k, s in enumerate(ss):
        sd.add_solver(k, s)
    with pytest.raises(SHDOMError, match="planted"):
        sd.solve(n_jobs=3)
    assert ss[0].calls == 1 and ss[2].calls == 1
    assert ss[1].sweep_mode == "persistent"


def test_type_checked():
    with pytest.raises(TypeError):
        SolversDict().add_solver(0, object())


def test_deferred_planning_error_surfaces_at_first_use():
    import dataclasses
    from at3d_gb300.scenes import cloud_blob
    pb = cloud_blob(nx=8, ny=8, nz=6)
    pb = dataclasses.replace(pb, params=dataclasses.replace(pb.params, split_accuracy=0.03))
    r = RTE.from_problem(pb, defer=True)   # returns at once
    with pytest.raises(SHDOMError, match="splitting"):
        r.sizes
