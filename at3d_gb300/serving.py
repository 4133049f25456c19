"""Request loop for RTE solves: continuous admission by slots and HBM budget.

A request is one medium at one or more wavelengths (one RTE problem per
wavelength, any grid and angular resolution) plus the rays to render from
each solved wavelength.  Each wavelength is a unit of work that goes
through two stages:

1. planning on the host (``HostPlan``: grid, sweep schedule, ordinates,
   medium, direct beam), by a pool of planner threads that touch no GPU;
   the plan reports the device memory the unit's state will hold;
2. admission: planned units are admitted in arrival order as soon as a
   device slot is free and their memory fits in what the budget has left.
   An admitted unit is put on the device, solved and rendered on its own
   handle and CUDA stream, so the kernels of all admitted units interleave
   on the GPU (each handle launches its sweep level by level, so no kernel
   waits on thread blocks that another unit's kernels could keep from
   running, and replays each solution iteration from a captured CUDA
   graph).  Its state stays in HBM from upload to render and is freed
   when the unit completes, which frees its slot and memory for the next.

Units of a request that arrives while others are on the GPU start as soon
as slots and memory free up: the loop never waits for a batch to drain.
Latency is measured per request, from submission (arrival) to the
radiances of all its wavelengths being back on the host; ``stats()``
reports p50 / p99 beside throughput.
"""
from __future__ import annotations

import os
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from .solver import RTE, HostPlan


@dataclass
class Result:
    radiances: list          # one float32 array per wavelength, in the order submitted
    iterations: list
    solcrit: list
    latency_s: float
    device_bytes: int        # the largest unit's device memory

    @property
    def radiance(self) -> np.ndarray:
        return self.radiances[0]


@dataclass
class _Request:
    future: Future
    t_arrival: float
    nunits: int
    rays: tuple
    maxiter: int
    transform_mode: str | None
    radiances: list = None
    iterations: list = None
    solcrit: list = None
    remaining: int = 0
    failed: bool = False
    need_max: int = 0


@dataclass
class _Unit:
    req: _Request
    index: int
    seq: int                 # arrival order over all units
    problem: object
    plan: HostPlan | None = None
    need: int = 0
    error: BaseException | None = None


@dataclass
class _Stats:
    completed: int = 0
    failed: int = 0
    units: int = 0
    rays: int = 0
    latencies: list = field(default_factory=list)
    t_first: float | None = None
    t_last: float | None = None
    peak_in_flight: int = 0
    peak_bytes: int = 0


class SolveServer:
    """Continuous-admission solve server on one GPU.

    slots: most units (wavelength solves) on the device at once.
    hbm_budget: bytes of device memory the server may hold for unit state
    (default: 80% of the memory free at start).
    planners: host threads that plan units ahead of admission.
    """

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int | None = None,
                 planners: int | None = None):
        self.device = device
        if hbm_budget is None:
            hbm_budget = int(0.8 * self._free_bytes())
        self.slots = int(slots)
        self.budget = int(hbm_budget)
        self._seq = 0
        self._in_use = 0
        self._in_flight = 0
        self._intake: queue.Queue = queue.Queue()
        self._planned: dict[int, _Unit] = {}   # seq -> unit, planned and waiting for admission
        self._next_seq = 0                     # the next unit to admit, in arrival order
        self._cv = threading.Condition()
        self._stop = False
        self._stats = _Stats()
        n_pl = planners or max(1, min(8, (os.cpu_count() or 2) // 2))
        self._planners = [threading.Thread(target=self._planner, daemon=True) for _ in range(n_pl)]
        self._workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(self.slots)]
        for t in self._planners + self._workers:
            t.start()

    # -------------------------------------------------------------- client
    def submit(self, problems, rays, maxiter: int = 100, transform_mode: str | None = None) -> Future:
        """Queue one request: a problem or a list of problems (wavelengths of
        one medium) and the rays (x, y, z, mu, phi) rendered from each.  The
        future resolves to a Result, or to the exception of the first unit
        that failed (a unit whose memory exceeds the whole budget fails with
        MemoryError)."""
        if not isinstance(problems, (list, tuple)):
            problems = [problems]
        n = len(problems)
        req = _Request(Future(), time.perf_counter(), n, tuple(rays), maxiter, transform_mode,
                       [None] * n, [0] * n, [0.0] * n, n)
        with self._cv:
            units = []
            for i, pb in enumerate(problems):
                units.append(_Unit(req, i, self._seq, pb))
                self._seq += 1
            if self._stats.t_first is None:
                self._stats.t_first = req.t_arrival
        for u in units:
            self._intake.put(u)
        return req.future

    def close(self):
        for _ in self._planners:
            self._intake.put(None)
        for t in self._planners:
            t.join()
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._workers:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def stats(self) -> dict:
        with self._cv:
            s = self._stats
            lat = np.asarray(s.latencies, np.float64)
            span = (s.t_last - s.t_first) if (s.t_first is not None and s.t_last is not None) else 0.0
            return {
                "completed": s.completed, "failed": s.failed, "units": s.units,
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
                "mean_ms": float(lat.mean() * 1e3) if lat.size else None,
                "requests_per_s": (s.completed / span) if span > 0 else None,
                "solves_per_s": (s.units / span) if span > 0 else None,
                "rays_per_s": (s.rays / span) if span > 0 else None,
                "peak_in_flight": s.peak_in_flight, "peak_device_bytes": s.peak_bytes,
                "budget_bytes": self.budget,
            }

    # -------------------------------------------------------------- device
    def _free_bytes(self) -> int:
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("SolveServer needs a CUDA device")
        return int(torch.cuda.mem_get_info(self.device)[0])

    def _bind_device(self):
        import torch
        torch.cuda.set_device(self.device)

    # -------------------------------------------------------------- stages
    def _planner(self):
        while True:
            u = self._intake.get()
            if u is None:
                return
            try:
                u.plan = HostPlan(u.problem)
                u.need = int(u.plan.sizes["device_bytes"])
                if u.need > self.budget:
                    raise MemoryError(f"unit needs {u.need} bytes of device memory, budget is {self.budget}")
            except BaseException as e:  # the unit fails at admission; the server goes on
                u.error = e
                if u.plan is not None:
                    u.plan.release()
                    u.plan = None
            with self._cv:
                self._planned[u.seq] = u
                self._cv.notify_all()

    def _take(self):
        """The next unit in arrival order, once planned and once its memory
        fits; blocks.  A failed unit is handed out at once (it needs nothing)."""
        with self._cv:
            while True:
                u = self._planned.get(self._next_seq)
                if u is not None and (u.error is not None or self._in_use + u.need <= self.budget):
                    del self._planned[self._next_seq]
                    self._next_seq += 1
                    if u.error is None:
                        self._in_use += u.need
                        self._in_flight += 1
                        st = self._stats
                        st.peak_in_flight = max(st.peak_in_flight, self._in_flight)
                        st.peak_bytes = max(st.peak_bytes, self._in_use)
                    self._cv.notify_all()
                    return u
                if self._stop and self._next_seq >= self._seq:
                    return None
                self._cv.wait(timeout=0.05)

    def _finish(self, u: _Unit, rad=None, it=0, sc=0.0, err=None):
        req = u.req
        done, lat = False, 0.0
        with self._cv:
            if err is not None:
                if not req.failed:
                    req.failed = True
                    self._stats.failed += 1
                    req.future.set_exception(err)
            else:
                req.radiances[u.index] = rad
                req.iterations[u.index] = it
                req.solcrit[u.index] = sc
                req.need_max = max(req.need_max, u.need)
                self._stats.units += 1
                self._stats.rays += len(rad)
            req.remaining -= 1
            if req.remaining == 0 and not req.failed:
                t = time.perf_counter()
                self._stats.completed += 1
                lat = t - req.t_arrival
                self._stats.latencies.append(lat)
                self._stats.t_last = t
                done = True
        if done:
            req.future.set_result(Result(req.radiances, req.iterations, req.solcrit, lat, req.need_max))

    def _worker(self):
        self._bind_device()
        while True:
            u = self._take()
            if u is None:
                return
            if u.error is not None:
                self._finish(u, err=u.error)
                continue
            rte = None
            try:
                if u.req.failed:
                    raise RuntimeError("request already failed")
                rte = RTE.from_plan(u.plan, device=self.device)
                u.plan = None
                rte.set_sweep_mode("graph")
                if u.req.transform_mode:
                    rte.set_transform_mode(u.req.transform_mode)
                it, sc = rte.solve(u.req.maxiter, verbose=False)
                rad = rte.render(*u.req.rays)
                self._finish(u, rad, it, sc)
            except BaseException as e:
                self._finish(u, err=e)
            finally:
                if rte is not None:
                    rte.close()
                if u.plan is not None:
                    u.plan.release()
                with self._cv:
                    self._in_use -= u.need
                    self._in_flight -= 1
                    self._cv.notify_all()


def poisson_arrivals(rate_per_s: float, n: int, seed: int = 0) -> np.ndarray:
    """Arrival times (s from start) of a Poisson stream."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))


def run_stream(server: SolveServer, requests, arrivals, **kw) -> list:
    """Submit (problems, rays) pairs at the given arrival times; returns the
    results in submission order."""
    t0 = time.perf_counter()
    futs = []
    for (pb, rays), ta in zip(requests, arrivals):
        dt = ta - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        futs.append(server.submit(pb, rays, **kw))
    return [f.result() for f in futs]
