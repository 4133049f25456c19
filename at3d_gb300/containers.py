"""Collections of solvers, mirroring at3d.containers.SolversDict
(at3d/containers.py:674-742): RTE objects keyed by wavelength, solved
together.

With n_jobs > 1 the reference runs the solvers' Fortran calls in joblib
threads.  Here the solvers run in threads as well, each on its own handle and
CUDA stream, so their kernels interleave on the device: the latency-bound
sweep levels of one solve share the GPU with the transforms and source
passes of the others.  During a threaded solve every solver uses the sweep
mode without waits between thread blocks (per-level launches replayed from a
captured CUDA graph), which is what makes concurrent solves safe; the mode
is restored afterwards.
"""
from __future__ import annotations

import threading
from collections import OrderedDict

from .solver import RTE


class SolversDict(OrderedDict):
    """RTE objects keyed (typically) by wavelength."""

    def add_solver(self, key, solver):
        if not isinstance(solver, RTE):
            raise TypeError(f"solver should be of type '{RTE}'")
        self[key] = solver

    def to_solve(self, overwrite_solver: bool):
        """Keys and solvers still to solve (all of them with overwrite_solver)."""
        if overwrite_solver:
            return list(self.keys()), list(self.values())
        keys = [k for k, s in self.items() if not s.check_solved(verbose=False)]
        return keys, [self[k] for k in keys]

    def solve(self, n_jobs: int = 1, mpi_comm=None, overwrite_solver: bool = False, maxiter: int = 100,
              verbose: bool = True, init_solution: bool = True, setup_grid: bool = True):
        """Solve every solver not yet converged (all with overwrite_solver);
        n_jobs > 1 solves up to n_jobs of them at once on the device.  On one
        GB300, n_jobs = 1 is the fastest for grids whose sweep runs as a plane
        march (each solve already fills the GPU; four 128x128x64 wavelengths:
        3.9 solves/s one at a time, 3.55 four at once); solvers created with
        defer=True still plan on host threads while earlier ones solve."""
        if mpi_comm is not None:
            raise NotImplementedError("MPI distribution is not supported: one process drives one GPU")
        _, to_solve = self.to_solve(overwrite_solver)
        kw = dict(maxiter=maxiter, init_solution=init_solution, setup_grid=setup_grid, verbose=verbose)
        if n_jobs == 1 or len(to_solve) <= 1:
            for s in to_solve:
                s.solve(**kw)
            return
        errors = []
        lock = threading.Lock()
        pending = list(to_solve)

        def worker():
            while True:
                with lock:
                    if not pending:
                        return
                    s = pending.pop(0)
                mode = s.sweep_mode
                try:
                    s.set_sweep_mode("graph")
                    s.solve(**kw)
                except BaseException as e:  # re-raised in the caller
                    with lock:
                        errors.append(e)
                finally:
                    s.set_sweep_mode(mode)

        threads = [threading.Thread(target=worker) for _ in range(min(n_jobs, len(to_solve)))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
