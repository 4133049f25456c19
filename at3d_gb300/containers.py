"""Collections of solvers and sensors, mirroring at3d.containers
(at3d/containers.py): ``SolversDict`` (:674-742), RTE objects keyed by
wavelength, solved together; ``SensorsDict`` (:39-672), the sensors of each
instrument with its uncertainty model, rendered by the solvers whose key is
the sensor's wavelength.

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

import copy
import threading
import warnings
from collections import OrderedDict

import numpy as np

from .sensor import STOKES_NAMES, calculate_observables
from .solver import RTE

_RAY_VARS = ("ray_x", "ray_y", "ray_z", "ray_mu", "ray_phi", "ray_weight", "pixel_index")


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


class SensorsDict(OrderedDict):
    """Sensors by instrument: ``self[instrument] = {'sensor_list': [...],
    'uncertainty_model': model}`` (at3d/containers.py:39-672)."""

    def add_sensor(self, instrument, sensor: dict):
        for k in ("ray_x", "ray_y", "ray_z", "ray_mu", "ray_phi", "cam_mu", "stokes"):
            if k not in sensor:
                raise KeyError(f"sensor is missing '{k}'")
        if instrument not in self:
            self._add_instrument(instrument)
        self[instrument]["sensor_list"].append(sensor)

    def _add_instrument(self, key):
        self[key] = {"sensor_list": [], "uncertainty_model": None}

    def add_uncertainty_model(self, instrument, uncertainty_model):
        if instrument not in self:
            self._add_instrument(instrument)
        self[instrument]["uncertainty_model"] = uncertainty_model

    def calculate_uncertainties(self, instrument):
        model = self[instrument].get("uncertainty_model")
        if model is None:
            raise KeyError(f"There is no uncertainty model for instrument '{instrument}'. please add one.")
        for sensor in self[instrument]["sensor_list"]:
            model.calculate_uncertainties(sensor)

    def add_noise(self, instrument):
        for sensor in self[instrument]["sensor_list"]:
            self[instrument]["uncertainty_model"].add_noise(sensor)

    def make_forward_sensors(self, instrument_list=None) -> "SensorsDict":
        """A deep copy of the sensors (for the forward model's output in a retrieval)."""
        out = SensorsDict()
        for key in (self if instrument_list is None else instrument_list):
            if key not in self:
                raise KeyError(f"Instrument '{key}' is not in SensorsDict")
            out[key] = OrderedDict(sensor_list=[copy.deepcopy(s) for s in self[key]["sensor_list"]],
                                   uncertainty_model=self[key]["uncertainty_model"])
        return out

    def sort_sensors(self, solvers):
        """Sensors grouped by solver key (the sensor's wavelength): one
        merged ray set per solver with the rays of each sensor in turn, and
        the (instrument, index) of each sensor (at3d/containers.py:235-353)."""
        merged, mappings = OrderedDict(), OrderedDict()
        for key in solvers:
            sensors, mapping = [], []
            for instrument, data in self.items():
                for i, sensor in enumerate(data["sensor_list"]):
                    if sensor.get("wavelength") == key:
                        sensors.append(sensor)
                        mapping.append((instrument, i))
            if not sensors:
                warnings.warn(f"No sensors found matching solver with key '{key}'")
                merged[key] = None
            else:
                m = {v: np.concatenate([np.asarray(s[v]) for s in sensors]) for v in _RAY_VARS}
                m["rays_per_image"] = np.array([len(s["ray_mu"]) for s in sensors])
                merged[key] = m
            mappings[key] = mapping
        return merged, mappings

    def get_measurements(self, solvers, n_jobs: int = 1, mpi_comm=None, maxiter: int = 100, verbose: bool = True,
                         init_solution: bool = True, setup_grid: bool = True, destructive: bool = False,
                         overwrite_solver: bool = False):
        """Solves the solvers that need it, renders every sensor's rays (one
        render per solver over the rays of all its sensors) and stores the
        pixel observables in the sensors (at3d/containers.py:133-233)."""
        if not isinstance(solvers, SolversDict):
            raise TypeError(f"`solvers` should be of type '{SolversDict}' not '{type(solvers)}'")
        if mpi_comm is not None:
            raise NotImplementedError("MPI distribution is not supported: one process drives one GPU")
        merged, mappings = self.sort_sensors(solvers)
        solvers.solve(n_jobs=n_jobs, maxiter=maxiter, verbose=verbose, init_solution=init_solution,
                      setup_grid=setup_grid, overwrite_solver=overwrite_solver)
        for key, m in merged.items():
            if m is None:
                continue
            rays = solvers[key].integrate_to_sensor(dict(m))
            ends = np.cumsum(m["rays_per_image"])
            starts = ends - m["rays_per_image"]
            for (instrument, i), a, b in zip(mappings[key], starts, ends):
                sensor = self[instrument]["sensor_list"][i]
                calculate_observables(sensor, {s: rays[s][a:b] for s in STOKES_NAMES if s in rays})

    def get_unique_solvers(self):
        return np.unique([s["wavelength"] for inst in self.values() for s in inst["sensor_list"]])

    def get_minimum_stokes(self):
        """The number of Stokes components each solver needs (1, 3 or 4)."""
        out = OrderedDict((float(k), 0) for k in self.get_unique_solvers())
        for inst in self.values():
            for s in inst["sensor_list"]:
                st = np.asarray(s["stokes"], bool)
                n = 4 if st.all() else int(np.flatnonzero(~st)[0])
                n = 3 if n == 2 else n
                out[float(s["wavelength"])] = max(out[float(s["wavelength"])], n)
        return out

    def get_image(self, instrument, sensor_index: int) -> dict:
        """The sensor's pixel observables reshaped to its image_shape
        ([nx, ny], x the slow axis as the projections order pixels)."""
        sensor = self[instrument]["sensor_list"][sensor_index]
        shape = sensor.get("image_shape")
        if shape is None:
            raise ValueError("the sensor has no image shape")
        img = lambda v: np.asarray(v).reshape(shape[1], shape[0]).T     # Fortran-order reshape to [nx, ny]
        out = {"x": img(sensor["cam_x"]), "y": img(sensor["cam_y"]), "mu": img(sensor["cam_mu"]),
               "phi": img(sensor["cam_phi"])}
        for s, on in zip(STOKES_NAMES, sensor["stokes"]):
            if on and s in sensor:
                out[s] = img(sensor[s])
        return out

    def get_images(self, instrument) -> list:
        return [self.get_image(instrument, i) for i in range(len(self[instrument]["sensor_list"]))]

    @property
    def npixels(self) -> int:
        return int(sum(len(s["cam_mu"]) for inst in self.values() for s in inst["sensor_list"]))

    @property
    def nmeasurements(self) -> int:
        return int(sum(len(s["cam_mu"]) * int(np.sum(s["stokes"])) for inst in self.values()
                       for s in inst["sensor_list"]))
