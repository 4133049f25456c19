"""``RTE``: the SHDOM solver object, GB300 edition.

Mirrors the surface of ``at3d.solver.RTE`` (at3d/solver.py:143-791) for the
solve / render path: construction from numerical parameters, medium, source
and surface; ``solve(maxiter)``; ``integrate_to_sensor(sensor)``; ``fluxes``;
``save_solution``-style state export.  All numerical work happens in the
CUDA library behind include/shdom_gb300.h; the solution stays resident in
HBM between calls.
"""
from __future__ import annotations

import ctypes as C
import threading
import warnings

import numpy as np

from . import _lib
from ._abi import NumericalParams, Problem, Species



_CREATOR = None
_CREATOR_LOCK = threading.Lock()


def _lower_priority():
    """Nice +10 for the calling thread (and the planning threads it starts,
    which inherit it): planning then yields the cores to the thread that
    launches a running solve's kernels, and still has them all when nothing
    else runs."""
    import os
    try:
        os.setpriority(os.PRIO_PROCESS, threading.get_native_id(), 10)
    except (AttributeError, OSError):
        pass


def _deferred_creator():
    """The one background thread that builds deferred handles, in the order
    they were requested: the first solver's planning has every host core to
    itself, and the later ones plan (and upload) while the earlier ones
    solve, instead of all competing for the cores before the first solve."""
    global _CREATOR
    with _CREATOR_LOCK:
        if _CREATOR is None:
            from concurrent.futures import ThreadPoolExecutor
            _CREATOR = ThreadPoolExecutor(max_workers=1, thread_name_prefix="shdom-create",
                                          initializer=_lower_priority)
        return _CREATOR


def compute_sh(radiance, dirflux, solarmu: float, solaraz: float, srctype: str = "S", mm: int = 1) -> np.ndarray:
    """COMPUTE_SH (src/polarized/shdomsub2.f:1770-1836) for its four outputs:
    per grid point the mean intensity C0 R_00, the net flux vector
    Fx = -A (R_11 + R_1-1), Fy = -A (R_1-1 - R_11), Fz = C R_10 (A = sqrt(2 pi/3),
    C = sqrt(4 pi/3), C0 = 1/sqrt(4 pi), terms j = 0..3 of the radiance
    series; Fx = Fy = 0 when MM = 0), plus the direct beam for solar sources
    (mean intensity + F sec(mu0)/4pi, horizontal flux + F tan(theta0) (cos,
    sin of the solar azimuth), Fz - F).  ``radiance``: [npts, nlm] or
    [npts, nstokes, nlm] (the I row is used).  Returns [4, npts]."""
    r = np.asarray(radiance, np.float64)
    if r.ndim == 3:
        r = r[:, 0, :]
    f = np.asarray(dirflux, np.float64)
    pi = np.pi
    a, c, c0 = np.sqrt(2 * pi / 3), np.sqrt(4 * pi / 3), 1 / np.sqrt(4 * pi)
    out = np.zeros((4, r.shape[0]))
    out[0] = c0 * r[:, 0]
    out[3] = c * r[:, 2]
    if mm > 0:
        out[1] = -a * (r[:, 3] + r[:, 1])
        out[2] = -a * (r[:, 1] - r[:, 3])
    if srctype in ("S", "B"):
        sec = 1.0 / abs(solarmu)
        sin0 = np.sqrt(1.0 - solarmu ** 2)
        out[0] += f * sec / (4 * pi)
        out[1] += f * sin0 * np.cos(solaraz) * sec
        out[2] += f * sin0 * np.sin(solaraz) * sec
        out[3] -= f
    return out.astype(np.float32)


class SHDOMError(RuntimeError):
    """Raised for a non-zero SHDOM error code (at3d/checks.py:300-311)."""


def _check(h, rc):
    if rc != 0:
        msg = _lib.lib().shdom_last_error(h)
        raise SHDOMError(msg.decode() if msg else f"SHDOM error code {rc}")


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _sizes_dict(s) -> dict:
    return {name: getattr(s, name) for name, _ in s._fields_}


def plan_summary(problem: Problem) -> dict:
    """Sizes, sweep depths and the device memory of a problem, planned on the
    host only (no GPU is touched): for admission by memory budget."""
    L = _lib.lib()
    st = problem.to_struct()
    out = _lib.ShdomSizes()
    rc = L.shdom_plan_summary(C.byref(st), C.byref(out))
    if rc:
        raise SHDOMError(L.shdom_last_error(None).decode())
    return _sizes_dict(out)


def compute_netfluxdiv(radiance, dirflux, absorb, emit, solarmu: float, srctype: str = "S") -> np.ndarray:
    """COMPUTE_NETFLUXDIV (src/polarized/shdomsub2.f:1725-1764): per grid
    point -(sqrt(4 pi) absorb R_00 + absorb F sec(mu0) - 4 pi emit), the
    solar term for 'S' and 'B' sources, the emission for 'T' and 'B'.
    ``radiance`` [npts, nlm] or [npts, nstokes, nlm] (the I row is used);
    ``absorb`` / ``emit`` as ``shdom_point_absorption`` gives them."""
    r = np.asarray(radiance, np.float32)
    if r.ndim == 3:
        r = r[:, 0, :]
    pi = np.float32(np.arccos(np.float32(-1.0)))
    c = np.sqrt(np.float32(4.0) * pi)
    a = np.asarray(absorb, np.float32)
    hr = c * a * r[:, 0]
    if srctype in ("S", "B"):
        hr = hr + a * np.asarray(dirflux, np.float32) * (np.float32(1.0) / np.float32(abs(solarmu)))
    if srctype in ("T", "B"):
        hr = hr - np.float32(4.0) * pi * np.asarray(emit, np.float32)
    return -hr


def _optical_path(call, handle, sensor: dict, deltam_scaled_path: bool) -> dict:
    for k in ("ray_x", "ray_y", "ray_z", "ray_mu", "ray_phi"):
        if k not in sensor:
            raise KeyError(f"sensor needs '{k}'")
    x, y, z, mu, phi = RTE._ray_arrays(sensor["ray_x"], sensor["ray_y"], sensor["ray_z"], sensor["ray_mu"],
                                       sensor["ray_phi"])
    out = np.zeros(len(x), np.float32)
    dp = C.POINTER(C.c_double)
    rc = call(len(x), _fp(x), _fp(y), _fp(z), mu.ctypes.data_as(dp), phi.ctypes.data_as(dp),
              int(bool(deltam_scaled_path)), _fp(out))
    _check(handle, rc)
    sensor["optical_path_deltam" if deltam_scaled_path else "optical_path"] = out
    return sensor


class HostPlan:
    """A problem planned on the host (grid, sweep schedule, ordinates,
    medium, direct beam), not yet on a GPU; ``sizes["device_bytes"]`` is the
    memory a handle for it will hold.  ``RTE.from_plan`` consumes it."""

    def __init__(self, problem: Problem):
        L = _lib.lib()
        st = problem.to_struct()
        out = _lib.ShdomSizes()
        p = C.c_void_p()
        rc = L.shdom_plan_create(C.byref(st), C.byref(p), C.byref(out))
        if rc:
            raise SHDOMError(L.shdom_last_error(None).decode())
        self.problem = problem
        self.sizes = _sizes_dict(out)
        self._p = p

    def min_optical_path(self, sensor: dict, deltam_scaled_path: bool = False, do_all: bool = False) -> np.ndarray:
        """RTE.min_optical_path (at3d/solver.py:921-990; MIN_OPTICAL_DEPTH):
        per grid point the smallest optical path, over the rays of ``sensor``,
        at which a ray leaves a cell the point is a corner of; [nx1, ny1, nz],
        or [nrays, nx1, ny1, nz] with ``do_all``; 999 where no ray passes."""
        if not self._p:
            raise ValueError("plan already used or released")
        x, y, z, mu, phi = RTE._ray_arrays(sensor["ray_x"], sensor["ray_y"], sensor["ray_z"], sensor["ray_mu"],
                                           sensor["ray_phi"])
        s = self.sizes
        shp = (s["nx1"], s["ny1"], s["nz"])
        out = np.zeros(((len(x) if do_all else 1) * s["npts"]), np.float32)
        dp = C.POINTER(C.c_double)
        _check(None, _lib.lib().shdom_plan_min_optical_path(self._p, len(x), _fp(x), _fp(y), _fp(z),
                                                            mu.ctypes.data_as(dp), phi.ctypes.data_as(dp),
                                                            int(bool(deltam_scaled_path)), int(bool(do_all)),
                                                            _fp(out)))
        return out.reshape((len(x),) + shp) if do_all else out.reshape(shp)

    def point_absorption(self):
        """(absorb, emit) per grid point of the plan's medium."""
        if not self._p:
            raise ValueError("plan already used or released")
        n = self.sizes["npts"]
        absorb = np.zeros(n, np.float32); emit = np.zeros(n, np.float32)
        _check(None, _lib.lib().shdom_plan_point_absorption(self._p, _fp(absorb), _fp(emit)))
        return absorb, emit

    def optical_path(self, sensor: dict, deltam_scaled_path: bool = False) -> dict:
        """RTE.optical_path on the host plan (no GPU needed)."""
        if not self._p:
            raise ValueError("plan already used or released")
        return _optical_path(lambda *a: _lib.lib().shdom_plan_optical_path(self._p, *a), None, sensor,
                             deltam_scaled_path)

    def release(self):
        if self._p:
            _lib.lib().shdom_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class RTE:
    """Radiative-transfer solve of one medium at one wavelength.

    Parameters follow the reference: ``numerical_params`` (a NumericalParams),
    ``medium`` (dict name -> Species on a common property grid, given by
    ``grid``), ``source`` (source.solar, source.thermal or source.combined),
    ``surface`` (surface.lambertian or a bidirectional surface.BRDFSurface)
    and, for a thermal source, ``atmosphere`` with the medium's
    ``temperature`` [npx, npy, npz] in K (at3d/solver.py:1765-1800).
    """

    def __init__(self, numerical_params: NumericalParams, medium: dict, source, surface, grid,
                 num_stokes: int = 1, name: str | None = None, device: int = 0, atmosphere: dict | None = None):
        if num_stokes not in (1, 3):
            raise ValueError("num_stokes must be 1 (scalar radiance) or 3 (I, Q, U)")
        species = list(medium.values())
        srctype = getattr(source, "srctype", "S")
        temperature = None
        if atmosphere is not None and "temperature" in atmosphere:
            temperature = np.asarray(atmosphere["temperature"], np.float32)
            if np.any(temperature <= 0.0):
                raise ValueError("temperature must be positive")
        elif srctype in ("T", "B"):
            raise KeyError("'temperature' variable was not specified in `atmosphere` "
                           "and is required for a thermal source")
        self.problem = Problem(delx=grid.delx, dely=grid.dely, zlevels=np.asarray(grid.z, np.float32),
                               species=species, solarmu=source.solarmu, solaraz=source.solaraz,
                               solarflux=source.solarflux, skyrad=source.skyrad,
                               surface_delx=surface.delx, surface_dely=surface.dely, params=numerical_params,
                               num_stokes=num_stokes, srctype=srctype, units=getattr(source, "units", "R"),
                               wavelength=source.wavelength, temperature=temperature,
                               ground_temperature=getattr(surface, "ground_temperature", 288.0))
        if hasattr(surface, "kind"):      # surface.BRDFSurface
            self.problem.surface_brdf, self.problem.surface_params = surface.kind, surface.params
        else:
            self.problem.surface_albedo = surface.albedo
        self.name = name or f"Radiance {source.wavelength:1.3f} micron"
        self._create(device)

    @classmethod
    def from_problem(cls, problem: Problem, device: int = 0, name: str | None = None, defer: bool = False):
        """An RTE for a ready Problem.  With defer=True the host planning and
        the upload run on a background thread: the call returns at once, the
        first method that needs the device state waits for them, and a
        planning error is raised there (so several solvers can be planned
        while others already solve).  Deferred creations run one at a time
        in the order they were requested."""
        self = cls.__new__(cls)
        self.problem = problem
        self.name = name or "RTE"
        self._create(device, defer)
        return self

    @classmethod
    def from_plan(cls, plan: HostPlan, device: int = 0, name: str | None = None):
        """Put a host plan on the device (the plan is consumed)."""
        if not plan._p:
            raise ValueError("plan already used or released")
        self = cls.__new__(cls)
        self.problem = plan.problem
        self.name = name or "RTE"
        L = _lib.lib()
        self._struct = None
        p, plan._p = plan._p, None
        h = C.c_void_p()
        rc = L.shdom_create_planned(p, int(device), C.byref(h))
        if rc:
            raise SHDOMError(L.shdom_last_error(None).decode())
        self._h = h
        self._device = int(device)
        self._initialized = False
        return self

    def _create(self, device, defer: bool = False):
        L = _lib.lib()
        self._device = int(device)
        self._initialized = False

        def make():
            self._struct = self.problem.to_struct()
            h = C.c_void_p()
            rc = L.shdom_create(C.byref(self._struct), int(device), C.byref(h))
            if rc:
                raise SHDOMError(L.shdom_last_error(None).decode())
            return h

        if not defer:
            self._h = make()
            return
        self.__dict__["_pending"] = _deferred_creator().submit(make)

    @property
    def _h(self):
        pend = self.__dict__.pop("_pending", None)
        if pend is not None:
            try:
                self.__dict__["_hv"] = pend.result()
            except BaseException:  # a planning error is raised at the first use of the handle
                self.__dict__["_hv"] = None
                raise
        return self.__dict__.get("_hv")

    @_h.setter
    def _h(self, value):
        self.__dict__["_hv"] = value

    # ------------------------------------------------------------------
    @property
    def sizes(self) -> dict:
        s = _lib.ShdomSizes()
        _check(self._h, _lib.lib().shdom_get_sizes(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def solve(self, maxiter: int, init_solution: bool = True, setup_grid: bool = True, verbose: bool = True,
              solve: bool = True):
        """Initialise (direct beam, Eddington radiance, first source) and
        iterate until the solution criterion reaches solution_accuracy or the
        iteration count reaches maxiter (at3d/solver.py:279-631)."""
        L = _lib.lib()
        if init_solution or not self._initialized:
            _check(self._h, L.shdom_init_solution(self._h))
            self._initialized = True
        it, sc = C.c_int(0), C.c_float(0)
        _check(self._h, L.shdom_solution_iterations(self._h, int(maxiter), C.byref(it), C.byref(sc)))
        if verbose:
            print(f"! Iterations: {it.value:6d}     Final Criterion: {sc.value:9.6f}   [{self.name}]")
        if sc.value > self.problem.params.solution_accuracy:
            warnings.warn(f"solver did not converge to solution_accuracy in {it.value} iterations")
        return it.value, sc.value

    def check_solved(self, verbose: bool = True) -> bool:
        # a solver whose deferred creation has not been collected has never
        # solved: answer without waiting for it (SolversDict.to_solve asks
        # every solver before the first one solves)
        ok = "_pending" not in self.__dict__ and self._initialized
        ok = ok and self.sizes["solcrit"] <= self.problem.params.solution_accuracy
        if not ok and verbose:
            warnings.warn("RTE is not converged to the specified solution_accuracy")
        return ok

    def integrate_to_sensor(self, sensor: dict, single_scatter: bool = False, nosurface: bool = False) -> dict:
        """Radiance along the sensor's rays (at3d/solver.py:633-791); writes
        sensor['I'] (and 'Q', 'U' for a polarized solve) and returns the sensor.
        single_scatter: only the exact single scattering of the direct beam
        is integrated; nosurface: no boundary radiance is added where a ray
        leaves the domain (RENDER's SINGLESCATTER / NOSURFACE)."""
        self.check_solved(verbose=False)
        L = _lib.lib()
        _check(self._h, L.shdom_set_render_options(self._h, int(bool(single_scatter)), int(bool(nosurface))))
        try:
            out = self.render(sensor["ray_x"], sensor["ray_y"], sensor["ray_z"], sensor["ray_mu"], sensor["ray_phi"])
        finally:
            _check(self._h, L.shdom_set_render_options(self._h, 0, 0))
        if out.ndim == 1:
            sensor["I"] = out
        else:
            sensor["I"], sensor["Q"], sensor["U"] = out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy()
        return sensor

    @property
    def num_stokes(self) -> int:
        return int(self.problem.num_stokes)

    def render(self, x, y, z, mu, phi) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32); y = np.ascontiguousarray(y, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        mu = np.ascontiguousarray(mu, np.float64); phi = np.ascontiguousarray(phi, np.float64)
        nst = self.num_stokes
        out = np.zeros(len(x) if nst == 1 else (len(x), nst), np.float32)  # Stokes fastest, as STOKES(NSTOKES, NPIX)
        dp = C.POINTER(C.c_double)
        _check(self._h, _lib.lib().shdom_render(self._h, len(x), _fp(x), _fp(y), _fp(z), mu.ctypes.data_as(dp),
                                                 phi.ctypes.data_as(dp), _fp(out)))
        return out

    def render_device(self, x_ptr: int, y_ptr: int, z_ptr: int, mu_ptr: int, phi_ptr: int, out_ptr: int,
                      nrays: int, stream: int = 0):
        """Device-resident variant: CUDA device pointers (e.g. torch
        ``data_ptr()``) to float32 x/y/z/out and float64 mu/phi; launched
        asynchronously on ``stream``."""
        ptrs = [C.c_void_p(v) for v in (x_ptr, y_ptr, z_ptr, mu_ptr, phi_ptr, out_ptr, stream)]
        _check(self._h, _lib.lib().shdom_render_device(self._h, int(nrays), *ptrs))

    def export_state(self) -> dict:
        s = self.sizes
        n, nlm, nst = s["npts"], s["nlm"], s["nstokes"]
        shape = (n, nlm) if nst == 1 else (n, nst, nlm)
        src = np.zeros(shape, np.float32); rad = np.zeros(shape, np.float32)
        ns = np.zeros(n, np.int32); nr = np.zeros(n, np.int32)
        flx = np.zeros((n, 2), np.float32); dfl = np.zeros(n, np.float32)
        ip = C.POINTER(C.c_int)
        _check(self._h, _lib.lib().shdom_export_state(self._h, _fp(src), ns.ctypes.data_as(ip), _fp(rad),
                                                       nr.ctypes.data_as(ip), _fp(flx), _fp(dfl)))
        return dict(source=src, ns=ns, radiance=rad, nr=nr, fluxes=flx, dirflux=dfl)

    @property
    def fluxes(self) -> dict:
        """Hemispheric fluxes on the base grid: flux_down, flux_up,
        flux_direct shaped [nx1, ny1, nz] (at3d/solver.py:1148-1200)."""
        s = self.sizes
        st = self.export_state()
        shp = (s["nx1"], s["ny1"], s["nz"])
        return {"flux_down": st["fluxes"][:, 0].reshape(shp), "flux_up": st["fluxes"][:, 1].reshape(shp),
                "flux_direct": st["dirflux"].reshape(shp)}

    @property
    def spherical_harmonics(self) -> dict:
        """Mean intensity and net flux vector (Fx, Fy, Fz) on the base grid,
        [nx1, ny1, nz] each (RTE.spherical_harmonics, at3d/solver.py:1039-1129,
        through COMPUTE_SH; the extra root-mean-square term of HIGHORDERRAD
        solves is not included)."""
        s = self.sizes
        st = self.export_state()
        p = self.problem
        sh = compute_sh(st["radiance"], st["dirflux"], p.solarmu, p.solaraz, p.srctype, s["mm"])
        shp = (s["nx1"], s["ny1"], s["nz"])
        return {"mean_intensity": sh[0].reshape(shp), "Fx": sh[1].reshape(shp), "Fy": sh[2].reshape(shp),
                "Fz": sh[3].reshape(shp)}

    @property
    def net_flux_divergence(self) -> dict:
        """The net flux divergence on the base grid, [nx1, ny1, nz]
        (RTE.net_flux_divergence, at3d/solver.py:1207-1260): the solved
        radiance's mean term and direct beam from the device, the absorption
        and emission of the medium from the host plan."""
        s = self.sizes
        st = self.export_state()
        n = s["npts"]
        absorb = np.zeros(n, np.float32); emit = np.zeros(n, np.float32)
        _check(self._h, _lib.lib().shdom_point_absorption(self._h, _fp(absorb), _fp(emit)))
        p = self.problem
        nfd = compute_netfluxdiv(st["radiance"], st["dirflux"], absorb, emit, p.solarmu, p.srctype)
        return {"net_flux_div": nfd.reshape(s["nx1"], s["ny1"], s["nz"])}

    @property
    def solution_accuracy(self) -> float:
        return float(self.problem.params.solution_accuracy)

    @property
    def num_iterations(self) -> int:
        """Iterations of the current solution (RTE.num_iterations)."""
        return int(self.sizes["iters"])

    def _property_shape(self):
        sp = self.problem.species[0]
        return tuple(np.asarray(sp.extinction).shape)

    def min_optical_path(self, sensor: dict, deltam_scaled_path: bool = False, do_all: bool = False):
        """HostPlan.min_optical_path of this solver's problem (planned on the
        host again; no GPU work)."""
        return HostPlan(self.problem).min_optical_path(sensor, deltam_scaled_path, do_all)

    def optical_path(self, sensor: dict, deltam_scaled_path: bool = False) -> dict:
        """The extinction integrated along each ray of ``sensor`` ('ray_x',
        'ray_y', 'ray_z', 'ray_mu', 'ray_phi'), stored in it as
        'optical_path' (or 'optical_path_deltam' with the delta-M scaled
        extinction) (RTE.optical_path, at3d/solver.py:793-867; OPTICAL_DEPTH).
        Computed on the host from the solver's medium, before or after a
        solve."""
        return _optical_path(lambda *a: _lib.lib().shdom_optical_path(self._h, *a), self._h, sensor,
                             deltam_scaled_path)

    @staticmethod
    def _ray_arrays(x, y, z, mu, phi):
        return (np.ascontiguousarray(x, np.float32), np.ascontiguousarray(y, np.float32),
                np.ascontiguousarray(z, np.float32), np.ascontiguousarray(mu, np.float64),
                np.ascontiguousarray(phi, np.float64))

    def levis_gradient(self, rays, measurements, species: int = 0):
        """Levis approximate gradient of the L2 cost 0.5*sum (I - m)^2 of
        one-ray pixels with respect to the extinction and albedo of
        `species` on the property grid (LEVISAPPROX_GRADIENT, adjoint
        branch).  Returns (gradient [npx, npy, npz, 2], cost, radiances)."""
        x, y, z, mu, phi = self._ray_arrays(*rays)
        meas = np.ascontiguousarray(measurements, np.float32)
        shp = self._property_shape()
        grad = np.zeros(int(np.prod(shp)) * 2, np.float64)
        out = np.zeros(len(x), np.float32)
        cost = C.c_double(0)
        dp = C.POINTER(C.c_double)
        _check(self._h, _lib.lib().shdom_levis_gradient(
            self._h, int(species), len(x), _fp(x), _fp(y), _fp(z), mu.ctypes.data_as(dp), phi.ctypes.data_as(dp),
            _fp(meas), grad.ctypes.data_as(dp), C.byref(cost), _fp(out)))
        return grad.reshape(shp + (2,)), float(cost.value), out

    def levis_adjoint(self, rays, weights, species: int = 0) -> np.ndarray:
        """Levis gradient of sum_r w_r I_r for given ray weights (the
        vector-Jacobian product of the rendered radiances): [npx, npy, npz, 2]."""
        x, y, z, mu, phi = self._ray_arrays(*rays)
        w = np.ascontiguousarray(weights, np.float64)
        shp = self._property_shape()
        grad = np.zeros(int(np.prod(shp)) * 2, np.float64)
        dp = C.POINTER(C.c_double)
        _check(self._h, _lib.lib().shdom_levis_adjoint(
            self._h, int(species), len(x), _fp(x), _fp(y), _fp(z), mu.ctypes.data_as(dp), phi.ctypes.data_as(dp),
            w.ctypes.data_as(dp), grad.ctypes.data_as(dp)))
        return grad.reshape(shp + (2,))

    def levis_adjoint_device(self, rays_dev, weights_ptr: int, grad_ptr: int, species: int = 0, stream: int = 0):
        """Device-resident form of ``levis_adjoint``: ``rays_dev`` holds the
        device pointers (x, y, z float32; mu, phi float64) and the number of
        rays, ``weights_ptr`` a float64 device array of ray weights and
        ``grad_ptr`` a float64 device array [npx*npy*npz*2] for the result;
        ordered on ``stream`` (a CUDA stream handle, 0 = legacy default)."""
        (x, y, z, mu, phi), nrays = rays_dev
        args = [C.c_void_p(v) for v in (x, y, z, mu, phi, weights_ptr, grad_ptr, stream)]
        _check(self._h, _lib.lib().shdom_levis_adjoint_device(self._h, int(species), int(nrays), *args))

    def species_properties(self, species: int = 0):
        """(extinction, ssalb) of one species on the property grid, as solved."""
        sp = self.problem.species[species]
        return np.asarray(sp.extinction, np.float32), np.asarray(sp.ssalb, np.float32)

    def update_species(self, species: int, extinction=None, ssalb=None):
        """Replace the extinction and/or single-scattering albedo of one
        species (property grid) and rebuild the device state for the new
        medium (the grid geometry is reused); the solution is reset and must
        be solved again.  This is the step an inversion makes between
        iterates (the reference builds a new medium and re-solves)."""
        import dataclasses
        sp = self.problem.species[species]
        shp = np.asarray(sp.extinction).shape
        ext = sp.extinction if extinction is None else np.ascontiguousarray(extinction, np.float32).reshape(shp)
        alb = sp.ssalb if ssalb is None else np.ascontiguousarray(ssalb, np.float32).reshape(shp)
        if np.any(ext < 0) or np.any(alb < 0) or np.any(alb > 1):
            raise ValueError("extinction must be >= 0 and ssalb within [0, 1]")
        species_list = list(self.problem.species)
        species_list[species] = dataclasses.replace(sp, extinction=ext, ssalb=alb)
        self.problem = dataclasses.replace(self.problem, species=species_list, _keep=[])
        modes = (getattr(self, "_sweep_mode", None), getattr(self, "_transform_mode", None))
        self.close()
        self._create(getattr(self, "_device", 0))
        if modes[0]:
            self.set_sweep_mode(modes[0])
        if modes[1]:
            self.set_transform_mode(modes[1])

    def set_sweep_mode(self, mode: str):
        """'persistent' (one cooperative kernel per hemisphere; default),
        'per_level' (one launch per wavefront level; for solves that run
        concurrently on one device), 'graph' (per-level launches, each
        iteration replayed from a captured CUDA graph) or 'levels_only'
        ('persistent' with the plane march turned off).  Hemispheres that
        the plane march can sweep use it in the first three modes."""
        modes = {"persistent": 0, "per_level": 1, "graph": 2, "levels_only": 3}
        if mode not in modes:
            raise ValueError(f"sweep mode must be one of {sorted(modes)}")
        _check(self._h, _lib.lib().shdom_set_sweep_mode(self._h, modes[mode]))
        self._sweep_mode = mode

    @property
    def sweep_mode(self) -> str:
        return getattr(self, "_sweep_mode", "persistent")

    TRANSFORM_MODES = {"tf32x3": 0, "tf32": 1, "fp32": 2}

    def set_transform_mode(self, mode: str):
        """Arithmetic of the SH <-> DO transforms: 'tf32x3' (tensor cores,
        FP32-level accuracy; default), 'tf32' (tensor cores, one TF32
        product) or 'fp32' (CUDA-core factorized transforms)."""
        if mode not in self.TRANSFORM_MODES:
            raise ValueError(f"transform mode must be one of {sorted(self.TRANSFORM_MODES)}")
        _check(self._h, _lib.lib().shdom_set_transform_mode(self._h, self.TRANSFORM_MODES[mode]))
        self._transform_mode = mode

    def set_transform_wait_limit(self, limit: int):
        """Polls of each tensor-core pipeline wait before a transform gives
        up and reports "pipeline wait expired" (the solve raises SHDOMError;
        the handle stays usable).  A negative limit restores the default; 0
        makes every transform give up at its first wait, to test that path."""
        _check(self._h, _lib.lib().shdom_set_transform_wait_limit(self._h, int(limit)))

    def timings(self) -> np.ndarray:
        t = np.zeros(5, np.float32)
        _check(self._h, _lib.lib().shdom_last_timings(self._h, _fp(t)))
        return t

    def sweep_timings(self) -> dict:
        """Device ms of the sweep's parts over the last solve: 'prep' (phase 1
        beside the source pass), 'levels' (the level pass), and the number of
        hemisphere sweeps timed."""
        t = np.zeros(2, np.float32)
        n = np.zeros(2, np.int32)
        _check(self._h, _lib.lib().shdom_sweep_timings(self._h, _fp(t), n.ctypes.data_as(C.POINTER(C.c_int))))
        return {"prep": float(t[0]), "levels": float(t[1]), "sweeps": int(n[1])}

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().shdom_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
