"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/shdom_oracle.cpp).

The oracle is a restatement of the reference Fortran path (see the header of
shdom_oracle.cpp for the citations).  Only tests/, __graft_entry__.smoke()
and bench.py's cpu_baseline leg use it; the at3d_gb300 package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        src = os.path.join(_HERE, "shdom_oracle.cpp")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = C.CDLL(path)
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p, C.c_int]
        L.oracle_error.restype = C.c_char_p
        L.oracle_error.argtypes = [C.c_void_p]
        for n in ("oracle_sizes", "oracle_solve", "oracle_init_solution", "oracle_export",
                  "oracle_render", "oracle_grid", "oracle_angles", "oracle_levis_gradient",
                  "oracle_frozen_render", "oracle_set_render_options", "oracle_levis_adjoint",
                  "oracle_levis_adjoint_phase", "oracle_frozen_render_phase", "oracle_tree"):
            getattr(L, n).restype = C.c_int
        L.oracle_destroy.argtypes = [C.c_void_p]
        _LIB = L
    return _LIB


def _p(a, t=C.c_float):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """One RTE problem solved on the CPU by the oracle (fp64=False mirrors
    the reference's REAL arithmetic, fp64=True is the FP64 oracle)."""

    def __init__(self, problem, fp64: bool = False):
        self._lib = lib()
        self._problem = problem
        st = problem.to_struct()
        self._h = self._lib.oracle_create(C.byref(st), int(fp64))
        err = self._lib.oracle_error(self._h)
        if err:
            raise RuntimeError(err.decode())
        self.sizes = self._sizes()

    def _sizes(self):
        out = np.zeros(16, np.int32)
        self._lib.oracle_sizes(C.c_void_p(self._h), _p(out, C.c_int))
        keys = ["npts", "nlm", "nmu", "nang", "ncells", "nx1", "ny1", "nz", "bcflag", "ipflag", "iters", "ml", "mm",
                "nstokes"]
        return dict(zip(keys, [int(v) for v in out[:len(keys)]]))

    def solve(self, maxiter: int, verbose: bool = False):
        sc = C.c_float(0)
        rc = self._lib.oracle_solve(C.c_void_p(self._h), int(maxiter), int(verbose), C.byref(sc))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        self.sizes = self._sizes()
        return self.sizes["iters"], float(sc.value)

    def init_solution(self):
        if self._lib.oracle_init_solution(C.c_void_p(self._h)):
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())

    def export(self):
        n, nlm, nst = self.sizes["npts"], self.sizes["nlm"], self.sizes["nstokes"]
        shape = (n, nlm) if nst == 1 else (n, nst, nlm)
        src = np.zeros(shape, np.float32); rad = np.zeros(shape, np.float32)
        ns = np.zeros(n, np.int32); nr = np.zeros(n, np.int32)
        flx = np.zeros((n, 2), np.float32); dfl = np.zeros(n, np.float32)
        self._lib.oracle_export(C.c_void_p(self._h), _p(src), _p(ns, C.c_int), _p(rad), _p(nr, C.c_int),
                                _p(flx), _p(dfl))
        return dict(source=src, ns=ns, radiance=rad, nr=nr, fluxes=flx, dirflux=dfl)

    def render(self, x, y, z, mu, phi, nthreads: int = 1, single_scatter: bool = False, nosurface: bool = False):
        self._lib.oracle_set_render_options(C.c_void_p(self._h), int(single_scatter), int(nosurface))
        x = np.ascontiguousarray(x, np.float32); y = np.ascontiguousarray(y, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        mu = np.ascontiguousarray(mu, np.float64); phi = np.ascontiguousarray(phi, np.float64)
        nst = self.sizes["nstokes"]
        out = np.zeros(len(x) if nst == 1 else (len(x), nst), np.float32)
        rc = self._lib.oracle_render(C.c_void_p(self._h), len(x), _p(x), _p(y), _p(z), _p(mu, C.c_double),
                                     _p(phi, C.c_double), _p(out), int(nthreads))
        self._lib.oracle_set_render_options(C.c_void_p(self._h), 0, 0)
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return out

    @staticmethod
    def _rays(x, y, z, mu, phi):
        return (np.ascontiguousarray(x, np.float32), np.ascontiguousarray(y, np.float32),
                np.ascontiguousarray(z, np.float32), np.ascontiguousarray(mu, np.float64),
                np.ascontiguousarray(phi, np.float64))

    def levis_gradient(self, species: int, rays, measurements, nthreads: int = 1):
        """Levis approximate gradient of the L2 cost (one ray per pixel) with
        respect to the extinction and albedo of `species` on the property
        grid: (gradient [npx*npy*npz, 2], cost, radiances)."""
        x, y, z, mu, phi = self._rays(*rays)
        meas = np.ascontiguousarray(measurements, np.float32)
        pb = self._problem
        ng = pb.species[0].extinction.size
        grad = np.zeros((ng, 2), np.float64)
        cost = C.c_double(0)
        out = np.zeros(len(x), np.float32)
        rc = self._lib.oracle_levis_gradient(C.c_void_p(self._h), int(species), len(x), _p(x), _p(y), _p(z),
                                             _p(mu, C.c_double), _p(phi, C.c_double), _p(meas),
                                             _p(grad, C.c_double), C.byref(cost), _p(out), int(nthreads))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return grad, float(cost.value), out

    def levis_adjoint(self, species: int, rays, weights, nthreads: int = 1):
        """The adjoint pass with given ray weights w_r: the Levis gradient
        of sum_r w_r I_r, [npx*npy*npz, 2]."""
        x, y, z, mu, phi = self._rays(*rays)
        w = np.ascontiguousarray(weights, np.float64)
        ng = self._problem.species[0].extinction.size
        grad = np.zeros((ng, 2), np.float64)
        rc = self._lib.oracle_levis_adjoint(C.c_void_p(self._h), int(species), len(x), _p(x), _p(y), _p(z),
                                            _p(mu, C.c_double), _p(phi, C.c_double), _p(w, C.c_double),
                                            _p(grad, C.c_double), int(nthreads))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return grad

    def frozen_render(self, species: int, voxel: int, dext: float, dalb: float, rays, nthreads: int = 1):
        """Render with one voxel's extinction / albedo perturbed and the source
        recomputed from the frozen radiance field (the forward model the
        Levis approximation differentiates)."""
        x, y, z, mu, phi = self._rays(*rays)
        out = np.zeros(len(x), np.float32)
        rc = self._lib.oracle_frozen_render(C.c_void_p(self._h), int(species), int(voxel), C.c_float(dext),
                                            C.c_float(dalb), len(x), _p(x), _p(y), _p(z), _p(mu, C.c_double),
                                            _p(phi, C.c_double), _p(out), int(nthreads))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return out

    def levis_adjoint_phase(self, species: int, rays, weights, dleg, diph, nthreads: int = 1):
        """The adjoint pass with a third unknown: the phase function moved
        along derivative series ``dleg`` [ndphase, nleg+1] (with the 2l+1
        factor), row ``diph`` [npx*npy*npz, maxnmicro] (1-based) at each
        property point (DLEG and DIPHASEP of LEVISAPPROX_GRADIENT).  Returns
        the gradient of sum_r w_r I_r, [npx*npy*npz, 3] (extinction,
        albedo, phase)."""
        x, y, z, mu, phi = self._rays(*rays)
        w = np.ascontiguousarray(weights, np.float64)
        dl = np.ascontiguousarray(np.atleast_2d(dleg), np.float32)
        di = np.ascontiguousarray(diph, np.int32)
        ng = self._problem.species[0].extinction.size
        grad = np.zeros((ng, 3), np.float64)
        rc = self._lib.oracle_levis_adjoint_phase(C.c_void_p(self._h), int(species), len(x), _p(x), _p(y), _p(z),
                                                  _p(mu, C.c_double), _p(phi, C.c_double), _p(w, C.c_double),
                                                  dl.shape[0], dl.shape[1] - 1, _p(dl), _p(di, C.c_int),
                                                  _p(grad, C.c_double), int(nthreads))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return grad

    def frozen_render_phase(self, species: int, voxel: int, eps: float, dleg_row, rays, nthreads: int = 1,
                            dext: float = 0.0, dalb: float = 0.0):
        """frozen_render with one voxel's phase function (its current mixture)
        plus eps x ``dleg_row`` (Legendre series with the 2l+1 factor), and
        its extinction and albedo moved by dext, dalb."""
        x, y, z, mu, phi = self._rays(*rays)
        row = np.ascontiguousarray(dleg_row, np.float32)
        out = np.zeros(len(x), np.float32)
        rc = self._lib.oracle_frozen_render_phase(C.c_void_p(self._h), int(species), int(voxel), C.c_float(eps),
                                                  row.size - 1, _p(row), C.c_float(dext), C.c_float(dalb),
                                                  len(x), _p(x), _p(y), _p(z),
                                                  _p(mu, C.c_double), _p(phi, C.c_double), _p(out), int(nthreads))
        if rc:
            raise RuntimeError(self._lib.oracle_error(C.c_void_p(self._h)).decode())
        return out

    def grid(self):
        n, nc = self.sizes["npts"], self.sizes["ncells"]
        gp = np.zeros((n, 3), np.float32); gptr = np.zeros((nc, 8), np.int32)
        nb = np.zeros((nc, 6), np.int32); cf = np.zeros(nc, np.int16)
        self._lib.oracle_grid(C.c_void_p(self._h), _p(gp), _p(gptr, C.c_int), _p(nb, C.c_int), _p(cf, C.c_short))
        return gp, gptr, nb, cf

    def tree(self):
        """The cell tree of an adaptive grid, [ncells, 2]: parent (-1 for a
        base cell) and first child (0 for an end cell); a neighbour pointer
        v <= -2 in grid() names cell -v - 2, which has children."""
        t = np.zeros((self.sizes["ncells"], 2), np.int32)
        self._lib.oracle_tree(C.c_void_p(self._h), _p(t, C.c_int))
        return t

    def __del__(self):
        try:
            self._lib.oracle_destroy(C.c_void_p(self._h))
        except Exception:
            pass
