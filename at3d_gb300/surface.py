"""Surfaces: Lambertian (at3d.surface.lambertian, at3d/surface.py:28-105)
and bidirectional ones -- RPV_unpolarized (at3d/surface.py:404-480),
wave_fresnel (:106-203) and diner (:204-307) -- with fixed or spatially varying parameters on a
surface grid of spacing (delx, dely)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class LambertianSurface:
    albedo: np.ndarray | float
    ground_temperature: float | np.ndarray = 298.15
    delx: float = 0.0
    dely: float = 0.0

    @property
    def variable(self):
        return np.size(self.albedo) > 1


def lambertian(albedo, ground_temperature=298.15, delx=None, dely=None) -> LambertianSurface:
    """at3d.surface.lambertian (at3d/surface.py:28-105): a fixed surface, or a
    variable one when the albedo or the ground temperature is an array on
    the surface grid [nxsfc, nysfc] of spacing (delx, dely)."""
    a = np.asarray(albedo, np.float32)
    t = np.asarray(ground_temperature, np.float32)
    if np.any(a > 1.0) or np.any(a < 0.0):
        raise ValueError(f"surface albedo should be in [0, 1] not '{albedo}'")
    if a.size > 1 or t.size > 1:
        if delx is None or dely is None:
            raise ValueError("dely and delx must be defined for variable surface parameters.")
        if a.size > 1 and t.size > 1 and np.atleast_2d(a).shape != np.atleast_2d(t).shape:
            raise ValueError("albedo and ground_temperature must have the same shape")
        shape = np.atleast_2d(a if a.size > 1 else t).shape
        a2 = np.broadcast_to(np.atleast_2d(a), shape).astype(np.float32)
        t2 = float(t.reshape(-1)[0]) if t.size == 1 else np.atleast_2d(t).astype(np.float32)
        return LambertianSurface(a2, t2, float(delx), float(dely))
    return LambertianSurface(float(a.reshape(-1)[0]), float(t.reshape(-1)[0]))


@dataclass
class BRDFSurface:
    """A bidirectional surface: ``kind`` 'R' (RPV: rho0, k, theta), 'W'
    (wave-Fresnel: real index, imaginary index, wind speed in m/s) or 'D'
    (Diner: a, k, b, zeta, sigma), with
    ``params`` of shape [nxsfc, nysfc, nparams]."""
    kind: str
    params: np.ndarray
    ground_temperature: float = 298.15
    delx: float = 0.0
    dely: float = 0.0


def _stack(*arrays, delx, dely):
    arrs = [np.atleast_2d(np.asarray(a, np.float32)) for a in arrays]
    shape = np.broadcast_shapes(*[a.shape for a in arrs])
    if any(a.size > 1 and a.shape != shape for a in arrs):
        raise ValueError("all surface parameters must have the same shape")
    par = np.stack([np.broadcast_to(a, shape) for a in arrs], axis=-1).astype(np.float32)
    if par.shape[0] * par.shape[1] > 1 and (delx is None or dely is None):
        raise ValueError("dely and delx must be defined for variable surface parameters.")
    return par, float(delx or 1.0), float(dely or 1.0)


def RPV_unpolarized(RHO0, K, THETA, ground_temperature=298.15, delx=None, dely=None) -> BRDFSurface:
    """Rahman-Pinty-Verstraete BRDF (scalar problems only)."""
    par, dx, dy = _stack(RHO0, K, THETA, delx=delx, dely=dely)
    return BRDFSurface("R", par, float(ground_temperature), dx, dy)


def wave_fresnel(real_refractive_index, imaginary_refractive_index, surface_wind_speed,
                 ground_temperature=298.15, delx=None, dely=None) -> BRDFSurface:
    """Polarized Fresnel reflection of a wind-roughened dielectric surface."""
    par, dx, dy = _stack(real_refractive_index, imaginary_refractive_index, surface_wind_speed,
                         delx=delx, dely=dely)
    return BRDFSurface("W", par, float(ground_temperature), dx, dy)


def diner(A, K, B, ZETA, SIGMA, ground_temperature=298.15, delx=None, dely=None) -> BRDFSurface:
    """Diner et al. (2012) polarized BRDF: modified-RPV volume term (a, k, b)
    plus Fresnel microfacets weighted by zeta, slope spread sigma (uniform
    orientation when sigma <= 0)."""
    par, dx, dy = _stack(A, K, B, ZETA, SIGMA, delx=delx, dely=dely)
    return BRDFSurface("D", par, float(ground_temperature), dx, dy)


def ocean_unpolarized(surface_wind_speed, pigmentation, ground_temperature=298.15, delx=None,
                      dely=None) -> BRDFSurface:
    """The 6S ocean BRDF (at3d/surface.py ocean_unpolarized; src/ocean_brdf.f):
    whitecaps, Cox-Munk sun glint and the Case I water body for a wind
    speed (m/s) and a pigment concentration (mg/m^3); scalar problems only,
    and the solver needs the wavelength."""
    par, dx, dy = _stack(surface_wind_speed, pigmentation, delx=delx, dely=dely)
    return BRDFSurface("O", par, float(ground_temperature), dx, dy)


def ross_li_thick_sparse(f_iso, f_geo, f_vol, hb_ratio=2.0, br_ratio=1.0, ground_temperature=298.15, delx=None,
                         dely=None) -> BRDFSurface:
    """The MODIS RossThick-LiSparse kernel BRDF (at3d/surface.py
    ross_li_thick_sparse; ROSS_THICK_LI_SPARSE): f_iso + f_vol K_vol +
    f_geo K_geo, scalar problems only.  The reference's SURFACE_BRDF calls
    the kernels with h/b = 2 and b/r = 1 whatever the ratios given, and so
    does this one."""
    if hb_ratio != 2.0 or br_ratio != 1.0:
        import warnings
        warnings.warn("the Ross-Li surface uses h/b = 2 and b/r = 1 (as the reference's SURFACE_BRDF)")
    par, dx, dy = _stack(f_iso, f_geo, f_vol, delx=delx, dely=dely)
    return BRDFSurface("M", par, float(ground_temperature), dx, dy)
