"""Particle size distributions sampled on the radii of a Mie table, and
look-up grids of them over distribution parameters.

Mirrors at3d.size_distribution (at3d/size_distribution.py): ``gamma`` (:26),
``lognormal`` (:104) and ``get_size_distribution_grid`` (:182), with the
distributions of MAKE_SIZE_DIST / DO_SIZE_DIST
(src/polarized/make_mie_table.f90:512-650):

* gamma:      n(r) = a r^alpha exp(-b r), b = (alpha + 3)/re;
* lognormal:  n(r) = (a/r) exp(-(ln(r/b))^2 / (2 alpha^2)), b = re exp(-2.5 alpha^2);
* each radius carries the width dr_j = sqrt(r_j r_{j+1}) - sqrt(r_j r_{j-1})
  (the end radii use themselves as the missing neighbour);
* the number densities [cm^-3] are scaled so that the liquid water content
  sum 1e-6 rho n_j (4 pi/3) r_j^3 is 1 g/m^3 (rho the particle density in
  g/cm^3); the constant ``a`` cancels in this scaling and is not formed;
* the true effective radius sum n r^3 / sum n r^2 of the discrete
  distribution differs from ``re``; as the reference does, the parameter is
  bracketed (up to 8 multiplications by re/true_re) and bisected until the
  true effective radius is within 0.1 % of the requested one, and a request
  that cannot be bracketed is an error.

The densities are computed in double precision (the reference stores them in
single precision).  There is no xarray here: a grid is a
:class:`SizeDistributionGrid` with the same fields.
"""
from __future__ import annotations

import math
import typing
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

_TOL = 0.001          # fractional tolerance on the effective radius (MAKE_SIZE_DIST TOL)
_NORMALIZATIONS = ("density", "geometric_extinction", "number_concentration")


def _widths(radii: np.ndarray) -> np.ndarray:
    r = np.asarray(radii, np.float64)
    up = np.concatenate([r[1:], r[-1:]])
    dn = np.concatenate([r[:1], r[:-1]])
    return np.sqrt(r * up) - np.sqrt(r * dn)


def _shape(distflag: str, radii: np.ndarray, dr: np.ndarray, re: float, alpha: float) -> np.ndarray:
    """Unnormalised n_j = n(r_j) dr_j, computed in logarithms (large gamma
    shape parameters overflow the plain form)."""
    r = radii
    if distflag == "G":
        b = (alpha + 3.0) / re
        logn = alpha * np.log(r) - b * r
    elif distflag == "L":
        b = re * math.exp(-2.5 * alpha * alpha)
        logn = -np.log(r) - 0.5 * np.log(r / b) ** 2 / (alpha * alpha)
    else:
        raise ValueError(f"unknown distribution flag '{distflag}'")
    logn = logn - logn.max()
    return np.exp(logn) * dr


def _do_size_dist(distflag, pardens, radii, dr, re, alpha):
    """DO_SIZE_DIST (make_mie_table.f90:589-650): densities scaled to
    1 g/m^3 of condensate, and the true effective radius."""
    nd = _shape(distflag, radii, dr, re, alpha)
    lwc = np.sum(1.0e-6 * pardens * nd * (4.0 * math.pi / 3.0) * radii ** 3)
    nd = nd / lwc
    true_re = float(np.sum(nd * radii ** 3) / np.sum(nd * radii ** 2))
    return nd, true_re


def make_size_dist(distflag: str, pardens: float, radii, reff: float, alpha: float) -> np.ndarray:
    """MAKE_SIZE_DIST (make_mie_table.f90:512-585): the distribution whose
    discrete effective radius is within 0.1 % of ``reff``."""
    radii = np.asarray(radii, np.float64)
    dr = _widths(radii)
    nd, true_re = _do_size_dist(distflag, pardens, radii, dr, reff, alpha)
    if abs(true_re - reff) < _TOL * reff:
        return nd
    f = reff / true_re
    if true_re < reff:
        lo, hi = reff, f * reff
        i = 0
        true_re = reff / f
        while true_re <= reff and i < 8:
            hi = f * hi
            i += 1
            nd, true_re = _do_size_dist(distflag, pardens, radii, dr, hi, alpha)
        if true_re <= reff:
            raise ValueError(f"MAKE_SIZE_DIST: effective radius cannot be achieved {reff} {true_re} {alpha}")
    else:
        hi, lo = reff, f * reff
        i = 0
        true_re = reff / f
        while true_re >= reff and i < 8:
            lo = f * lo
            i += 1
            nd, true_re = _do_size_dist(distflag, pardens, radii, dr, lo, alpha)
        if true_re >= reff:
            raise ValueError(f"MAKE_SIZE_DIST: effective radius cannot be achieved {reff} {true_re} {alpha}")
    for _ in range(200):
        if abs(true_re - reff) <= _TOL * reff:
            break
        mid = 0.5 * (lo + hi)
        nd, true_re = _do_size_dist(distflag, pardens, radii, dr, mid, alpha)
        if true_re < reff:
            lo = mid
        else:
            hi = mid
    else:
        raise ValueError(f"MAKE_SIZE_DIST: bisection did not reach {reff} (at {true_re})")
    return nd


def _normalize(number_density: np.ndarray, radii, normalization: str) -> np.ndarray:
    if normalization == "geometric_extinction":
        r = np.atleast_1d(np.asarray(radii, np.float64))[:, None]
        return number_density / (1e-3 * (2 * number_density * np.pi * r ** 2).sum(axis=0))
    if normalization == "number_concentration":
        return number_density / number_density.sum(axis=0)
    if normalization == "density":
        return number_density
    raise ValueError(f"Invalid `normalization` argument '{normalization}'")


def _multi(distflag, radii, reff, alpha, particle_density, normalization):
    radii = np.atleast_1d(np.asarray(radii, np.float64))
    nd = np.zeros((radii.size, len(reff)))
    for k, (re, al) in enumerate(zip(reff, alpha)):
        nd[:, k] = make_size_dist(distflag, particle_density, radii, float(re), float(al))
    return _normalize(nd, radii, normalization).astype(np.float32)


def gamma(radii, reff, veff=None, alpha=None, particle_density=1.0, normalization="density"):
    """Gamma size distribution n(r) ~ r^alpha exp(-(alpha+3) r/reff) at
    ``radii`` [um], one column per (reff, veff or alpha); alpha = 1/veff - 3.
    Returns number densities [len(radii), len(reff)] in cm^-3 per g/m^3 of
    condensate ('density'), per 1/km of geometric extinction
    ('geometric_extinction', extinction efficiency 2) or per particle
    ('number_concentration')."""
    reff = np.atleast_1d(reff)
    if veff is not None:
        veff = np.atleast_1d(veff)
        if len(reff) != len(veff):
            raise ValueError("'reff' and 'veff' must have the same length")
        alpha = 1.0 / veff - 3.0
    elif alpha is not None:
        alpha = np.atleast_1d(alpha)
        if len(reff) != len(alpha):
            raise ValueError("'reff' and 'alpha' must have the same length")
    else:
        raise ValueError("One of 'veff' of 'alpha' must be specified.")
    return _multi("G", radii, reff, alpha, particle_density, normalization)


def lognormal(radii, reff, veff=None, alpha=None, particle_density=1.0, normalization="density"):
    """Log-normal size distribution at ``radii`` [um]; alpha is the standard
    deviation of ln r, alpha = sqrt(ln(veff + 1)).  Units as :func:`gamma`."""
    reff = np.atleast_1d(reff)
    if veff is not None:
        veff = np.atleast_1d(veff)
        if len(reff) != len(veff):
            raise ValueError("'reff' and 'veff' must have the same length")
        alpha = np.sqrt(np.log(veff + 1.0))
    elif alpha is not None:
        alpha = np.atleast_1d(alpha)
        if len(reff) != len(alpha):
            raise ValueError("'reff' and 'alpha' must have the same length")
    else:
        raise ValueError("One of 'veff' of 'alpha' must be specified.")
    return _multi("L", radii, reff, alpha, particle_density, normalization)


@dataclass
class SizeDistributionGrid:
    """Number densities on a grid of distribution parameters: the fields of
    the reference's size-distribution Dataset (``number_density`` with
    dimensions ('radius', parameter names...))."""
    radius: np.ndarray                         # [nradius] um
    number_density: np.ndarray                 # [nradius, *grid] cm^-3
    coords: "OrderedDict[str, np.ndarray]"     # parameter name -> 1-D coordinate
    attrs: dict = field(default_factory=dict)

    @property
    def dims(self) -> list:
        return ["radius"] + list(self.coords)


def _coordinate(parameter) -> np.ndarray:
    if isinstance(parameter, np.ndarray):
        if parameter.ndim != 1:
            raise ValueError("a parameter given as an array must be 1-D")
        return parameter
    if "coords" in parameter:
        return np.asarray(parameter["coords"])
    if "coord" in parameter:
        return np.asarray(parameter["coord"])
    if parameter["spacing"] == "logarithmic":
        return np.logspace(np.log10(parameter["coord_min"]), np.log10(parameter["coord_max"]),
                           parameter["npoints"])
    if parameter["spacing"] == "linear":
        return np.linspace(parameter["coord_min"], parameter["coord_max"], parameter["npoints"])
    raise NotImplementedError(f"spacing '{parameter['spacing']}'")


def get_size_distribution_grid(radii, size_distribution_function=gamma, particle_density=1.0,
                               radius_units="micron", **size_distribution_parameters) -> SizeDistributionGrid:
    """Number densities of ``size_distribution_function`` at ``radii`` on the
    grid spanned by the named parameters (get_size_distribution_grid,
    at3d/size_distribution.py:182-310).  Each parameter is a dict with
    coord_min, coord_max, npoints and spacing ('logarithmic' or 'linear') --
    or 'coords' with the exact points -- or a 1-D array of the points."""
    names, coords = [], []
    for name, parameter in size_distribution_parameters.items():
        names.append(name)
        coords.append(_coordinate(parameter))
    mesh = np.meshgrid(*coords, indexing="ij")
    params = OrderedDict((n, g.ravel()) for n, g in zip(names, mesh))
    radii = np.asarray(radii)
    nd = size_distribution_function(radii, **params, particle_density=particle_density)
    if np.any(np.isnan(nd)) or np.any(nd < 0.0):
        raise ValueError(f"size_distribution_function: {size_distribution_function} produced NaN or "
                         "negative values when being evaluated on grid of parameters.")
    shape = [radii.size] + [c.size for c in coords]
    attrs = OrderedDict()
    for name, parameter in size_distribution_parameters.items():
        if isinstance(parameter, typing.Dict):
            for k, v in parameter.items():
                attrs[f"{name}_{k}"] = v
    attrs["distribution_type"] = size_distribution_function.__name__
    attrs["radius_units"] = f"radius units [{radius_units}]"
    return SizeDistributionGrid(radius=radii, number_density=nd.reshape(shape),
                                coords=OrderedDict(zip(names, coords)), attrs=attrs)
