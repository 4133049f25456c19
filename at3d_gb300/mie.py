"""Mie scattering tables: the monodisperse table over radii and the
polydisperse table over size-distribution parameters.

Mirrors at3d.mie (at3d/mie.py): ``get_mono_table`` (:46-121, computing as
``_compute_table`` :123-270 does) and ``get_poly_table`` (:365-460).

* The radius grid is GET_NSIZE / GET_SIZES
  (src/polarized/make_mie_table.f90:232-281) in single precision: from
  0.02 x the minimum effective radius, steps of
  min(max(0.01, 0.03 sqrt(x)) lambda/2pi, 0.002 x the maximum radius).
* The band centre is GET_CENTER_WAVELEN (:285-324): the Planck-weighted
  mean wavelength (5800 K below 3 um, 270 K above 5 um, flat between),
  rounded to 1 nm; a monochromatic band is its own centre.
* The Legendre limit is round(2 (x + 4 x^0.3334 + 2)) at the largest size
  parameter.
* The single-scattering properties come from the library's Lorenz-Mie
  routine (``shdom_mie_mono``), computed on the host in double precision.
  Band averaging (``wavelength_averaging``) sums them over wavelengths
  lambda1, lambda1 + resolution, ... <= lambda2 with Planck weights, as
  COMPUTE_MIE_ALL_SIZES (:381-482) does with avgflag 'A'.
* The poly table is GET_POLY_TABLE (:953-997): extinction = 0.001 sum n_j
  ext_j [1/km per g/m^3], albedo = sum n_j sca_j / sum n_j ext_j, and
  legcoef = sum n_j leg_j / sum n_j sca_j, whose a1_0 must be 1 to 1e-4;
  nleg is the last l with a1_l > 0.5e-5.  Sums are in double precision.

The refractive index of water is a tabulated function of wavelength and
temperature in the reference (REFWAT, src/polarized/indexwatice.f); that
table is not part of this package, so 'Water' takes the index from
``refractive_index`` (a complex number n - ik, or a callable of wavelength
returning one) and raises without it.  'Aerosol' is as in the reference.
Tables are saved and loaded as .npz files (the reference uses netCDF).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

STOKES_INDEX = ("P11", "P22", "P33", "P44", "P12", "P34")


def _f32(v):
    return np.float32(v)


def get_center_wavelen(wavelen1: float, wavelen2: float) -> float:
    """Planck-weighted centre of a band [um] (GET_CENTER_WAVELEN)."""
    w1, w2 = _f32(wavelen1), _f32(wavelen2)
    if w1 == w2:
        return float(w1)
    cen = _f32(0.5) * (w1 + w2)
    bbtemp = 5800.0 if cen < 3.0 else (270.0 if cen > 5.0 else -1.0)
    dw = min(cen / _f32(100.0), _f32(0.1) * abs(w2 - w1))
    sump = sumw = _f32(0.0)
    wave = w1
    while wave <= w2:
        planck = _f32(1.0) if bbtemp < 0 else _f32((1.19e8 / wave ** 5) / (np.exp(1.439e4 / (wave * bbtemp)) - 1))
        sump = _f32(sump + planck)
        sumw = _f32(sumw + planck * wave)
        wave = _f32(wave + dw)
    return float(_f32(0.001) * np.rint(_f32(1000) * sumw / sump))


def _planck_weight(wave: float, bbtemp: float) -> float:
    if bbtemp < 0:
        return 1.0
    return (1.19e8 / wave ** 5) / (np.exp(1.439e4 / (wave * bbtemp)) - 1.0)


def get_sizes(minimum_effective_radius: float, max_integration_radius: float, wavelength: float) -> np.ndarray:
    """Radii [um] of the monodisperse table (GET_NSIZE and GET_SIZES, single precision)."""
    twopi = _f32(2.0) * _f32(np.arccos(_f32(-1.0)))
    wl = _f32(wavelength)
    rad = _f32(0.02) * _f32(minimum_effective_radius)
    maxr = _f32(max_integration_radius)
    delmax = _f32(0.002) * maxr
    radii = [rad]
    while rad < maxr:
        x = twopi * rad / wl
        delx = max(_f32(0.01), _f32(0.03) * _f32(x ** _f32(0.5)))
        rad = _f32(rad + min(_f32(delx * wl / twopi), delmax))
        radii.append(rad)
    return np.asarray(radii, np.float32)


def maximum_legendre(max_integration_radius: float, wavelength: float) -> int:
    """Legendre limit of a table: round(2 (x + 4 x^0.3334 + 2)) at the largest radius."""
    xmax = 2 * np.pi * max_integration_radius / wavelength
    return int(np.round(2.0 * (xmax + 4.0 * xmax ** 0.3334 + 2.0)))


@dataclass
class MonoTable:
    """Monodisperse Mie table: the fields of the reference's mono-table Dataset."""
    radius: np.ndarray            # [nsize] um
    extinction: np.ndarray        # [nsize] um^2 (cross section)
    scatter: np.ndarray           # [nsize] um^2
    nleg: np.ndarray              # [nsize]
    legendre: np.ndarray          # [6, maxleg+1, nsize]: (stokes_index, legendre_index, radius)
    attrs: dict = field(default_factory=dict)
    stokes_index: tuple = STOKES_INDEX

    def save(self, path: str) -> None:
        np.savez_compressed(path, radius=self.radius, extinction=self.extinction, scatter=self.scatter,
                            nleg=self.nleg, legendre=self.legendre, attrs=np.array(repr(self.attrs)))

    @classmethod
    def load(cls, path: str) -> "MonoTable":
        import ast
        with np.load(path, allow_pickle=False) as z:
            attrs = ast.literal_eval(str(z["attrs"]))
            return cls(radius=z["radius"], extinction=z["extinction"], scatter=z["scatter"], nleg=z["nleg"],
                       legendre=z["legendre"], attrs=attrs)


def mie_mono(wavelength: float, refractive_index: complex, radii, maxleg: int, n_threads: int = 0):
    """Single-wavelength Lorenz-Mie properties of spheres of ``radii`` [um]:
    (extinction, scatter, nleg, legendre [6, maxleg+1, nsize]), as
    COMPUTE_MIE_ALL_SIZES with avgflag 'C'.  ``refractive_index`` is n - ik."""
    from . import _lib
    lib = _lib.lib()
    radii = np.ascontiguousarray(radii, np.float32)
    n = radii.size
    ext = np.zeros(n, np.float32)
    sca = np.zeros(n, np.float32)
    nleg = np.zeros(n, np.int32)
    leg = np.zeros((n, maxleg + 1, 6), np.float32)
    m = complex(refractive_index)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rc = lib.shdom_mie_mono(float(wavelength), m.real, m.imag, n, fp(radii), int(maxleg), int(n_threads),
                            fp(ext), fp(sca), nleg.ctypes.data_as(C.POINTER(C.c_int)), fp(leg))
    if rc != 0:
        raise ValueError(lib.shdom_last_error(None).decode())
    return ext, sca, nleg, np.ascontiguousarray(leg.transpose(2, 1, 0))


def _index_at(refractive_index, wavelength):
    return complex(refractive_index(wavelength) if callable(refractive_index) else refractive_index)


def _compute_table(particle_type, wavelength_band, minimum_effective_radius, max_integration_radius,
                   wavelength_averaging, wavelength_resolution, refractive_index, temperature=283.15,
                   verbose=True, n_threads=0) -> MonoTable:
    wavelen1, wavelen2 = wavelength_band
    if wavelen1 > wavelen2:
        raise ValueError("wavelen1 must be <= wavelen2")
    wavelencen = get_center_wavelen(wavelen1, wavelen2)
    if particle_type == "Water":
        if refractive_index is None:
            raise ValueError("the tabulated refractive index of water is not part of this package: pass "
                             "refractive_index (n - ik, or a callable of wavelength) for 'Water'")
        source = "user_input"
    elif particle_type == "Aerosol":
        if refractive_index is None:
            raise AttributeError("A refractive index should be supplied for Aerosol particles")
        source = "user_input"
    else:
        raise AttributeError("Particle type not implemented")
    if not callable(refractive_index) and complex(refractive_index).imag > 0.0:
        raise AttributeError("The refractive index should have a negative imaginary part. ri = n - ik")
    xwave = wavelen1 if wavelength_averaging else wavelencen
    maxleg = maximum_legendre(max_integration_radius, xwave)
    radii = get_sizes(minimum_effective_radius, max_integration_radius, wavelencen)
    if verbose:
        print(f"computing Mie properties of {radii.size} radii ({maxleg} Legendre terms)")
    if not wavelength_averaging:
        ext, sca, nleg, leg = mie_mono(wavelencen, _index_at(refractive_index, wavelencen), radii, maxleg,
                                       n_threads)
    else:
        cen = 0.5 * (wavelen1 + wavelen2)
        bbtemp = 5800.0 if cen < 3.0 else (270.0 if cen > 5.0 else -1.0)
        ext = np.zeros(radii.size)
        sca = np.zeros(radii.size)
        leg = np.zeros((6, maxleg + 1, radii.size))
        nleg = np.ones(radii.size, np.int32)
        sump = 0.0
        wave = _f32(wavelen1)
        while wave <= _f32(wavelen2):
            p = _planck_weight(float(wave), bbtemp)
            sump += p
            e1, s1, n1, l1 = mie_mono(float(wave), _index_at(refractive_index, float(wave)), radii, maxleg,
                                      n_threads)
            ext += p * e1
            sca += p * s1
            leg += p * l1
            nleg = np.maximum(nleg, n1)
            wave = _f32(wave + _f32(wavelength_resolution))
        ext, sca, leg = (ext / sump).astype(np.float32), (sca / sump).astype(np.float32), \
            (leg / sump).astype(np.float32)
    ri = _index_at(refractive_index, wavelencen)
    attrs = OrderedDict(
        particle_type=particle_type, refractive_index=(ri.real, ri.imag),
        refractive_index_source=source, units=["Radius [micron]", "Wavelength [micron]"],
        wavelength_band=tuple(float(w) for w in wavelength_band), wavelength_center=wavelencen,
        wavelength_averaging=str(wavelength_averaging), wavelength_resolution=wavelength_resolution,
        maximum_legendre=maxleg, minimum_effective_radius=minimum_effective_radius,
        maximum_integration_radius=max_integration_radius, temperature=temperature)
    return MonoTable(radius=radii, extinction=ext, scatter=sca, nleg=nleg, legendre=leg, attrs=dict(attrs))


def _same(a, b) -> bool:
    if a is None or isinstance(a, str) or isinstance(b, str):
        return a == b
    a, b = np.atleast_1d(np.asarray(a, float)), np.atleast_1d(np.asarray(b, float))
    return a.shape == b.shape and bool(np.allclose(a, b))


def _load_table(relative_dir, particle_type, wavelength_band, minimum_effective_radius,
                max_integration_radius, wavelength_averaging, wavelength_resolution, temperature=283.15,
                refractive_index=None):
    """A saved table under ``relative_dir`` (a ``*mie_table*.npz`` file)
    whose attributes match the request, or None (at3d/mie.py:272-362)."""
    want = dict(particle_type=particle_type, wavelength_band=tuple(float(w) for w in wavelength_band),
                minimum_effective_radius=minimum_effective_radius,
                maximum_integration_radius=max_integration_radius,
                wavelength_averaging=str(wavelength_averaging), wavelength_resolution=wavelength_resolution,
                temperature=temperature)
    for path in sorted(glob.glob(os.path.join(relative_dir, "*mie_table*.npz"))):
        t = MonoTable.load(path)
        if all(_same(t.attrs.get(k), v) for k, v in want.items()):
            if refractive_index is None or callable(refractive_index):
                return t
            ri = complex(refractive_index)
            if _same(t.attrs.get("refractive_index"), (ri.real, ri.imag)):
                return t
    return None


def get_mono_table(particle_type, wavelength_band, minimum_effective_radius=4.0, max_integration_radius=65.0,
                   wavelength_averaging=False, wavelength_resolution=0.001, refractive_index=None,
                   temperature=283.15, relative_dir=None, verbose=True, n_threads: int = 0) -> MonoTable:
    """Monodisperse Mie table of spheres over the radii the effective-radius
    range needs (get_mono_table, at3d/mie.py:46-121).  ``relative_dir``: a
    folder searched for a saved table with the same parameters before
    computing one.  ``n_threads``: host threads (0 = every core)."""
    table = None
    if relative_dir is not None:
        table = _load_table(relative_dir, particle_type, wavelength_band, minimum_effective_radius,
                            max_integration_radius, wavelength_averaging, wavelength_resolution,
                            temperature=temperature, refractive_index=refractive_index)
    if table is None:
        table = _compute_table(particle_type, wavelength_band, minimum_effective_radius, max_integration_radius,
                               wavelength_averaging, wavelength_resolution, refractive_index,
                               temperature=temperature, verbose=verbose, n_threads=n_threads)
    return table


@dataclass
class PolyTable:
    """Polydisperse table over size-distribution parameters: the fields of
    the reference's poly-table Dataset."""
    coords: "OrderedDict[str, np.ndarray]"   # parameter name -> 1-D coordinate (e.g. reff, veff)
    extinction: np.ndarray                   # [*grid] 1/km per g/m^3 (or per the distribution's unit)
    ssalb: np.ndarray                        # [*grid]
    legcoef: np.ndarray                      # [6, maxleg+1, *grid]
    nleg: np.ndarray                         # [*grid]
    table_index: np.ndarray                  # [*grid] flat index of each grid point
    attrs: dict = field(default_factory=dict)
    stokes_index: tuple = STOKES_INDEX

    @property
    def shape(self) -> tuple:
        return self.extinction.shape


def get_poly_table(size_distribution, mie_mono_table: MonoTable) -> PolyTable:
    """Integrates the mono table over each size distribution of the grid
    (get_poly_table, at3d/mie.py:365-460; GET_POLY_TABLE,
    make_mie_table.f90:953-997).  When the distribution's radii differ from
    the table's, the number densities are interpolated linearly onto the
    table's radii, which must lie within the distribution's radius range."""
    sd_r = np.asarray(size_distribution.radius, np.float64)
    mr = np.asarray(mie_mono_table.radius, np.float64)
    if np.any(mr < sd_r.min()) or np.any(mr > sd_r.max()):
        raise ValueError(f"Values outside of range '[{sd_r.min()}, {sd_r.max()}]' found in variable 'radius'")
    nd = np.asarray(size_distribution.number_density, np.float64).reshape(sd_r.size, -1)
    if sd_r.size != mr.size or np.any(sd_r != mr):
        print("Warning: size_distribution radii differ to mie_mono_table radii. "
              "Interpolating the size distribution onto the Mie table grid.")
        nd = np.stack([np.interp(mr, sd_r, nd[:, k]) for k in range(nd.shape[1])], axis=1)
    ext1 = np.asarray(mie_mono_table.extinction, np.float64)
    sca1 = np.asarray(mie_mono_table.scatter, np.float64)
    leg1 = np.asarray(mie_mono_table.legendre, np.float64)          # [6, L+1, nsize]
    extinct = nd.T @ ext1                                            # [ndist]
    scatter = nd.T @ sca1
    leg = np.einsum("klr,rd->kld", leg1, nd) / scatter               # [6, L+1, ndist]
    bad = np.abs(leg[0, 0] - 1.0) > 1e-4
    if np.any(bad):
        raise ValueError(f"Phase function not normalized: {np.flatnonzero(bad)[:5]} {leg[0, 0][bad][:5]}")
    above = leg[0] > 0.5e-5
    nleg = np.where(above.any(axis=0), leg.shape[1] - 1 - np.argmax(above[::-1], axis=0), 0)
    ssalb = np.where(extinct > 0, scatter / np.where(extinct > 0, extinct, 1.0), 0.0)
    extinct = 0.001 * extinct
    coords = OrderedDict((k, np.asarray(v)) for k, v in size_distribution.coords.items())
    grid = tuple(c.size for c in coords.values()) if coords else (nd.shape[1],)
    table_index = np.arange(int(np.prod(grid))).reshape(grid)
    attrs = dict(size_distribution.attrs)
    attrs.update(mie_mono_table.attrs)
    return PolyTable(coords=coords, extinction=extinct.reshape(grid).astype(np.float32),
                     ssalb=ssalb.reshape(grid).astype(np.float32),
                     legcoef=leg.reshape(leg.shape[:2] + grid).astype(np.float32),
                     nleg=nleg.reshape(grid), table_index=table_index, attrs=attrs)
