"""Optical-property producers the benchmark scenes need.

* :func:`rayleigh_legcoef` -- Rayleigh phase-function Legendre coefficients
  with the King depolarisation factor (RAYLEIGH_PHASE_FUNCTION,
  src/polarized/shdomsub4.f:2350-2386, scalar P11 row).
* :func:`rayleigh_extinction_profile` -- molecular extinction from a
  temperature profile (at3d.rayleigh.compute_extinction,
  at3d/rayleigh.py:139-185, and RAYLEIGH_EXTINCT, src/shdomsub5.f:1457-1490),
  evaluated in single precision like the reference.
* :func:`henyey_greenstein_legcoef` -- a_l = (2l+1) g^l.
* :func:`rayleigh_legcoef6` -- the six Wigner-function expansion elements
  (a1, a2, a3, a4, b1, b2) of the Rayleigh phase matrix with depolarisation
  (RAYLEIGH_PHASE_FUNCTION, src/polarized/shdomsub4.f:2350-2386).
* :func:`gas_species` -- gaseous absorption as a non-scattering species,
  the reference's own route for a 3D gas field (at3d/solver.py:1802-1840).
* :func:`hg_matrix_legcoef6` -- a phase matrix whose I-I element is
  Henyey-Greenstein and whose polarization elements follow the same series
  scaled by a linear depolarisation factor (synthetic polarized medium).
* :func:`table_to_grid` -- optical properties on the grid from microphysics
  through a poly table (at3d.medium.table_to_grid, at3d/medium.py:1927).
* :func:`mix_optical_properties` -- several species as one, with a reduced
  table of mixed phase functions (at3d/medium.py:900).
* :class:`OpticalPropertyGenerator` -- a scatterer's optical properties at
  several wavelengths from its microphysics, by poly-table interpolation or
  exact size distributions (at3d/medium.py:152).
"""
from __future__ import annotations

import numpy as np

from ._abi import Species


def rayleigh_legcoef(wavelength: float) -> np.ndarray:
    """Scalar Rayleigh Legendre series [a_0, a_1, a_2] at ``wavelength`` (um)."""
    a_k, b_k, c_k = 1.0469541, 3.2503153e-04, 3.8622851e-05
    w = np.float32(wavelength)
    fking = np.float32(a_k + b_k / np.float64(w) ** 2 + c_k / np.float64(w) ** 4)
    depol = np.float32(6.0 * (np.float64(fking) - 1.0) / (3.0 + 7.0 * np.float64(fking)))
    delta = np.float32((np.float32(1.0) - depol) / (np.float32(1.0) + np.float32(0.5) * depol))
    return np.array([1.0, 0.0, np.float32(0.5) * delta], np.float32)


def rayleigh_extinction_profile(wavelength: float, zlevels, temperature, surface_pressure: float = 1013.25):
    """Rayleigh extinction [1/km] at each level of a temperature profile."""
    lam = float(wavelength)
    raylcoef = 0.03370 * (surface_pressure / 1013.25) * 0.0021520 * (
        1.0455996 - 341.29061 / lam ** 2 - 0.90230850 * lam ** 2) / \
        (1 + 0.0027059889 / lam ** 2 - 85.968563 * lam ** 2)
    f32 = np.float32
    z = np.asarray(zlevels, f32)
    t = np.asarray(temperature, f32)
    rc = f32(raylcoef)
    pres = f32(surface_pressure)
    ts = t[0]
    lapse = f32(6.5) * f32(0.001)
    pres = f32(pres * (ts / (ts + lapse * z[0] * f32(1000.0))) ** (f32(9.8) / (f32(287.0) * lapse)))
    out = np.zeros(len(z), f32)
    for i in range(len(z) - 1):
        out[i] = rc * pres / t[i]
        dz = f32(1000.0) * (z[i + 1] - z[i])
        lapse = (t[i] - t[i + 1]) / dz
        if abs(lapse) > 0.00001:
            pres = f32(pres * (t[i + 1] / t[i]) ** (f32(9.8) / (f32(287.0) * lapse)))
        else:
            pres = f32(pres * np.exp(f32(-9.8) * dz / (f32(287.0) * t[i])))
    out[-1] = rc * pres / t[-1]
    return out


def henyey_greenstein_legcoef(g: float, nterms: int) -> np.ndarray:
    """Henyey-Greenstein Legendre series a_l = (2l+1) g^l, l = 0..nterms-1."""
    l = np.arange(nterms, dtype=np.float64)
    return ((2 * l + 1) * g ** l).astype(np.float32)


def rayleigh_legcoef6(depol: float) -> np.ndarray:
    """Rayleigh phase matrix [6, 3] for linear depolarisation ratio ``depol``:
    a1 = (1, 0, D/2), a2 = (0, 0, 3D), a4 = (0, 3DD'/2, 0), b1 = (0, 0, sqrt(3/2) D),
    with D = (1-depol)/(1+depol/2), D' = (1-2 depol)/(1-depol)."""
    d = (1.0 - depol) / (1.0 + 0.5 * depol)
    dp = (1.0 - 2.0 * depol) / (1.0 - depol)
    c = np.zeros((6, 3), np.float64)
    c[0, 0] = 1.0
    c[0, 2] = 0.5 * d
    c[1, 2] = 3.0 * d
    c[3, 1] = 1.5 * dp * d
    c[4, 2] = np.sqrt(1.5) * d
    return c.astype(np.float32)


def hg_matrix_legcoef6(g: float, depol: float, nterms: int) -> np.ndarray:
    """[6, nterms] phase matrix: a1 = (2l+1) g^l; a2 = a3 = (1-depol) a1 for
    l >= 2 (the generalized functions of a2, a3 start at l = 2); a4 =
    (1-2 depol) a1; b1 = b2 = 0 (no polarization created by single scattering)."""
    a1 = henyey_greenstein_legcoef(g, nterms).astype(np.float64)
    c = np.zeros((6, nterms), np.float64)
    c[0] = a1
    c[1, 2:] = (1.0 - depol) * a1[2:]
    c[2, 2:] = (1.0 - depol) * a1[2:]
    c[3] = (1.0 - 2.0 * depol) * a1
    return c.astype(np.float32)


def gas_species(gas_absorption, num_stokes: int = 1) -> Species:
    """Gaseous absorption [1/km] on the property grid as a species with
    single-scattering albedo 0 (its phase function is never used)."""
    g = np.asarray(gas_absorption, np.float32)
    if np.any(g < 0):
        raise ValueError("gas_absorption must be non-negative")
    leg = np.zeros((6, 2), np.float32) if num_stokes == 3 else np.zeros(2, np.float32)
    if num_stokes == 3:
        leg[0, 0] = 1.0
    else:
        leg[0] = 1.0
    return Species(extinction=g, ssalb=np.zeros_like(g), legcoef=leg)


def table_to_grid(microphysics, poly_table, inverse_mode: bool = False, num_stokes: int = 1) -> Species:
    """Optical properties on the property grid from microphysics and a poly
    table (table_to_grid, at3d/medium.py:1927-2080).

    ``microphysics``: a mapping with 'density' [npx, npy, npz] (g/m^3, or the
    unit the table's extinction is per) and, for each coordinate of the
    table (e.g. 'reff', 'veff'), an array of the same shape.  Every
    coordinate value must lie strictly inside the table's range.

    * extinction = density x the table's extinction interpolated linearly in
      all coordinates (only the interpolated extinction per unit density
      with ``inverse_mode``);
    * ssalb: linear interpolation;
    * phase functions: the table entry nearest in every coordinate; the
      entries used are gathered into the species' Legendre table and the
      grid holds their 1-based index (``table_index`` [1, npx, npy, npz],
      ``phase_weights`` ones);
    * a table without coordinates gives every point its single entry.

    The Legendre rows are a1 ([ntable, nleg+1]) for a scalar problem, all six
    elements ([ntable, 6, nleg+1]) for ``num_stokes`` = 3."""
    return _poly_to_species(microphysics, poly_table, inverse_mode, num_stokes, strict=True)


def _poly_to_species(microphysics, poly_table, inverse_mode: bool, num_stokes: int, strict: bool) -> Species:
    """table_to_grid's interpolation; ``strict``: coordinates must lie strictly
    inside the table (table_to_grid), else on or inside its bounds (the
    nearest mode of OpticalPropertyGenerator)."""
    from scipy.interpolate import RegularGridInterpolator

    density = np.asarray(microphysics["density"], np.float64)
    if np.any(density < 0) or np.any(~np.isfinite(density)):
        raise ValueError("'density' must be finite and non-negative")
    leg = np.asarray(poly_table.legcoef, np.float64)
    if leg.shape[0] != 6:
        raise ValueError("'stokes_index' dimension of 'legcoef' must have 6 components.")
    if not inverse_mode:
        a0 = leg[0, 0]
        if not np.allclose(a0, 1.0, atol=1e-7):
            raise ValueError("0th Legendre/Wigner Coefficients must be normalized to 1.0")
        if np.any(np.abs(leg[0, 1] / 3.0) > 1.0):
            raise ValueError("Asymmetry Parameter (1st Legendre coefficient divided by 3)is not in the range "
                             "[-1.0, 1.0]")
    names = list(poly_table.coords)
    missing = [n for n in names if n not in microphysics]
    if missing:
        raise KeyError("microphysics dataset is missing variables for interpolation of table onto grid.",
                       *missing)
    if not names:
        ext_eff = np.full(density.shape, float(np.asarray(poly_table.extinction).reshape(-1)[0]))
        ssalb = np.full(density.shape, float(np.asarray(poly_table.ssalb).reshape(-1)[0]))
        rows = leg.reshape(6, leg.shape[1], -1)[..., :1]
        index = np.ones(density.shape, np.int32)
    else:
        axes = [np.asarray(poly_table.coords[n], np.float64) for n in names]
        pts = []
        for n, ax in zip(names, axes):
            v = np.asarray(microphysics[n], np.float64)
            if v.shape != density.shape:
                raise ValueError(f"microphysical variable '{n}' has shape {v.shape}, density {density.shape}")
            outside = (np.any(v <= ax.min()) or np.any(v >= ax.max())) if strict else \
                (np.any(v < ax.min()) or np.any(v > ax.max()))
            if outside:
                raise ValueError(f"Microphysical coordinate '{n}' is not within the range of the mie table.")
            pts.append(v.reshape(-1))
        pts = np.stack(pts, axis=1)
        lin = lambda table: RegularGridInterpolator(axes, np.asarray(table, np.float64), method="linear")(pts)
        ext_eff = lin(poly_table.extinction).reshape(density.shape)
        ssalb = lin(poly_table.ssalb).reshape(density.shape)
        nearest = np.stack([np.abs(ax[None, :] - p[:, None]).argmin(axis=1) for ax, p in zip(axes, pts.T)],
                           axis=1)
        flat = np.ravel_multi_index(tuple(nearest.T), tuple(ax.size for ax in axes))
        used, inverse = np.unique(flat, return_inverse=True)
        rows = leg.reshape(6, leg.shape[1], -1)[..., used]
        index = (inverse.reshape(density.shape) + 1).astype(np.int32)
    extinction = ext_eff if inverse_mode else ext_eff * density
    if np.any(np.isnan(extinction)) or np.any(np.isnan(ssalb)):
        raise ValueError("Unexpected NaN in interpolated optical properties")
    if num_stokes == 3:
        legcoef = np.ascontiguousarray(rows.transpose(2, 0, 1), np.float32)       # [ntable, 6, L+1]
    elif num_stokes == 1:
        legcoef = np.ascontiguousarray(rows[0].T, np.float32)                     # [ntable, L+1]
    else:
        raise ValueError("num_stokes must be 1 or 3")
    return Species(extinction=extinction.astype(np.float32), ssalb=ssalb.astype(np.float32), legcoef=legcoef,
                   table_index=index[None].astype(np.int32),
                   phase_weights=np.ones((1,) + density.shape, np.float32))


def _species_table(sp: Species, num_stokes: int):
    """A species' Legendre rows as [ntable, nleg+1, 6] (scalar rows fill a1),
    its 1-based indices and weights as [nmicro, npts] in x-fastest order."""
    lc = np.asarray(sp.legcoef, np.float32)
    if num_stokes == 3:
        lc = lc.reshape(-1, 6, lc.shape[-1])
        rows = np.ascontiguousarray(lc.transpose(0, 2, 1))
    else:
        lc = np.atleast_2d(lc)
        rows = np.zeros(lc.shape + (6,), np.float32)
        rows[..., 0] = lc
    shape = np.asarray(sp.extinction).shape
    if sp.table_index is None:
        idx = np.ones((1, int(np.prod(shape))), np.int32)
        wt = np.ones((1, idx.shape[1]), np.float32)
    else:
        ti = np.asarray(sp.table_index)
        nm = ti.shape[0]
        idx = ti.reshape((nm,) + shape).transpose(0, 3, 2, 1).reshape(nm, -1).astype(np.int32)
        wt = np.asarray(sp.phase_weights, np.float32).reshape((nm,) + shape).transpose(0, 3, 2, 1).reshape(nm, -1)
    return rows, idx, wt


def mix_optical_properties(*species, asymmetry_tol: float = 0.002, phase_tol: float = 0.01,
                           linear_polarization_tol: float = 0.01, nangles: int = 180, maxnphase=None,
                           maxiter: int = 1, num_stokes: int = 1) -> Species:
    """One species equivalent to the given species on the same grid
    (mix_optical_properties, at3d/medium.py:900-1068): extinctions add,
    the albedo is the scattering-weighted mean, and the phase functions are
    the greedy subset of the library's ``shdom_phase_function_mixing``: each
    point's scattering-weighted mixture is represented by a kept entry whose
    asymmetry, P11 at ``nangles`` angles and P12/P11 are within
    ``asymmetry_tol``, ``phase_tol`` and ``linear_polarization_tol`` of it.
    Points are visited x fastest, as the reference does.  ``maxnphase``
    (default: all input phase functions) bounds the table; with ``maxiter``
    > 1 an overflow retries with the table size extrapolated from the points
    mixed so far.  Where nothing scatters the point takes entry 1 (its
    phase function is never used there).  ``num_stokes``: the row layout of
    the inputs and the result (1: a1 rows, 3: all six elements)."""
    import ctypes as C

    from . import _lib

    if not species:
        raise ValueError("no species to mix")
    shape = np.asarray(species[0].extinction).shape
    for sp in species:
        if np.asarray(sp.extinction).shape != shape or np.asarray(sp.ssalb).shape != shape:
            raise ValueError("species must be on the same grid")
    parts = [_species_table(sp, num_stokes) for sp in species]
    nleg = max(p[0].shape[1] for p in parts) - 1
    nmicro = max(p[1].shape[0] for p in parts)
    npts = int(np.prod(shape))
    tables, offsets = [], []
    for rows, _, _ in parts:
        offsets.append(sum(t.shape[0] for t in tables))
        pad = np.zeros((rows.shape[0], nleg + 1, 6), np.float32)
        pad[:, :rows.shape[1]] = rows
        tables.append(pad)
    table = np.ascontiguousarray(np.concatenate(tables))
    idx = np.ones((len(species), npts, nmicro), np.int32)
    wt = np.zeros((len(species), npts, nmicro), np.float32)
    scat = np.zeros((npts, len(species)), np.float32)
    for k, ((rows, ix, w), sp) in enumerate(zip(parts, species)):
        idx[k, :, :ix.shape[0]] = ix.T + offsets[k]
        wt[k, :, :w.shape[0]] = w.T
        e = np.asarray(sp.extinction, np.float32).transpose(2, 1, 0).reshape(-1)
        a = np.asarray(sp.ssalb, np.float32).transpose(2, 1, 0).reshape(-1)
        scat[:, k] = e * a
    maxn = int(table.shape[0] if maxnphase is None else maxnphase)
    lib = _lib.lib()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    for attempt in range(max(1, int(maxiter))):
        mixed = np.zeros((maxn, nleg + 1, 6), np.float32)
        index = np.zeros(npts, np.int32)
        nphase = np.zeros(1, np.int32)
        fail = np.zeros(1, np.int32)
        rc = lib.shdom_phase_function_mixing(npts, len(species), nmicro, fp(scat), ip(idx), fp(wt), table.shape[0],
                                             nleg, 6, fp(table), float(asymmetry_tol), float(phase_tol),
                                             float(linear_polarization_tol), int(nangles), maxn, fp(mixed),
                                             ip(index), ip(nphase), ip(fail))
        if rc == 0:
            break
        msg = lib.shdom_last_error(None).decode()
        if attempt == max(1, int(maxiter)) - 1 or fail[0] <= 0:
            raise ValueError(msg)
        maxn = int(nphase[0] / fail[0] * npts) + 10
    n = int(nphase[0])
    mixed = mixed[:max(n, 1)]
    mixed[:, 0, 0] = 1.0
    ext = np.sum([np.asarray(sp.extinction, np.float64) for sp in species], axis=0)
    sca = scat.sum(axis=1).reshape(shape[::-1]).transpose(2, 1, 0).astype(np.float64)
    alb = np.where(ext > 0, sca / np.where(ext > 0, ext, 1.0), 0.0)
    index = np.where(index > 0, index, 1).reshape(shape[::-1]).transpose(2, 1, 0)
    legcoef = mixed.transpose(0, 2, 1) if num_stokes == 3 else mixed[:, :, 0]
    return Species(extinction=ext.astype(np.float32), ssalb=alb.astype(np.float32),
                   legcoef=np.ascontiguousarray(legcoef, np.float32),
                   table_index=index[None].astype(np.int32), phase_weights=np.ones((1,) + shape, np.float32))


class OpticalPropertyGenerator:
    """Optical properties of one scatterer at several wavelengths from its
    microphysics (at3d.medium.OpticalPropertyGenerator,
    at3d/medium.py:152-900).

    ``monodisperse_tables``: {key (wavelength): MonoTable};
    ``size_distribution_function``: ``size_distribution.gamma`` or
    ``lognormal`` (called with ``normalization=density_normalization``);
    ``size_distribution_parameters``: the grid of distribution parameters
    (e.g. ``reff={'coord_min': 4, 'coord_max': 25, 'npoints': 30,
    'spacing': 'logarithmic'}``, ``veff=np.array([...])``).

    Calling it with microphysics (a mapping with 'density' and each
    parameter on the property grid) returns {key: Species}:

    * ``interpolation_mode='nearest'``: the poly table of the parameter grid
      (made once per key), extinction and albedo interpolated linearly,
      phase functions from the nearest table entry (the poly table route of
      :func:`table_to_grid`, with the parameter range inclusive);
    * ``'exact'``: a size distribution for each distinct parameter tuple of
      the grid, integrated over the Mie table; when there are more than
      ``maxnphase`` distinct tuples (default: the number of distributions of
      the parameter grid), parameters are turned into tables one at a time
      (those whose bracketing grid points repeat most, first) until the
      bracketing tuples are few enough, and each point mixes the
      distributions at the corners of its bracket with multilinear phase
      weights (``table_index`` and ``phase_weights`` of num_micro = 2^k
      entries).  Parameters left exact must then be uniform over the grid.

    The last call's result is kept and returned again for the same
    microphysics."""

    VALID_INTERPOLATION_MODES = ("exact", "nearest")

    def __init__(self, scatterer_name, monodisperse_tables, size_distribution_function, particle_density=1.0,
                 maxnphase=None, interpolation_mode="exact", density_normalization="density",
                 num_stokes: int = 1, **size_distribution_parameters):
        import functools

        from . import size_distribution as sdmod
        if not isinstance(monodisperse_tables, dict):
            raise TypeError("`monodisperse_tables` should be a dictionary of mie monodisperse tables.")
        if interpolation_mode not in self.VALID_INTERPOLATION_MODES:
            raise ValueError(f"`interpolation_mode` must be in '{self.VALID_INTERPOLATION_MODES}' not "
                             f"'{interpolation_mode}'")
        self.scatterer_name = scatterer_name
        self.interpolation_mode = interpolation_mode
        self.num_stokes = num_stokes
        self._particle_density = particle_density
        self._size_distribution_function = functools.update_wrapper(
            functools.partial(size_distribution_function, normalization=density_normalization),
            size_distribution_function)
        self._monodisperse_tables = monodisperse_tables
        self.size_distribution_parameters = dict(size_distribution_parameters)
        self.size_distribution_grids = {
            key: sdmod.get_size_distribution_grid(table.radius, size_distribution_function=self._size_distribution_function,
                                                  particle_density=particle_density, radius_units="micron",
                                                  **size_distribution_parameters)
            for key, table in monodisperse_tables.items()}
        first = next(iter(self.size_distribution_grids.values()))
        self._names = list(first.coords)
        self._grid_coords = [np.asarray(first.coords[n], np.float64) for n in self._names]
        self._maxnphase = int(np.prod([c.size for c in self._grid_coords])) if maxnphase is None else int(maxnphase)
        self._poly_tables = {}
        self._cache = None

    @property
    def size_distribution_function(self):
        return self._size_distribution_function

    def _check_input(self, microphysics):
        density = np.asarray(microphysics["density"], np.float64)
        if np.any(density < 0) or np.any(~np.isfinite(density)):
            raise ValueError("'density' must be finite and non-negative")
        missing = [n for n in self._names if n not in microphysics]
        if missing:
            raise KeyError("microphysics dataset is missing variables for interpolation of table onto grid.",
                           *missing)
        data = []
        for n, c in zip(self._names, self._grid_coords):
            v = np.asarray(microphysics[n], np.float64)
            if v.shape != density.shape:
                raise ValueError(f"microphysical variable '{n}' has shape {v.shape}, density {density.shape}")
            if np.any(v < c.min()) or np.any(v > c.max()):
                raise ValueError(f"Microphysical coordinate '{n}' is not within the range of the size "
                                 "distribution parameters.")
            data.append(v.reshape(-1))
        return density, np.stack(data) if data else np.zeros((0, density.size))

    def __call__(self, microphysics) -> dict:
        key = {k: np.asarray(v) for k, v in microphysics.items() if k == "density" or k in self._names}
        if self._cache is not None and key.keys() == self._cache[0].keys() and \
                all(np.array_equal(key[k], self._cache[0][k]) for k in key):
            return dict(self._cache[1])
        density, data = self._check_input(microphysics)
        out = {}
        if self.interpolation_mode == "nearest":
            from .mie import get_poly_table
            for k, table in self._monodisperse_tables.items():
                if k not in self._poly_tables:
                    self._poly_tables[k] = get_poly_table(self.size_distribution_grids[k], table)
                out[k] = _poly_to_species(dict(microphysics), self._poly_tables[k], False, self.num_stokes,
                                          strict=False)
        else:
            params, weights, phase_index = self._exact_size_distributions(data)
            for k, table in self._monodisperse_tables.items():
                out[k] = self._exact_species(density, table, params, weights, phase_index)
        self._cache = ({k: v.copy() for k, v in key.items()}, dict(out))
        return out

    def _exact_size_distributions(self, data):
        """Distinct parameter tuples (or the bracketing table tuples), the
        per-point weights [ncorner, npts] and indices into the tuples."""
        import itertools
        nvar, npts = data.shape
        uniq, inv = np.unique(data, axis=1, return_inverse=True)
        inv = np.asarray(inv).reshape(-1)
        if uniq.shape[1] <= self._maxnphase or nvar == 0:
            return ({n: uniq[i] for i, n in enumerate(self._names)}, np.ones((1, npts)), inv[None, :])
        # bracketing grid indices of every point in every parameter, clipped so
        # that a value on the top grid point is bracketed by the last interval
        dig = np.stack([np.clip(np.digitize(data[i], self._grid_coords[i]), 1, self._grid_coords[i].size - 1)
                        for i in range(nvar)])
        flags = np.array(list(itertools.product([-1, 0], repeat=nvar)))          # [ncorner, nvar]
        corners = dig[None] + flags[..., None]                                   # [ncorner, nvar, npts]
        exact_vals, combos = [], []
        for i in range(nvar):
            u, iv = np.unique(data[i], return_inverse=True)
            exact_vals.append(u)
            combos.append(np.asarray(iv).reshape(-1))
        combos = np.repeat(np.stack(combos)[None], flags.shape[0], axis=0)
        ucorn = np.unique(corners, axis=2)
        ratio = np.array([np.unique(ucorn[:, i, :]).size / exact_vals[i].size for i in range(nvar)])
        order = np.argsort(ratio, kind="stable")
        ntab, nuniq = 0, uniq.shape[1]
        if self._maxnphase <= 0:
            ntab = nvar
        while nuniq > self._maxnphase and ntab < nvar:
            idx = order[ntab]
            combos[:, idx, :] = corners[:, idx, :]
            nuniq = np.unique(combos.transpose(0, 2, 1).reshape(-1, nvar), axis=0).shape[0]
            ntab += 1
        if nuniq > self._maxnphase:
            raise ValueError(f"All variables are represented using tables but `maxnphase`='{self._maxnphase}' is "
                             f"still exceeded num_unique='{nuniq}'. Please increase `maxnphase` or set to `None` "
                             "so that all of the table may be used.")
        tab = order[:ntab]
        tflags = np.array(list(itertools.product([-1, 0], repeat=ntab)))       # [nct, ntab]
        tcorn = dig[tab][None] + tflags[..., None]                              # [nct, ntab, npts]
        tuniq, tinv = np.unique(tcorn.transpose(0, 2, 1).reshape(-1, ntab), axis=0, return_inverse=True)
        phase_index = np.asarray(tinv).reshape(tflags.shape[0], npts)
        weights = np.ones((tflags.shape[0], ntab, npts))
        params = {}
        for i, idx in enumerate(tab):
            g = self._grid_coords[idx]
            params[self._names[idx]] = g[tuniq[:, i]]
            lower, upper = g[tuniq[phase_index[0], i]], g[tuniq[phase_index[-1], i]]
            w = (data[idx] - lower) / (upper - lower)
            weights[tflags[:, i] == -1, i] = 1.0 - w
            weights[tflags[:, i] == 0, i] = w
        for idx in order[ntab:]:
            if exact_vals[idx].size != 1:
                raise ValueError(f"parameter '{self._names[idx]}' varies over the grid but is not tabulated: "
                                 "increase `maxnphase` or use interpolation_mode='nearest'")
            params[self._names[idx]] = np.full(tuniq.shape[0], exact_vals[idx][0])
        params = {n: params[n] for n in self._names}
        return params, np.prod(weights, axis=1), phase_index

    def _exact_species(self, density, table, params, weights, phase_index):
        from .mie import get_poly_table
        from .size_distribution import SizeDistributionGrid
        nd = self._size_distribution_function(table.radius, **params, particle_density=self._particle_density)
        poly = get_poly_table(SizeDistributionGrid(radius=np.asarray(table.radius), number_density=nd,
                                                   coords={}, attrs={}), table)
        ext = np.sum(weights * np.asarray(poly.extinction, np.float64)[phase_index], axis=0)
        alb = np.sum(weights * np.asarray(poly.ssalb, np.float64)[phase_index], axis=0)
        shape = density.shape
        leg = np.asarray(poly.legcoef, np.float32)                               # [6, L+1, n]
        legcoef = leg.transpose(2, 0, 1) if self.num_stokes == 3 else leg[0].T
        return Species(extinction=(density * ext.reshape(shape)).astype(np.float32),
                       ssalb=alb.reshape(shape).astype(np.float32),
                       legcoef=np.ascontiguousarray(legcoef, np.float32),
                       table_index=(1 + phase_index).reshape((-1,) + shape).astype(np.int32),
                       phase_weights=weights.reshape((-1,) + shape).astype(np.float32))


def _point_mixtures(sp: Species, num_stokes: int) -> np.ndarray:
    """Per grid point the phase mixture sum_q w_q legcoef[table_index_q - 1]:
    [npts, nleg+1] (scalar) or [npts, 6, nleg+1]."""
    leg = np.asarray(sp.legcoef, np.float64)
    ti = np.asarray(sp.table_index).reshape(np.asarray(sp.table_index).shape[0], -1)
    pw = np.asarray(sp.phase_weights, np.float64).reshape(ti.shape)
    out = np.zeros((ti.shape[1],) + leg.shape[1:])
    for q in range(ti.shape[0]):
        out += pw[q].reshape((-1,) + (1,) * (leg.ndim - 1)) * leg[ti[q] - 1]
    return out


def _generator_derivatives(self, variable_names, microphysics, rel_step: float = 0.01) -> dict:
    """Derivatives of the optical properties with respect to microphysical
    variables (OpticalPropertyGenerator.calculate_derivatives,
    at3d/medium.py:322-510), by central differences of this generator's own
    output: each named variable ('density' or a distribution parameter) is
    moved by +-rel_step x its value (+-rel_step where it is 0) at every
    point at once (the properties are pointwise).  Returns {key: {name:
    {'extinction', 'ssalb': [npx, npy, npz], 'legcoef': the derivative of
    each point's phase mixture, [npts, nleg+1] or [npts, 6, nleg+1]}}}.
    Inside a bracket of a tabulated parameter the mixing is multilinear, so
    the differences are the exact derivative there.  The phase derivatives
    hold one series per point: for large grids ask for few variables."""
    out = {k: {} for k in self._monodisperse_tables}
    for name in np.atleast_1d(variable_names):
        name = str(name)
        if name != "density" and name not in self._names:
            raise ValueError(f"Invalid variable name to differentiate '{name}'")
        v = np.asarray(microphysics[name], np.float64)
        step = np.where(v != 0, rel_step * np.abs(v), rel_step)
        plus = self(dict(microphysics, **{name: v + step}))
        minus = self(dict(microphysics, **{name: v - step}))
        for k in out:
            d = 2.0 * step
            dleg = (_point_mixtures(plus[k], self.num_stokes) - _point_mixtures(minus[k], self.num_stokes))
            out[k][name] = {
                "extinction": (np.asarray(plus[k].extinction, np.float64) - minus[k].extinction) / d,
                "ssalb": (np.asarray(plus[k].ssalb, np.float64) - minus[k].ssalb) / d,
                "legcoef": dleg / d.reshape((-1,) + (1,) * (dleg.ndim - 1)),
            }
    self(microphysics)   # keep the result of the unperturbed microphysics
    return out


OpticalPropertyGenerator.calculate_derivatives = _generator_derivatives
