"""Input formats and small helpers around the solver.

Mirrors part of at3d.util (at3d/util.py): the microphysics readers
``load_from_csv`` (:465-492) and ``load_2parameter_lwc_file`` (:377-417) with
the writer ``to_2parameter_lwc_file`` (:419-463), ``planck_function``
(:336-347), ``freq_to_wavelength`` (:349-352) and ``get_phase_function``
(:74-235, the phase-matrix elements of TRANSFORM_LEG_TO_PHASE,
src/polarized/make_mie_table.f90:760-869).  Fields come back as numpy
arrays in dicts (x, y, z, delx, dely and one [nx, ny, nz] array per
variable, NaN where the file has no value), the input of
``grid.resample_onto_grid`` and ``medium.table_to_grid``.

File layouts (as the reference reads them):
* CSV: one comment line, ``nx,ny,nz``, ``dx,dy``, the z levels
  (comma-separated; text after '#' ignored), a header naming the columns
  (``x,y,z,<variables>``), then one row per given point with 0-based
  integer indices;
* 2-parameter LWC: a title line, ``nx ny nz``, ``dx dy``, the z levels, the
  temperature of each level, then rows ``i j k lwc reff`` with 1-based
  indices.
"""
from __future__ import annotations

import numpy as np

PHASE_ELEMENTS = ("P11", "P22", "P33", "P44", "P12", "P34")


def _numbers(line: str, sep=None) -> np.ndarray:
    text = line.split("#", 1)[0].strip()
    parts = [p for p in (text.split(sep) if sep else text.split()) if p.strip() != ""]
    return np.array([float(p) for p in parts])


def _grid_dict(nx, ny, nz, dx, dy, z) -> dict:
    return {"x": np.arange(nx) * dx, "y": np.arange(ny) * dy, "z": np.asarray(z, np.float64),
            "delx": float(dx), "dely": float(dy)}


def load_from_csv(path, density=None, origin=(0.0, 0.0)) -> dict:
    """Microphysics from a CSV file (load_from_csv, at3d/util.py:465-492);
    ``density`` names the column that becomes 'density'.  ``origin`` is
    accepted as in the reference, which does not use it either."""
    with open(path) as f:
        lines = f.read().splitlines()
    nx, ny, nz = _numbers(lines[1], ",").astype(int)
    dx, dy = _numbers(lines[2], ",")
    z = _numbers(lines[3], ",")
    if z.size != nz:
        raise ValueError(f"{z.size} z levels for nz = {nz}")
    header = [h.strip() for h in lines[4].split("#", 1)[0].split(",")]
    if header[:3] != ["x", "y", "z"]:
        raise ValueError("the column header must start with x,y,z")
    rows = [r for r in lines[5:] if r.split("#", 1)[0].strip()]
    data = np.array([_numbers(r, ",") for r in rows]).reshape(-1, len(header))
    out = _grid_dict(nx, ny, nz, dx, dy, z)
    i, j, k = (data[:, c].astype(int) for c in range(3))
    for c, name in enumerate(header[3:], start=3):
        v = np.full((nx, ny, nz), np.nan)
        v[i, j, k] = data[:, c]
        out[name] = v
    if density is not None:
        if density not in out:
            raise KeyError(f"density variable: '{density}' must be in the file")
        out["density"] = out.pop(density)
        out["density_name"] = density
    out["file_name"] = str(path)
    return out


def load_2parameter_lwc_file(file_name, density="lwc") -> dict:
    """'density' (liquid water content), 'reff' and the 'temperature' profile
    of a 2-parameter LWC file (load_2parameter_lwc_file, at3d/util.py:377-417)."""
    with open(file_name) as f:
        lines = f.read().splitlines()
    nx, ny, nz = _numbers(lines[1]).astype(int)
    dx, dy = _numbers(lines[2])
    z = _numbers(lines[3])
    temperature = _numbers(lines[4])
    rows = [r for r in lines[5:] if r.strip()]
    out = _grid_dict(nx, ny, nz, dx, dy, z)
    lwc = np.full((nx, ny, nz), np.nan)
    reff = np.full((nx, ny, nz), np.nan)
    if rows:
        data = np.array([_numbers(r) for r in rows])
        i, j, k = (data[:, c].astype(int) - 1 for c in range(3))
        lwc[i, j, k] = data[:, 3]
        reff[i, j, k] = data[:, 4]
    out.update(density=lwc, reff=reff, temperature=temperature, density_name=density, file_name=str(file_name))
    return out


def to_2parameter_lwc_file(file_name, cloud_scatterer: dict, temperature=None, fill_temperature: float = 280.0):
    """Write 'density' and 'reff' of a scatterer ([nx, ny, nz], coordinates
    x, y, z) as a 2-parameter LWC file (to_2parameter_lwc_file,
    at3d/util.py:419-463); ``temperature``: a profile on z (the reference
    interpolates an atmosphere onto z), else ``fill_temperature``."""
    lwc = np.asarray(cloud_scatterer["density"], np.float64)
    reff = np.asarray(cloud_scatterer["reff"], np.float64)
    nx, ny, nz = lwc.shape
    x, y, z = (np.asarray(cloud_scatterer[k], np.float64) for k in ("x", "y", "z"))
    dx, dy = x[1] - x[0], y[1] - y[0]
    t = np.full(nz, fill_temperature) if temperature is None else np.asarray(temperature, np.float64)
    i, j, k = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    with open(file_name, "w") as f:
        f.write("2 parameter LWC file\n")
        f.write(f" {nx} {ny} {nz}\n")
        f.write(f"{dx} {dy}\n")
        f.write(" ".join(f"{v}" for v in z) + "\n")
        f.write(" ".join(f"{v:5.2f}" for v in t) + "\n")
        for a, b, c, l, r in zip(i.ravel(), j.ravel(), k.ravel(), lwc.ravel(), reff.ravel()):
            f.write(f"{a} {b} {c} {l:5.4f} {r:3.2f}\n")


def planck_function(temperature, wavelength, c=2.99792458e8, h=6.62606876e-34, k=1.3806503e-23):
    """Planck radiance [W/m^2/um/sr] at ``wavelength`` [um] and ``temperature`` [K]."""
    lam = np.asarray(wavelength, np.float64) * 1e-6
    return 2 * h * c ** 2 / lam ** 5 / (np.exp((h * c) / (lam * k * np.asarray(temperature, np.float64))) - 1.0) * 1e-6


def freq_to_wavelength(mu):
    """Wavelength [um] of a frequency [GHz]."""
    return 1e6 * (299792458.0 / (np.asarray(mu, np.float64) * 1e9))


def _wigner(x: np.ndarray, L: int, kind: str) -> np.ndarray:
    """d^l_00, d^l_22 or d^l_20 at x, [L+1, len(x)] (three-term recurrences in l)."""
    d = np.zeros((L + 1, x.size))
    if kind == "00":
        d[0] = 1.0
        if L >= 1:
            d[1] = x
        for l in range(1, L):
            d[l + 1] = ((2 * l + 1) * x * d[l] - l * d[l - 1]) / (l + 1)
        return d
    if L < 2:
        return d
    if kind == "22":
        d[2] = 0.25 * (1 + x) ** 2
        for l in range(2, L):
            q = (l + 1) ** 2 - 4.0
            d[l + 1] = ((2 * l + 1) * (l * (l + 1) * x - 4) * d[l] - (l + 1) * (l * l - 4.0) * d[l - 1]) / (l * q)
    else:
        d[2] = 0.25 * np.sqrt(6.0) * (1 - x * x)
        for l in range(2, L):
            d[l + 1] = ((2 * l + 1) * x * d[l] - np.sqrt(l * l - 4.0) * d[l - 1]) / np.sqrt((l + 1) ** 2 - 4.0)
    return d


def get_phase_function(legcoef, angles, phase_elements="All") -> np.ndarray:
    """Phase-matrix elements at scattering ``angles`` [degrees] from Wigner
    coefficients ``legcoef`` [6, L+1, *grid] (a1, a2, a3, a4, b1, b2; a
    [L+1] or [1, L+1] series gives P11 only) (get_phase_function,
    at3d/util.py:74-235; TRANSFORM_LEG_TO_PHASE): P11 = sum a1 d00,
    P22 / P33 = (sum (a2+a3) d22(x) +- sum (a2-a3) (-1)^l d22(-x)) / 2,
    P44 = sum a4 d00, P12 = -sum b1 d20, P34 = -sum b2 d20.  Returns
    [n_elements, n_angles, *grid]."""
    names = list(PHASE_ELEMENTS) if phase_elements == "All" else \
        ([phase_elements] if isinstance(phase_elements, str) else list(phase_elements))
    for n in names:
        if n not in PHASE_ELEMENTS:
            raise ValueError(f"Invalid value for phase_elements '{n}' Valid values are '{PHASE_ELEMENTS}'")
    lc = np.asarray(legcoef, np.float64)
    if lc.ndim == 1:
        lc = lc[None]
    if lc.shape[0] == 1 and any(n != "P11" for n in names):
        raise ValueError("a series without polarization elements gives P11 only")
    L = lc.shape[1] - 1
    grid = lc.shape[2:]
    flat = lc.reshape(lc.shape[0], L + 1, -1)
    x = np.cos(np.deg2rad(np.asarray(angles, np.float64)))
    sign = (-1.0) ** np.arange(L + 1)
    out = []
    d00 = _wigner(x, L, "00")
    for n in names:
        if n == "P11":
            v = np.einsum("lg,la->ag", flat[0], d00)
        elif n == "P44":
            v = np.einsum("lg,la->ag", flat[3], d00)
        elif n in ("P22", "P33"):
            dp, dm = _wigner(x, L, "22"), _wigner(-x, L, "22")
            p3 = np.einsum("lg,la->ag", flat[1] + flat[2], dp)
            m3 = np.einsum("lg,la->ag", (flat[1] - flat[2]) * sign[:, None], dm)
            v = 0.5 * (p3 + m3) if n == "P22" else 0.5 * (p3 - m3)
        else:
            d20 = _wigner(x, L, "20")
            v = -np.einsum("lg,la->ag", flat[4 if n == "P12" else 5], d20)
        out.append(v.reshape((x.size,) + grid))
    return np.stack(out)
