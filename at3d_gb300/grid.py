"""Property grids (at3d.grid, at3d/grid.py): ``make_grid`` (:23-94), regular
x/y spacing starting at 0 and explicit z levels; ``resample_onto_grid``
(:96-180) and ``from_scatterer`` (:295-306) for fields given on other
coordinates; ``combine_z_coordinates`` / ``merge_two_z_coordinates``
(:194-293) for the z levels of several scatterers.  Fields are numpy arrays
in plain dicts (no xarray)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Grid:
    delx: float
    npx: int
    dely: float
    npy: int
    z: np.ndarray

    @property
    def x(self):
        return np.arange(self.npx) * self.delx

    @property
    def y(self):
        return np.arange(self.npy) * self.dely

    @property
    def shape(self):
        return (self.npx, self.npy, len(self.z))


def make_grid(delx: float, npx: int, dely: float, npy: int, z) -> Grid:
    z = np.asarray(z, np.float32)
    if np.any(np.diff(z) <= 0):
        raise ValueError("z levels must be strictly increasing")
    return Grid(float(delx), int(npx), float(dely), int(npy), z)


def _fill_axis(a: np.ndarray, axis: int) -> np.ndarray:
    """Backward then forward fill of NaNs along one axis (xarray's bfill then
    ffill): a NaN takes the next valid value along the axis, or the previous
    one where none follows."""
    a = np.moveaxis(np.array(a, np.float64, copy=True), axis, -1)
    n = a.shape[-1]
    idx = np.arange(n)
    valid = ~np.isnan(a)
    nxt = np.where(valid, idx, n)
    nxt = np.minimum.accumulate(nxt[..., ::-1], axis=-1)[..., ::-1]          # next valid index (n: none)
    prv = np.where(valid, idx, -1)
    prv = np.maximum.accumulate(prv, axis=-1)                                # previous valid index (-1: none)
    src = np.where(nxt < n, nxt, prv)
    has = src >= 0
    out = np.take_along_axis(a, np.clip(src, 0, n - 1), axis=-1)
    out = np.where(has, out, np.nan)
    return np.moveaxis(out, -1, axis)


def resample_onto_grid(grid: Grid, data: dict) -> dict:
    """Variables of ``data`` (coordinates 'x', 'y', 'z' and fields [nx, ny, nz],
    or z profiles [nz]) interpolated linearly onto ``grid`` (resample_onto_grid,
    at3d/grid.py:96-180): missing values of 'density' become 0, those of other
    fields take the nearest valid value along x, then y, then z (backward,
    then forward fill), before and again after the interpolation, where
    points of the grid outside the data's coordinates are missing."""
    from scipy.interpolate import RegularGridInterpolator
    xs, ys, zs = (np.asarray(data[k], np.float64) for k in ("x", "y", "z"))
    gx, gy, gz = np.asarray(grid.x, np.float64), np.asarray(grid.y, np.float64), np.asarray(grid.z, np.float64)
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    out = {}
    for name, v in data.items():
        if name in ("x", "y", "z"):
            continue
        v = np.asarray(v, np.float64)
        if v.ndim == 1 and v.size == zs.size:
            v = np.broadcast_to(v, (xs.size, ys.size, zs.size))
        if v.shape != (xs.size, ys.size, zs.size):
            raise ValueError(f"variable '{name}' has shape {v.shape}, expected {(xs.size, ys.size, zs.size)} "
                             "or a z profile")
        if name == "density":
            filled = np.nan_to_num(v, nan=0.0)
        else:
            filled = v
            for ax in range(3):
                filled = _fill_axis(filled, ax)
        # degenerate axes (a single x or y column) are held constant
        axes, pts = [], []
        for c, g in ((xs, X), (ys, Y), (zs, Z)):
            axes.append(c if c.size > 1 else np.array([c[0] - 1.0, c[0] + 1.0]))
            pts.append(g.ravel() if c.size > 1 else np.full(g.size, c[0]))
        vals = filled
        for ax, c in enumerate((xs, ys, zs)):
            if c.size == 1:
                vals = np.repeat(vals, 2, axis=ax)
        r = RegularGridInterpolator(axes, vals, method="linear", bounds_error=False, fill_value=np.nan)
        res = r(np.stack(pts, axis=1)).reshape(X.shape)
        if name == "density":
            res = np.nan_to_num(res, nan=0.0)
        else:
            for ax in range(3):
                res = _fill_axis(res, ax)
            if np.all(np.isnan(res)):
                raise ValueError(f"Unexpected NaN in '{name}'")
        out[name] = res
    out["x"], out["y"], out["z"] = gx, gy, gz
    out["delx"], out["dely"] = grid.delx, grid.dely
    return out


def merge_two_z_coordinates(z1, z2) -> np.ndarray:
    """Two increasing, non-negative vertical coordinates as one
    (merge_two_z_coordinates, at3d/grid.py:217-293): below and above their
    overlap each one's own levels, inside it the levels of the one with more
    points there.  (The reference also meant to add one extra level at each
    end of the overlap, but its test, ``z_bottom.any() & len(z_middle) > 2``,
    is ``(flag & length) > 2`` and never holds, so no level is added; the
    result here is the same.)"""
    z1, z2 = np.asarray(z1), np.asarray(z2)
    for z, nm in ((z1, "z1"), (z2, "z2")):
        if z.ndim != 1 or not np.all(np.sort(z) == z) or not np.all(z >= 0.0) or np.unique(z).size != z.size:
            raise ValueError(f"{nm} must be >= 0,strictly increasing and 1-D")
    z_bottom = z1[z1 < z2[0]] if z1[0] < z2[0] else z2[z2 < z1[0]]
    z_top = z2[z2 > z1[-1]] if z1[-1] < z2[-1] else z1[z1 > z2[-1]]
    m1, m2 = z1, z2
    if z_bottom.size > 0 and z_top.size > 0:
        m1 = z1[(z1 > z_bottom[-1]) & (z1 < z_top[0])]
        m2 = z2[(z2 > z_bottom[-1]) & (z2 < z_top[0])]
    elif z_top.size > 0:
        m1, m2 = z1[z1 < z_top[0]], z2[z2 < z_top[0]]
    elif z_bottom.size > 0:
        m1, m2 = z1[z1 > z_bottom[-1]], z2[z2 > z_bottom[-1]]
    middle = m1 if len(m1) > len(m2) else m2
    combined = np.concatenate((z_bottom, middle, z_top))
    if np.unique(combined).size != combined.size or not np.all(np.sort(combined) == combined):
        raise ValueError("merged z levels are not strictly increasing")
    return combined


def combine_z_coordinates(z_list) -> np.ndarray:
    """The z levels of several scatterers (arrays, or objects with ``z``) merged
    pairwise in turn (combine_z_coordinates, at3d/grid.py:194-215)."""
    if not isinstance(z_list, (list, tuple)):
        raise TypeError(f"scatterer_list should be a Tuple or List not '{type(z_list)}'")
    zs = [np.asarray(getattr(z, "z", z)) for z in z_list]
    combined = zs[0]
    if len(zs) > 1:
        combined = merge_two_z_coordinates(zs[0], zs[1])
        for z in zs[2:]:
            combined = merge_two_z_coordinates(z, combined)
    return combined


def from_scatterer(scatterer: dict) -> dict:
    """A scatterer resampled onto the grid its own coordinates define: x and
    y spacing from their first step, its z levels (from_scatterer,
    at3d/grid.py:295-306)."""
    x, y, z = (np.asarray(scatterer[k]) for k in ("x", "y", "z"))
    grid = make_grid(float(x[1] - x[0]) if x.size > 1 else 1.0, x.size,
                     float(y[1] - y[0]) if y.size > 1 else 1.0, y.size, z)
    return resample_onto_grid(grid, scatterer)
