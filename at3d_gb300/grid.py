"""Property grids (at3d.grid.make_grid, at3d/grid.py:23-94): regular x/y
spacing starting at 0 and explicit z levels."""
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
