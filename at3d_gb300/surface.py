"""Lambertian surfaces (at3d.surface.lambertian, at3d/surface.py:28-105)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class LambertianSurface:
    albedo: np.ndarray | float
    ground_temperature: float = 298.15
    delx: float = 0.0
    dely: float = 0.0

    @property
    def variable(self):
        return np.size(self.albedo) > 1


def lambertian(albedo, ground_temperature=298.15, delx=None, dely=None) -> LambertianSurface:
    a = np.asarray(albedo, np.float32)
    if np.any(a > 1.0) or np.any(a < 0.0):
        raise ValueError(f"surface albedo should be in [0, 1] not '{albedo}'")
    if a.size > 1:
        if delx is None or dely is None:
            raise ValueError("dely and delx must be defined for variable surface parameters.")
        return LambertianSurface(np.atleast_2d(a), float(ground_temperature), float(delx), float(dely))
    return LambertianSurface(float(a.reshape(-1)[0]), float(ground_temperature))
