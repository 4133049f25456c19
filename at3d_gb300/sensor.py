"""Ray sets (at3d.sensor.make_sensor_dataset, at3d/sensor.py:31-106): mu and
phi point from the scene towards the sensor."""
from __future__ import annotations

import numpy as np


def make_sensor_dataset(x, y, z, mu, phi, stokes=("I",), wavelength=None) -> dict:
    n = np.size(x)
    for v in (y, z, mu, phi):
        if np.size(v) != n:
            raise ValueError("ray arrays must have the same length")
    return {"ray_x": np.asarray(x, np.float64).ravel(), "ray_y": np.asarray(y, np.float64).ravel(),
            "ray_z": np.asarray(z, np.float64).ravel(), "ray_mu": np.asarray(mu, np.float64).ravel(),
            "ray_phi": np.asarray(phi, np.float64).ravel(), "stokes": list(stokes), "wavelength": wavelength}


def average_subpixel_rays(radiance, pixel_index, ray_weight, npixels):
    """Pixel value = weighted sum of its rays (src/util.f90:484-519)."""
    out = np.zeros(npixels, np.float64)
    np.add.at(out, np.asarray(pixel_index), np.asarray(ray_weight, np.float64) * np.asarray(radiance, np.float64))
    return out
