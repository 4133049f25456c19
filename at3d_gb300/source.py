"""Solar source (at3d.source.solar, at3d/source.py:14-80)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SolarSource:
    wavelength: float
    solarmu: float      # < 0: direction of propagation of the beam
    solaraz: float      # radians
    solarflux: float = 1.0
    skyrad: float = 0.0


def solar(wavelength, solarmu, solar_azimuth, solarflux=1.0, skyrad=0.0) -> SolarSource:
    """solarmu is forced negative; solar_azimuth in degrees (reference convention)."""
    solarmu = -1 * np.abs(solarmu)
    if not (-1.0 <= solarmu < 0.0):
        raise ValueError(f"solarmu must be in the range -1.0 <= solarmu < 0.0 not '{solarmu}'.")
    if np.size(skyrad) != 1:
        raise ValueError("only an isotropic sky radiance is supported")
    return SolarSource(float(wavelength), float(solarmu), float(np.deg2rad(solar_azimuth)),
                       float(solarflux), float(skyrad))
