"""Solar, thermal and combined sources (at3d.source, at3d/source.py:14-215)."""
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


@dataclass
class ThermalSource:
    """Thermal emission (srctype 'T') or thermal plus solar ('B').  skyrad
    is the sky's brightness temperature for 'T' (a radiance for 'B', as the
    reference's COMPUTE_TOP_RADIANCES takes it)."""
    wavelength: float
    skyrad: float = 0.0
    units: str = "R"
    srctype: str = "T"
    solarmu: float = -0.5
    solaraz: float = 0.0
    solarflux: float = 0.0


def _units_flag(units):
    if units == "radiance":
        return "R"
    if units == "brightness_temperature":
        return "T"
    raise ValueError("`units` should be either 'radiance' or 'brightness_temperature'.")


def thermal(wavelength, skyrad=0.0, units="radiance") -> ThermalSource:
    """at3d.source.thermal (at3d/source.py:82-140): emission from the medium
    (which then needs a temperature), the ground and the sky."""
    if np.size(skyrad) != 1:
        raise ValueError("only an isotropic sky is supported")
    return ThermalSource(float(wavelength), float(skyrad), _units_flag(units))


def combined(wavelength, solarmu, solar_azimuth, solarflux=1.0, skyrad=0.0) -> ThermalSource:
    """at3d.source.combined (at3d/source.py:143-215): the solar beam and
    thermal emission together (srctype 'B'), in radiance units."""
    solarmu = -1 * np.abs(solarmu)
    if not (-1.0 <= solarmu < 0.0):
        raise ValueError(f"solarmu must be in the range -1.0 <= solarmu < 0.0 not '{solarmu}'.")
    if np.size(skyrad) != 1:
        raise ValueError("only an isotropic sky is supported")
    return ThermalSource(float(wavelength), float(skyrad), "R", "B", float(solarmu),
                         float(np.deg2rad(solar_azimuth)), float(solarflux))
