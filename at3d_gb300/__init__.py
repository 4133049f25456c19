"""GB300-native SHDOM solve / render path (drop-in for AT3D's RTE hot path).

The numerical work runs in the CUDA library built from at3d_gb300/csrc
(include/shdom_gb300.h is its C-ABI); this package holds the host-side
mirror of the reference's Python interface.
"""
from . import configuration, grid, medium, scenes, sensor, source, surface  # noqa: F401
from ._abi import NumericalParams, Problem, Species  # noqa: F401

__all__ = ["RTE", "NumericalParams", "Problem", "Species", "configuration", "grid", "medium", "scenes",
           "sensor", "source", "surface"]


def __getattr__(name):
    if name == "RTE":
        from .solver import RTE
        return RTE
    raise AttributeError(name)
