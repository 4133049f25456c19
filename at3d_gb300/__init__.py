"""GB300-native SHDOM solve / render path (drop-in for AT3D's RTE hot path).

The numerical work runs in the CUDA library built from at3d_gb300/csrc
(include/shdom_gb300.h is its C-ABI); this package holds the host-side
mirror of the reference's Python interface.
"""
from . import (configuration, grid, medium, mie, regularization, scenes, sensor,  # noqa: F401
               size_distribution, source, surface, transforms, uncertainties, util)
from ._abi import NumericalParams, Problem, Species  # noqa: F401

__all__ = ["RTE", "NumericalParams", "Problem", "Species", "configuration", "grid", "medium", "mie", "scenes",
           "regularization", "sensor", "size_distribution", "source", "surface", "transforms", "uncertainties", "util",
           "optimize", "containers"]


def __getattr__(name):
    if name == "RTE":
        from .solver import RTE
        return RTE
    if name in ("optimize", "containers"):   # import the solver (and its library binding) on first use
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
