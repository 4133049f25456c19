"""ctypes binding of the C-ABI declared in include/shdom_gb300.h.

The library must have been built (at3d_gb300.build.build()); there is no
fallback implementation: a missing library raises ImportError-style
RuntimeError at first use.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

_f, _i, _d = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double)


class ShdomSizes(C.Structure):
    _fields_ = [("npts", C.c_int), ("ncells", C.c_int), ("nx1", C.c_int), ("ny1", C.c_int), ("nz", C.c_int),
                ("nlm", C.c_int), ("nmu", C.c_int), ("nang", C.c_int), ("ml", C.c_int), ("mm", C.c_int),
                ("bcflag", C.c_int), ("ipflag", C.c_int), ("iters", C.c_int), ("nlevels_down", C.c_int),
                ("nlevels_up", C.c_int), ("solcrit", C.c_float), ("albmax", C.c_float),
                ("launches", C.c_longlong), ("device_bytes", C.c_longlong), ("nstokes", C.c_int),
                ("march", C.c_int), ("march_units_down", C.c_int), ("march_units_up", C.c_int),
                ("march_cluster_down", C.c_int), ("march_cluster_up", C.c_int)]


# name -> (restype, argtypes): the exported surface of include/shdom_gb300.h
SIGNATURES = {
    "shdom_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "shdom_init_solution": (C.c_int, [C.c_void_p]),
    "shdom_solution_iterations": (C.c_int, [C.c_void_p, C.c_int, _i, _f]),
    "shdom_render": (C.c_int, [C.c_void_p, C.c_int, _f, _f, _f, _d, _d, _f]),
    "shdom_render_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "shdom_render_noalloc": (C.c_int, [C.c_void_p, C.c_int, _f, _f, _f, _d, _d, _f]),
    "shdom_export_state": (C.c_int, [C.c_void_p, _f, _i, _f, _i, _f, _f]),
    "shdom_get_sizes": (C.c_int, [C.c_void_p, C.POINTER(ShdomSizes)]),
    "shdom_last_timings": (C.c_int, [C.c_void_p, _f]),
    "shdom_sweep_timings": (C.c_int, [C.c_void_p, _f, _i]),
    "shdom_set_transform_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "shdom_set_sweep_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "shdom_set_render_options": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "shdom_set_transform_wait_limit": (C.c_int, [C.c_void_p, C.c_int]),
    "shdom_plan_summary": (C.c_int, [C.c_void_p, C.POINTER(ShdomSizes)]),
    "shdom_levis_gradient": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _f, _f, _f, _d, _d, _f, _d,
                                       C.POINTER(C.c_double), _f]),
    "shdom_levis_adjoint": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _f, _f, _f, _d, _d, _d, _d]),
    "shdom_levis_adjoint_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 8),
    "shdom_last_error": (C.c_char_p, [C.c_void_p]),
    "shdom_destroy": (None, [C.c_void_p]),
    "shdom_plan_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(ShdomSizes)]),
    "shdom_create_planned": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "shdom_plan_destroy": (None, [C.c_void_p]),
    "shdom_plan_optical_path": (C.c_int, [C.c_void_p, C.c_int, _f, _f, _f, _d, _d, C.c_int, _f]),
    "shdom_optical_path": (C.c_int, [C.c_void_p, C.c_int, _f, _f, _f, _d, _d, C.c_int, _f]),
    "shdom_plan_point_absorption": (C.c_int, [C.c_void_p, _f, _f]),
    "shdom_plan_min_optical_path": (C.c_int, [C.c_void_p, C.c_int, _f, _f, _f, _d, _d, C.c_int, C.c_int, _f]),
    "shdom_point_absorption": (C.c_int, [C.c_void_p, _f, _f]),
    "shdom_mie_mono": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int, _f, C.c_int, C.c_int, _f, _f, _i,
                                 _f]),
    "shdom_phase_function_mixing": (C.c_int, [C.c_int, C.c_int, C.c_int, _f, _i, _f, C.c_int, C.c_int, C.c_int, _f,
                                              C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _f, _i, _i,
                                              _i]),
}

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"CUDA library {LIB} is not built: run at3d_gb300.build.build() "
                               "(there is no CPU fallback for the solver)")
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB
