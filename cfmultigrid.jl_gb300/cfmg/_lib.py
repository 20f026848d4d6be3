"""ctypes binding of libcfmg.so (the C ABI declared in include/cfmg.h).

The library is built in-tree (``cfmultigrid.jl_gb300/build.py``) and loaded
from this directory. There is no fallback: if the shared library is missing
the import of the package fails loudly.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcfmg.so")

# status codes
OK = 0
ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_STATE, ERR_NONFINITE, ERR_UNSUPPORTED = 1, 2, 3, 4, 5, 6

# Param symbols
CASES = {"twod": 0, "threed": 1}
LOCATIONS = {"centers": 0, "vertices": 1}
OPERATORS = {"laplacian": 0, "laplacian9": 1, "varcoef": 2}
TOPOLOGIES = {"closed": 0, "xperio": 1}
CYCLES = {"v": 0, "f": 1, "onelev": 2, "twolev": 3, "nlev": 4, "vrec": 5}
PRECISIONS = {"fp64": 0, "mixed": 1}
NORMS = {"ref_squared": 0, "l2": 1}
FIELDS = {"x": 0, "r": 1, "b": 2, "y": 3, "diag": 4, "idiag": 5, "Rcoef": 6, "Pcoef": 7, "kappa": 8, "msk": 9}

# every entry point of include/cfmg.h
EXPORTS = (
    "cfmg_desc_default", "cfmg_create", "cfmg_destroy", "cfmg_last_error", "cfmg_nlevels", "cfmg_level_dims",
    "cfmg_set_stream", "cfmg_synchronize", "cfmg_upload", "cfmg_download", "cfmg_field_ptr", "cfmg_bind_level",
    "cfmg_set_default_msk", "cfmg_setup_operators", "cfmg_smooth", "cfmg_residual", "cfmg_restrict",
    "cfmg_prolong", "cfmg_zero", "cfmg_fill", "cfmg_norm", "cfmg_normresidual", "cfmg_cycle", "cfmg_solve",
    "cfmg_launch_count", "cfmg_profile", "cfmg_profile_read", "cfmg_set_option", "cfmg_norm_noalloc",
    "cfmg_adjoint", "cfmg_solve_tol", "cfmg_adjoint_solve", "cfmg_batch_create", "cfmg_batch_destroy", "cfmg_batch_instance", "cfmg_batch_solve",
    "cfmg_batch_last_error", "cfmg_batch_set_option",
)
OPTIONS = {"engine_cells": 0, "temporal_blocking": 1, "coarsest_fp64": 2, "int_residual": 3, "host_loop": 4,
           "fused_descent": 5, "fused_update": 6, "dependent_launch": 7,
           "coded_widiag": 8, "staged_residual": 9, "skip_dry": 10, "small_smooth": 11}
BATCH_OPTIONS = {"host_loop": 0, "coarse_runs": 1, "interleave": 2}
KERNEL_CLASSES = {"sweep": 0, "residual": 1, "restrict": 2, "prolong": 3, "norm": 4, "fill": 5, "convert": 6,
                  "engine": 7,
                  "descent": 8}


class Desc(ctypes.Structure):
    """cfmg_desc (include/cfmg.h)."""

    _fields_ = [
        ("kase", ctypes.c_int), ("location", ctypes.c_int), ("op", ctypes.c_int), ("topology", ctypes.c_int),
        ("cycle", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("nh", ctypes.c_int), ("nlevels", ctypes.c_int), ("npre", ctypes.c_int), ("npost", ctypes.c_int),
        ("ndeepest", ctypes.c_int), ("maxite", ctypes.c_int), ("omega", ctypes.c_double), ("tol", ctypes.c_double),
        ("precision", ctypes.c_int), ("norm_kind", ctypes.c_int),
    ]


_lib = None


def load() -> ctypes.CDLL:
    """Load libcfmg.so and declare the signatures of its entry points."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libcfmg.so not found at {LIB_PATH}: build it with `python cfmultigrid.jl_gb300/build.py` "
            "(there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    pi, pd = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    sig = {
        "cfmg_desc_default": [ctypes.POINTER(Desc)],
        "cfmg_create": [ctypes.POINTER(Desc), ctypes.POINTER(vp)],
        "cfmg_destroy": [vp],
        "cfmg_nlevels": [vp, pi],
        "cfmg_level_dims": [vp, i, pi],
        "cfmg_set_stream": [vp, vp],
        "cfmg_synchronize": [vp],
        "cfmg_upload": [vp, i, i, vp],
        "cfmg_download": [vp, i, i, vp],
        "cfmg_field_ptr": [vp, i, i, ctypes.POINTER(vp)],
        "cfmg_bind_level": [vp, i, vp, vp, vp, vp, vp],
        "cfmg_set_default_msk": [vp],
        "cfmg_setup_operators": [vp],
        "cfmg_smooth": [vp, i, i],
        "cfmg_residual": [vp, i],
        "cfmg_restrict": [vp, i, i],
        "cfmg_prolong": [vp, i],
        "cfmg_zero": [vp, i, i],
        "cfmg_fill": [vp, i, i],
        "cfmg_norm": [vp, i, i, pd],
        "cfmg_normresidual": [vp, d, pd],
        "cfmg_cycle": [vp, i],
        "cfmg_solve": [vp, pd, pi, pd],
        "cfmg_launch_count": [vp, ctypes.POINTER(ctypes.c_longlong)],
        "cfmg_profile": [vp, i, i, i],
        "cfmg_profile_read": [vp, ctypes.POINTER(ctypes.c_longlong), pd],
        "cfmg_set_option": [vp, i, ctypes.c_longlong],
        "cfmg_norm_noalloc": [vp, vp, ctypes.c_longlong, vp, vp],
        "cfmg_adjoint": [vp, vp, vp, vp, pd, pi],
        "cfmg_solve_tol": [vp, d, i, i, pd, pi, pd],
        "cfmg_adjoint_solve": [vp, vp, vp, vp],
        "cfmg_batch_create": [ctypes.POINTER(Desc), i, vp, vp, vp, ctypes.POINTER(vp)],
        "cfmg_batch_destroy": [vp],
        "cfmg_batch_instance": [vp, i, ctypes.POINTER(vp)],
        "cfmg_batch_solve": [vp, i, vp, vp, vp],
        "cfmg_batch_set_option": [vp, i, ctypes.c_longlong],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.cfmg_last_error.argtypes = [vp]
    L.cfmg_last_error.restype = ctypes.c_char_p
    L.cfmg_batch_last_error.argtypes = [vp]
    L.cfmg_batch_last_error.restype = ctypes.c_char_p
    _lib = L
    return L
