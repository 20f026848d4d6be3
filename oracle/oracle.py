"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is what the CUDA product path is compared against: only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module. It restates CFMultigrid.jl's ``Gmg`` object (src/gmg_types.jl,
src/gmg_setup.jl, src/gmg_cycles.jl, src/gmg_solver.jl) on the CPU in FP64;
see cfmg_oracle.cpp for the per-function citations.

Field arrays are exposed as zero-copy numpy views in Fortran order with shape
(tx, ty, tz), so ``g.b[i-1, j-1, k-1]`` is Julia's ``mg.data[1].b[i, j, k]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcfmg_oracle.so")
# OpenMP build of the same source (identical results, element-wise loops
# split over threads); selected with CFMG_ORACLE_THREADS > 1 before import.
_LIB_OMP_PATH = os.path.join(_HERE, "_build", "libcfmg_oracle_omp.so")

LOCATIONS = {"centers": 0, "vertices": 1}
CASES = {"twod": 0, "threed": 1}
OPERATORS = {"laplacian": 0, "laplacian9": 1, "varcoef": 2}
CYCLES = {"v": 0, "f": 1, "onelev": 2, "twolev": 3, "nlev": 4, "vrec": 5}
TOPOLOGIES = {"closed": 0, "xperio": 1}
FIELDS = {"x": 0, "r": 1, "b": 2, "y": 3, "diag": 4, "idiag": 5, "Rcoef": 6, "Pcoef": 7, "kappa": 8}


class _Param(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nh", ctypes.c_int),
        ("npre", ctypes.c_int), ("npost", ctypes.c_int), ("ndeepest", ctypes.c_int), ("maxite", ctypes.c_int),
        ("tol", ctypes.c_double), ("omega", ctypes.c_double),
        ("location", ctypes.c_int), ("kase", ctypes.c_int), ("op", ctypes.c_int), ("cycle", ctypes.c_int),
        ("topology", ctypes.c_int), ("nlevels", ctypes.c_int),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _LIB_OMP_PATH if int(os.environ.get("CFMG_ORACLE_THREADS", "1")) > 1 else _LIB_PATH
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.orc_get_gmg.restype = vp
        L.orc_get_gmg.argtypes = [ctypes.POINTER(_Param)]
        L.orc_allocate.restype = vp
        L.orc_allocate.argtypes = [ctypes.POINTER(_Param)]
        L.orc_free.argtypes = [vp]
        L.orc_nlevels.argtypes = [vp]
        L.orc_nlevels.restype = ctypes.c_int
        L.orc_level_dims.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_field.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_field.restype = ctypes.POINTER(ctypes.c_double)
        L.orc_msk.argtypes = [vp, ctypes.c_int]
        L.orc_msk.restype = ctypes.POINTER(ctypes.c_uint8)
        for name in ("orc_set_default_msk", "orc_setup_operators"):
            getattr(L, name).argtypes = [vp]
        L.orc_smooth.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_residual.argtypes = [vp, ctypes.c_int]
        L.orc_restrict.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_prolong.argtypes = [vp, ctypes.c_int]
        L.orc_zero.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_fill.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_norm.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.orc_norm.restype = ctypes.c_double
        L.orc_normresidual.argtypes = [vp, ctypes.c_double]
        L.orc_normresidual.restype = ctypes.c_double
        L.orc_cycle.argtypes = [vp, ctypes.c_int]
        L.orc_solve.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def _param_struct(p) -> _Param:
    get = (lambda k, d=None: p.get(k, d)) if isinstance(p, dict) else (lambda k, d=None: getattr(p, k, d))
    return _Param(
        nx=int(get("nx", 64)), ny=int(get("ny", 64)), nz=int(get("nz", 64)), nh=int(get("nh", 3)),
        npre=int(get("npre", 1)), npost=int(get("npost", 1)), ndeepest=int(get("ndeepest", 20)),
        maxite=int(get("maxite", 15)), tol=float(get("tol", 1e-10)), omega=float(get("omega", 0.9)),
        location=LOCATIONS[get("location", "centers")], kase=CASES[get("case", "threed")],
        op=OPERATORS[get("operator", "laplacian")], cycle=CYCLES[get("cycle", "v")],
        topology=TOPOLOGIES[get("topology", "closed")], nlevels=int(get("nlevels", 0) or 0),
    )


class OracleGmg:
    """The CPU oracle's multigrid object, mirroring CFMultigrid's ``Gmg``."""

    def __init__(self, param, setup: bool = True):
        L = lib()
        self._p = _param_struct(param)
        h = L.orc_get_gmg(ctypes.byref(self._p)) if setup else L.orc_allocate(ctypes.byref(self._p))
        if not h:
            raise ValueError("invalid multigrid parameters")
        self._h = ctypes.c_void_p(h)
        self.nlevels = L.orc_nlevels(self._h)
        self.maxite = self._p.maxite

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.orc_free(h)
            self._h = None

    def dims(self, lev: int):
        d = (ctypes.c_int * 7)()
        lib().orc_level_dims(self._h, lev, d)
        return tuple(d)

    def shape(self, lev: int):
        d = self.dims(lev)
        return (d[4], d[5], d[6])

    def field(self, lev: int, name: str) -> np.ndarray:
        shape = self.shape(lev)
        n = shape[0] * shape[1] * shape[2]
        if name == "msk":
            ptr = lib().orc_msk(self._h, lev)
            flat = np.ctypeslib.as_array(ptr, shape=(n,))
        else:
            ptr = lib().orc_field(self._h, lev, FIELDS[name])
            flat = np.ctypeslib.as_array(ptr, shape=(n,))
        return flat.reshape(shape, order="F")

    # Julia-style accessors for level 1
    @property
    def x(self):
        return self.field(1, "x")

    @property
    def b(self):
        return self.field(1, "b")

    @property
    def msk(self):
        return self.field(1, "msk")

    def set_default_msk(self):
        lib().orc_set_default_msk(self._h)

    def setup_operators(self):
        lib().orc_setup_operators(self._h)

    def smooth(self, lev, nite):
        lib().orc_smooth(self._h, lev, nite)

    def residual(self, lev):
        lib().orc_residual(self._h, lev)

    def restrict(self, lev, field="r"):
        lib().orc_restrict(self._h, lev, FIELDS[field])

    def prolong(self, lev):
        lib().orc_prolong(self._h, lev)

    def zero(self, lev, field):
        lib().orc_zero(self._h, lev, FIELDS[field])

    def fill(self, lev, field):
        lib().orc_fill(self._h, lev, 9 if field == "msk" else FIELDS[field])

    def norm(self, lev, field):
        return lib().orc_norm(self._h, lev, FIELDS[field])

    def normresidual(self, normb):
        return lib().orc_normresidual(self._h, normb)

    def cycle(self, kind="v"):
        lib().orc_cycle(self._h, CYCLES[kind])

    def solve(self):
        """solve!(mg): returns (res, nite, history[0..nite])."""
        res = ctypes.c_double()
        nite = ctypes.c_int()
        hist = (ctypes.c_double * (self.maxite + 1))()
        lib().orc_solve(self._h, ctypes.byref(res), ctypes.byref(nite), hist)
        return res.value, nite.value, np.array(hist[: nite.value + 1])
