"""cfmg: GB300-native geometric multigrid, with CFMultigrid.jl's interface.

This package is the Python host side of libcfmg.so. It mirrors the Julia
reference's public API (src/CFMultigrid.jl:3 exports solve!, Param,
get_gmg, setup_operators!, vcycle!, fill!) so that code written against the
reference reads the same:

    param = Param(nx=512, ny=512, nz=1, case="twod")
    mg = get_gmg(param)                # src/gmg_setup.jl:26-35
    b = mg.data[1].b                   # host copy of level-1 b (Fortran order)
    b[8, 258, 0] = 1.0
    mg.data[1].b = b                   # upload
    res, nite = solve(mg)              # src/gmg_solver.jl:9-42
    x = mg.data[1].x

Every operator runs as a CUDA kernel inside libcfmg; the function tables
``mg.smoother[lev](mg, lev, nite)``, ``mg.residual[lev](mg, lev)``,
``mg.restriction[lev](mg, lev, field)`` and ``mg.prolongation[lev](mg, lev)``
call the library's per-level entry points, exactly as the Julia cycles call
theirs. Levels are 1-based, as in Julia. A non-zero status from the library
raises ``CfmgError`` (the reference raises AssertionError).
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Optional

import numpy as np

from . import _lib
from ._lib import CASES, CYCLES, FIELDS, LOCATIONS, NORMS, OPERATORS, PRECISIONS, TOPOLOGIES

__all__ = ["Param", "Gmg", "CfmgError", "get_gmg", "solve", "setup_operators", "vcycle", "fcycle", "fill",
           "norm", "normresidual", "set_to_zero", "set_default_msk", "adjoint", "loss_and_grad", "Batch"]


class CfmgError(RuntimeError):
    """A libcfmg call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"cfmg error {code}: {msg}")
        self.code = code


@dataclasses.dataclass
class Param:
    """Param (src/gmg_types.jl:41-59), same names and defaults, plus:

    nlevels        cap on the number of levels (0: the reference's hierarchy)
    precision      "fp64" (bit-identical drop-in) or "mixed" (FP32 cycles in
                   FP64 defect correction)
    residual_norm  "ref_squared" (the reference's sum(msk r^2)/sum(msk b^2))
                   or "l2" (||r||/||b||)
    """

    nx: int = 64
    ny: int = 64
    nz: int = 64
    nh: int = 3
    npre: int = 1
    npost: int = 1
    ndeepest: int = 20
    maxite: int = 15
    tol: float = 1e-10
    omega: float = 0.9
    location: str = "centers"
    case: str = "threed"
    operator: str = "laplacian"
    cycle: str = "v"
    verbose: bool = True
    topology: str = "closed"
    nlevels: int = 0
    precision: str = "fp64"
    residual_norm: str = "ref_squared"

    def desc(self) -> _lib.Desc:
        try:
            return _lib.Desc(
                kase=CASES[self.case], location=LOCATIONS[self.location], op=OPERATORS[self.operator],
                topology=TOPOLOGIES[self.topology], cycle=CYCLES[self.cycle], nx=int(self.nx), ny=int(self.ny),
                nz=int(self.nz), nh=int(self.nh), nlevels=int(self.nlevels or 0), npre=int(self.npre),
                npost=int(self.npost), ndeepest=int(self.ndeepest), maxite=int(self.maxite),
                omega=float(self.omega), tol=float(self.tol), precision=PRECISIONS[self.precision],
                norm_kind=NORMS[self.residual_norm])
        except KeyError as e:
            raise CfmgError(_lib.ERR_ARG, f"unknown symbol {e}") from None


@dataclasses.dataclass(frozen=True)
class Grid:
    """Grid (src/gmg_types.jl:68-84)."""

    nx: int
    ny: int
    nz: int
    nh: int
    tx: int
    ty: int
    tz: int

    @property
    def shape(self):
        return (self.tx, self.ty, self.tz)


class _Fields:
    """mg.data[lev] / mg.oper[lev]: attribute reads download a host copy,
    attribute writes upload."""

    def __init__(self, mg: "Gmg", lev: int, names):
        object.__setattr__(self, "_mg", mg)
        object.__setattr__(self, "_lev", lev)
        object.__setattr__(self, "_names", names)

    def __getattr__(self, name):
        if name in self._names:
            return self._mg.download(self._lev, name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name not in self._names:
            raise AttributeError(name)
        self._mg.upload(self._lev, name, value)


class _OneBased(list):
    """A list indexed 1..n like a Julia Vector."""

    def __getitem__(self, lev):
        if not isinstance(lev, int) or lev < 1 or lev > len(self):
            raise IndexError(f"level {lev} out of range 1..{len(self)}")
        return list.__getitem__(self, lev - 1)


class Gmg:
    """The multigrid object (Gmg, src/gmg_types.jl:121-132) living on the GPU."""

    def __init__(self, param: Param, _handle: Optional[ctypes.c_void_p] = None):
        self._L = _lib.load()
        self.param = param
        self._owned = _handle is None
        if _handle is None:
            d = param.desc()
            h = ctypes.c_void_p()
            rc = self._L.cfmg_create(ctypes.byref(d), ctypes.byref(h))
            if rc != 0:
                raise CfmgError(rc, self._L.cfmg_last_error(None).decode())
        else:
            h = _handle
        self._h = h
        n = ctypes.c_int()
        self._check(self._L.cfmg_nlevels(h, ctypes.byref(n)))
        self.nlevels = n.value
        levels = []
        for lev in range(1, self.nlevels + 1):
            dims = (ctypes.c_int * 7)()
            self._check(self._L.cfmg_level_dims(h, lev, dims))
            levels.append(Grid(*dims))
        self.levels = _OneBased(levels)
        self.data = _OneBased(_Fields(self, lev, ("x", "r", "b", "y")) for lev in range(1, self.nlevels + 1))
        self.oper = _OneBased(_Fields(self, lev, ("diag", "idiag", "Rcoef", "Pcoef", "msk", "kappa"))
                              for lev in range(1, self.nlevels + 1))
        # the four per-level function tables (src/gmg_types.jl:128-131)
        self.smoother = _OneBased(_smoother for _ in range(self.nlevels))
        self.residual = _OneBased(_residual for _ in range(self.nlevels))
        self.restriction = _OneBased(_restriction for _ in range(self.nlevels))
        self.prolongation = _OneBased(_prolongation for _ in range(self.nlevels))

    # --- plumbing
    def _check(self, rc: int):
        if rc != 0:
            raise CfmgError(rc, self._L.cfmg_last_error(self._h).decode())

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and getattr(self, "_owned", True):
            self._L.cfmg_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def shape(self, lev: int):
        return self.levels[lev].shape

    def upload(self, lev: int, name: str, arr) -> None:
        g = self.levels[lev]
        dtype = np.uint8 if name == "msk" else np.float64
        a = np.asfortranarray(np.asarray(arr, dtype=dtype))
        if a.shape != g.shape:
            if a.size != g.tx * g.ty * g.tz:
                raise CfmgError(_lib.ERR_ARG, f"{name}: shape {a.shape} != {g.shape}")
            a = np.asfortranarray(a.reshape(g.shape, order="F"))
        self._check(self._L.cfmg_upload(self._h, lev, FIELDS[name], a.ctypes.data_as(ctypes.c_void_p)))

    def upload_ptr(self, lev: int, name: str, ptr: int) -> None:
        """Upload from a raw host or device address (the caller keeps it alive)."""
        self._check(self._L.cfmg_upload(self._h, lev, FIELDS[name], ctypes.c_void_p(ptr)))

    def download(self, lev: int, name: str) -> np.ndarray:
        g = self.levels[lev]
        out = np.empty(g.shape, dtype=np.uint8 if name == "msk" else np.float64, order="F")
        self._check(self._L.cfmg_download(self._h, lev, FIELDS[name], out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def download_ptr(self, lev: int, name: str, ptr: int) -> None:
        self._check(self._L.cfmg_download(self._h, lev, FIELDS[name], ctypes.c_void_p(ptr)))

    def field_ptr(self, lev: int, name: str) -> int:
        p = ctypes.c_void_p()
        self._check(self._L.cfmg_field_ptr(self._h, lev, FIELDS[name], ctypes.byref(p)))
        return p.value

    def bind_level(self, lev: int, diag=None, idiag=None, Rcoef=None, Pcoef=None, msk=None) -> None:
        """Bind coefficients computed by the caller's own setup. Every array
        must hold the level's tx*ty*tz values (the C ABI takes bare pointers,
        so the size is checked here)."""
        keep = []
        g = self.levels[lev]

        def ptr(a, dtype):
            if a is None:
                return None
            a = np.asfortranarray(np.asarray(a, dtype=dtype))
            if a.size != g.tx * g.ty * g.tz:
                raise CfmgError(_lib.ERR_ARG, f"bind_level: {a.size} values for a level of "
                                              f"{g.tx}x{g.ty}x{g.tz} = {g.tx * g.ty * g.tz} cells")
            keep.append(a)
            return a.ctypes.data_as(ctypes.c_void_p)

        self._check(self._L.cfmg_bind_level(self._h, lev, ptr(diag, np.float64), ptr(idiag, np.float64),
                                             ptr(Rcoef, np.float64), ptr(Pcoef, np.float64), ptr(msk, np.uint8)))

    def synchronize(self):
        self._check(self._L.cfmg_synchronize(self._h))

    def set_option(self, name: str, value: int) -> None:
        """Tuning knobs: ``engine_cells`` (levels of at most this many cells
        run in the coarse-level program engine; 0 turns it off),
        ``temporal_blocking`` (5 lean packed passes, 3 first packed form,
        1 scalar passes, 0 off),
        ``coarsest_fp64`` (-1 auto, 0, 1), ``int_residual`` (1 fixed-point
        level-1 residual of the mixed loop, 0 FP64 arithmetic), ``host_loop``
        (1: the solve loop iterates from the host, one graph per iteration),
        ``fused_descent`` (1: the last pre-smoothing pass of a descent step
        also forms and restricts the residual, 0: separate kernels),
        ``fused_update`` (1: the cycle's last level-1 post-smoothing pass
        also applies the FP64 solution update, 0: a separate kernel)."""
        self._check(self._L.cfmg_set_option(self._h, _lib.OPTIONS[name], int(value)))

    def set_stream(self, stream_ptr: Optional[int]):
        self._check(self._L.cfmg_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))


# --- function-table entries (the Julia signatures)
def _smoother(mg: Gmg, lev: int, nite: int):
    mg._check(mg._L.cfmg_smooth(mg._h, lev, int(nite)))


def _residual(mg: Gmg, lev: int):
    mg._check(mg._L.cfmg_residual(mg._h, lev))


def _restriction(mg: Gmg, lev: int, field: str):
    mg._check(mg._L.cfmg_restrict(mg._h, lev, FIELDS[field]))


def _prolongation(mg: Gmg, lev: int):
    mg._check(mg._L.cfmg_prolong(mg._h, lev))


# --- public functions
def set_default_msk(mg: Gmg) -> None:
    """set_default_msk! (src/gmg_setup.jl:106-122)."""
    mg._check(mg._L.cfmg_set_default_msk(mg._h))


def setup_operators(mg: Gmg) -> None:
    """setup_operators! (src/gmg_setup.jl:264-287), on the device."""
    mg._check(mg._L.cfmg_setup_operators(mg._h))


def set_to_zero(mg: Gmg, lev: int, field: str) -> None:
    """set_to_zero! (src/operators_at_level.jl:7-10)."""
    mg._check(mg._L.cfmg_zero(mg._h, lev, FIELDS[field]))


def fill(mg: Gmg, lev: int, field: str) -> None:
    """fill! (src/halo.jl:1-15) on a named field of a level."""
    mg._check(mg._L.cfmg_fill(mg._h, lev, FIELDS[field]))


def norm(mg: Gmg, lev: int, field: str) -> float:
    """norm (src/operators_at_level.jl:12-27): sum(msk*x^2), 0 -> 1."""
    out = ctypes.c_double()
    mg._check(mg._L.cfmg_norm(mg._h, lev, FIELDS[field], ctypes.byref(out)))
    return out.value


def normresidual(mg: Gmg, normb: float) -> float:
    """normresidual! (src/operators_at_level.jl:29-36)."""
    out = ctypes.c_double()
    mg._check(mg._L.cfmg_normresidual(mg._h, float(normb), ctypes.byref(out)))
    return out.value


def get_gmg(param: Param) -> Gmg:
    """get_gmg (src/gmg_setup.jl:26-35): hierarchy, default mask, operator
    setup, then every b, x, y, r zeroed."""
    mg = Gmg(param)
    set_default_msk(mg)
    setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("b", "x", "y", "r"):
            set_to_zero(mg, lev, f)
    mg.synchronize()
    return mg


def vcycle(mg: Gmg, lev0: int = 1) -> None:
    """vcycle! (src/gmg_cycles.jl:67-83). lev0 = 1 runs the library's fused
    cycle; other lev0 compose the function tables as the reference does."""
    if lev0 == 1:
        mg._check(mg._L.cfmg_cycle(mg._h, CYCLES["v"]))
        return
    p = mg.param
    for lev in range(lev0, mg.nlevels):
        mg.smoother[lev](mg, lev, p.npre)
        mg.residual[lev](mg, lev)
        mg.restriction[lev](mg, lev, "r")
        set_to_zero(mg, lev + 1, "x")
    mg.smoother[mg.nlevels](mg, mg.nlevels, p.ndeepest)
    for lev in range(mg.nlevels - 1, lev0 - 1, -1):
        mg.prolongation[lev](mg, lev)
        mg.smoother[lev](mg, lev, p.npost)


def fcycle(mg: Gmg) -> None:
    """fcycle! (src/gmg_cycles.jl:85-100)."""
    mg._check(mg._L.cfmg_cycle(mg._h, CYCLES["f"]))


def cycle(mg: Gmg, kind: Optional[str] = None) -> None:
    mg._check(mg._L.cfmg_cycle(mg._h, CYCLES[kind or mg.param.cycle]))


def solve(mg: Gmg, history: bool = False, tol: Optional[float] = None, maxite: Optional[int] = None,
          residual_norm: Optional[str] = None):
    """solve!(mg) (src/gmg_solver.jl:9-42): returns (res, nite), plus the
    per-cycle residual history when ``history`` is true. ``tol``, ``maxite``
    and ``residual_norm`` override the Param's for this and later solves
    (cfmg_solve_tol)."""
    res = ctypes.c_double()
    nite = ctypes.c_int()
    if tol is not None or maxite is not None or residual_norm is not None:
        mg.param = dataclasses.replace(mg.param, tol=mg.param.tol if tol is None else float(tol),
                                       maxite=mg.param.maxite if maxite is None else int(maxite),
                                       residual_norm=residual_norm or mg.param.residual_norm)
        hist = (ctypes.c_double * (mg.param.maxite + 1))()
        mg._check(mg._L.cfmg_solve_tol(mg._h, mg.param.tol, mg.param.maxite, NORMS[mg.param.residual_norm],
                                       ctypes.byref(res), ctypes.byref(nite), hist))
    else:
        hist = (ctypes.c_double * (mg.param.maxite + 1))()
        mg._check(mg._L.cfmg_solve(mg._h, ctypes.byref(res), ctypes.byref(nite), hist))
    if mg.param.verbose:
        print(" ----------------\n  ite     res    \n ----------------")
        for k in range(nite.value + 1):
            print(f" {k:3d}   {hist[k]:.3e}")
    if history:
        return res.value, nite.value, np.array(hist[: nite.value + 1])
    return res.value, nite.value


def adjoint(mg: Gmg, g):
    """Backward pass of ``solve(mg)`` (the body of a ChainRulesCore rrule on a
    Julia host): with the cotangent g = dL/dx of level 1, returns
    (dL/db, dL/dkappa); dL/dkappa is None unless the operator is "varcoef".
    Needs a preceding forward ``solve(mg)``; the forward x and b are kept."""
    shape = mg.shape(1)
    ga = np.asfortranarray(np.asarray(g, dtype=np.float64).reshape(shape, order="F"))
    gb = np.empty(shape, dtype=np.float64, order="F")
    vc = mg.param.operator == "varcoef"
    gk = np.empty(shape, dtype=np.float64, order="F") if vc else None
    res = ctypes.c_double()
    nite = ctypes.c_int()
    mg._check(mg._L.cfmg_adjoint(mg._h, ga.ctypes.data_as(ctypes.c_void_p), gb.ctypes.data_as(ctypes.c_void_p),
                                 gk.ctypes.data_as(ctypes.c_void_p) if vc else None, ctypes.byref(res),
                                 ctypes.byref(nite)))
    return gb, gk


def _wet_mean_removed(x, msk):
    w = msk.astype(bool)
    y = np.where(w, x, 0.0)
    if w.any():
        y[w] -= y[w].mean()
    return y


def loss_and_grad(mg: Gmg, b, xstar, kappa=None):
    """L = 1/2 sum_wet (P x - x*)^2 with A(kappa) x = b and P the wet-mean
    projection (cell-centred) or the mask (vertex-centred); returns
    (L, dL/db, dL/dkappa) from one forward and one adjoint solve."""
    if kappa is not None:
        mg.oper[1].kappa = kappa
        setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                set_to_zero(mg, lev, f)
    msk = mg.download(1, "msk")
    mg.data[1].b = b
    set_to_zero(mg, 1, "x")
    solve(mg)
    x = mg.data[1].x
    neumann = mg.param.location == "centers"
    px = _wet_mean_removed(x, msk) if neumann else x * msk
    d = (px - xstar) * msk
    loss = 0.5 * float(np.sum(d * d))
    gb, gk = adjoint(mg, d)
    return loss, gb, gk


class Batch:
    """Many independent 2D masked solves of uneven sizes sharing one Param
    (precision "mixed"), run in one launch of the batched engine.

    ``batch.instance(i)`` is a Gmg for instance i (upload its mask, call
    setup_operators, upload b, read x back). ``batch.solve()`` returns
    (res, nite, t_done_ms) arrays; t_done_ms is the time from the batch start
    until that instance met its tolerance."""

    def __init__(self, param: Param, nx, ny, nlevels=None):
        self._L = _lib.load()
        self.param = param
        n = len(nx)
        d = param.desc()
        ax = (ctypes.c_int * n)(*[int(v) for v in nx])
        ay = (ctypes.c_int * n)(*[int(v) for v in ny])
        al = (ctypes.c_int * n)(*[int(v) for v in nlevels]) if nlevels is not None else None
        b = ctypes.c_void_p()
        rc = self._L.cfmg_batch_create(ctypes.byref(d), n, ax, ay, al, ctypes.byref(b))
        if rc != 0:
            raise CfmgError(rc, self._L.cfmg_last_error(None).decode())
        self._b = b
        self.n = n
        self._inst = []
        for i in range(n):
            h = ctypes.c_void_p()
            self._check(self._L.cfmg_batch_instance(b, i, ctypes.byref(h)))
            p = dataclasses.replace(param, nx=int(nx[i]), ny=int(ny[i]),
                                    nlevels=int(nlevels[i]) if nlevels is not None else param.nlevels)
            self._inst.append(Gmg(p, _handle=h))

    def _check(self, rc):
        if rc != 0:
            raise CfmgError(rc, self._L.cfmg_batch_last_error(self._b).decode())

    def instance(self, i: int) -> Gmg:
        return self._inst[i]

    def solve(self, from_zero: bool = True):
        res = np.zeros(self.n)
        nite = np.zeros(self.n, dtype=np.int32)
        t = np.zeros(self.n)
        self._check(self._L.cfmg_batch_solve(self._b, 1 if from_zero else 0, res.ctypes.data_as(ctypes.c_void_p),
                                             nite.ctypes.data_as(ctypes.c_void_p),
                                             t.ctypes.data_as(ctypes.c_void_p)))
        return res, nite, t

    def set_option(self, name: str, value: int) -> None:
        """Batch options: "host_loop" (1: the host repeats the lockstep
        iteration instead of the graph's while node; for profilers),
        "coarse_runs" (1, default: each instance's coarse-level steps run as
        one block per run of steps; 0: a launch per step), "interleave" (1,
        default: work tables list chunk c of every instance before chunk
        c + 1; 0: each instance's chunks together). Same values either way."""
        self._check(self._L.cfmg_batch_set_option(self._b, _lib.BATCH_OPTIONS[name], int(value)))

    def close(self):
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            for g in self._inst:
                g._h = None
            self._L.cfmg_batch_destroy(b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
