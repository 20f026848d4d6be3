"""Masks, right-hand sides and known-answer scenarios of CFMultigrid's tests.

Restated in numpy from the reference test suite:
  * get_closed_domain / get_circular_domain / get_mask_at_corners /
    subtract_mean!        -- test/test_RP.jl:46-160
  * get_spherical_domain / get_mask_at_3Dcorners -- test/test_3d.jl:15-51
  * the scenario drivers test_solve (test/tests.jl:4-32), test_convergence
    (test/test_RP.jl:162-202), run_3d_test (test/test_3d.jl:53-119) and
    run_topology (test/test_topology.jl:24-88).

Arrays use Fortran order, shape (tx, ty, tz); index [i-1, j-1, k-1] is
Julia's [i, j, k]. Scenarios are backend-neutral: ``run_scenario`` drives any
object with the small adapter interface used below (the CPU oracle or the
CUDA library).
"""
from __future__ import annotations

import dataclasses
import hashlib
import json
import os
from typing import Callable, Optional

import numpy as np


def get_closed_domain(shape, nh=3):
    msk = np.zeros(shape, dtype=np.uint8, order="F")
    msk[nh:shape[0] - nh, nh:shape[1] - nh, :] = 1
    return msk


def get_circular_domain(shape, nh=3, radius=0.5):
    msk = get_closed_domain(shape, nh)
    nx, ny, nz = shape
    dx = 1.0 / (nx - 2 * nh)
    dy = 1.0 / (ny - 2 * nh)
    i = np.arange(nh + 1, nx - nh + 2)  # Julia 1+nh : nx-nh+1
    j = np.arange(nh + 1, ny - nh + 2)
    x = (i - nh - 0.5) * dx
    y = (j - nh - 0.5) * dy
    d2 = ((x - 0.5) * (x - 0.5))[:, None] + ((y - 0.5) * (y - 0.5))[None, :]
    inside = (d2 < radius * radius).astype(np.uint8)
    for k in range(nz):
        msk[i[0] - 1:i[-1], j[0] - 1:j[-1], k] = inside
    return msk


def get_mask_at_corners(msk):
    """Vertex wet iff its four cells are wet (test/test_RP.jl:46-54). Like the
    Julia version, every k-plane reads the cells of plane k=1."""
    nx, ny, nz = msk.shape
    m = msk[:, :, 0].astype(np.int32)
    four = m[1:, 1:] + m[:-1, 1:] + m[1:, :-1] + m[:-1, :-1]
    out = np.zeros_like(msk)
    for k in range(nz):
        out[1:, 1:, k] = (four == 4).astype(np.uint8)
    return out


def get_spherical_domain(shape, nh=3, radius=0.5):
    msk = get_closed_domain(shape, nh)
    nx, ny, nz = shape
    dx = 1.0 / (nx - 2 * nh)
    dy = 1.0 / (ny - 2 * nh)
    dz = 1.0 / (nz - 2 * nh)
    i = np.arange(nh + 1, nx - nh + 2)
    j = np.arange(nh + 1, ny - nh + 2)
    k = np.arange(nh + 1, nz - nh + 2)
    x = (i - nh - 0.5) * dx
    y = (j - nh - 0.5) * dy
    z = (k - nh - 0.5) * dz
    d2 = (((x - 0.5) * (x - 0.5))[:, None, None] + ((y - 0.5) * (y - 0.5))[None, :, None]) + \
        ((z - 0.5) * (z - 0.5))[None, None, :]
    msk[i[0] - 1:i[-1], j[0] - 1:j[-1], k[0] - 1:k[-1]] = (d2 < radius * radius).astype(np.uint8)
    return msk


def get_mask_at_3Dcorners(msk):
    m = msk.astype(np.int32)
    eight = (m[1:, 1:, 1:] + m[:-1, 1:, 1:] + m[1:, :-1, 1:] + m[:-1, :-1, 1:] +
             m[1:, 1:, :-1] + m[:-1, 1:, :-1] + m[1:, :-1, :-1] + m[:-1, :-1, :-1])
    out = np.zeros_like(msk)
    out[1:, 1:, 1:] = (eight == 8).astype(np.uint8)
    return out


def subtract_mean(b, msk):
    """subtract_mean! (test/test_RP.jl:153-160), in place."""
    b *= msk
    bmean = b.sum() / float(msk.sum(dtype=np.int64))
    b -= bmean * msk


@dataclasses.dataclass
class Scenario:
    name: str
    param: dict
    rhs: Callable  # (shape, msk, rng) -> b (Fortran order float64)
    custom_msk: Optional[Callable] = None  # shape -> uint8 mask, then setup_operators!
    premask: bool = False  # b .*= msk before subtract_mean!
    mean_removed: bool = False
    expect_res: Optional[float] = None
    atol: Optional[float] = None
    expect_ite: Optional[int] = None
    seed: int = 0


def _dipole_tests_jl(p):
    """test_solve's point charges (test/tests.jl:19-31)."""
    def rhs(shape, msk, rng):
        b = np.zeros(shape, order="F")
        nh = p.get("nh", 3)
        ny = p["ny"]
        i0, i1, j0 = nh + 6, nh + 4, nh + ny // 2
        if p.get("case", "threed") == "threed":
            k0 = nh + 4
            b[i0 - 1, i0 - 1, k0 - 1] = 1.0
            b[i1 - 1, i1 - 1, k0 - 1] = -1.0
        else:
            b[i0 - 1, j0 - 1, 0] = 1.0
            b[i1 - 1, j0 - 1, 0] = -1.0
        return b
    return rhs


def _rhs_test_rp(config):
    """test_convergence's right-hand sides (test/test_RP.jl:174-187)."""
    def rhs(shape, msk, rng):
        nx, ny, nz = shape
        b = np.zeros(shape, order="F")
        if config == "dipole":
            i0, j0 = nx // 2, ny // 2
            b[i0 - 4 - 1, j0 - 1, 0] = -1
            b[i0 + 4 - 1, j0 - 1, 0] = +1
        elif config == "gradient":
            i = np.arange(1, nx + 1, dtype=np.float64)
            b[:] = ((i - 3 - (nx - 6) / 2 - 0.5)[:, None, None]) * msk
        elif config == "random":
            b[:] = rng.standard_normal(shape)
        else:
            raise ValueError(config)
        return b
    return rhs


def _rhs_3d(n, config, case="threed"):
    """run_3d_test / run_topology right-hand sides (test/test_3d.jl:94-110,
    test/test_topology.jl:183-200)."""
    def rhs(shape, msk, rng):
        b = np.zeros(shape, order="F")
        if config == "dipole":
            di = n // 4
            nh = 3
            i0 = nh + n // 2
            k0 = i0 if case == "threed" else 1
            b[i0 - di - 1, i0 - 1, k0 - 1] = 1
            b[i0 + di - 1, i0 - 1, k0 - 1] = -1
        elif config == "random":
            b[:] = rng.standard_normal(shape)
        else:
            nx = shape[0]
            i = np.arange(1, nx + 1, dtype=np.float64)
            b[:] = ((i - 3 - (nx - 6) / 2 - 0.5)[:, None, None]) * msk
        return b
    return rhs


def tests_jl(name, extra, res, atol, ite):
    p = dict(nx=64, ny=64, nz=64, case="threed")
    p.update(extra)
    return Scenario(name, p, _dipole_tests_jl(p), expect_res=res, atol=atol, expect_ite=ite)


def test_rp(n, location, config="dipole", res=None, atol=None, ite=8, seed=0):
    """test_convergence (test/test_RP.jl:162-202, setup_test :101-122)."""
    p = dict(nx=n, ny=n, nz=1, case="twod", cycle="v", tol=1e-12, ndeepest=20, npre=2, npost=2,
             omega=0.92, maxite=15, location=location)

    def custom(shape):
        msk = get_circular_domain(shape)
        return get_mask_at_corners(msk) if location == "vertices" else msk

    return Scenario(f"test_rp_{location}_{n}_{config}", p, _rhs_test_rp(config), custom_msk=custom,
                    mean_removed=True, expect_res=res, atol=atol, expect_ite=ite, seed=seed)


def test_3d(n, location, domain, res, atol, ite):
    """run_3d_test (test/test_3d.jl:53-119): omega ends at 0.84 (:62-63)."""
    p = dict(nx=n, ny=n, nz=n, case="threed", cycle="v", tol=1e-12, ndeepest=20, npre=2, npost=2,
             omega=0.84, maxite=15, location=location)
    custom = None
    if domain == "spherical":
        def custom(shape):
            msk = get_spherical_domain(shape)
            return get_mask_at_3Dcorners(msk) if location == "vertices" else msk
    return Scenario(f"test_3d_{location}_{domain}", p, _rhs_3d(n, "dipole"), custom_msk=custom,
                    premask=True, mean_removed=True, expect_res=res, atol=atol, expect_ite=ite)


def test_topology(n, location, case, res, atol, ite):
    """run_topology (test/test_topology.jl:24-88): omega ends at 0.9."""
    p = dict(nx=n, ny=n, nz=n if case == "threed" else 1, case=case, location=location, cycle="v",
             tol=1e-12, ndeepest=60, npre=2, npost=2, omega=0.9, maxite=15, topology="xperio")
    return Scenario(f"test_perio_{case}_{location}", p, _rhs_3d(n, "dipole", case), premask=True,
                    mean_removed=True, expect_res=res, atol=atol, expect_ite=ite)


def test_rectangular(location, res, atol, ite):
    """run_rectangular (test/test_rectangular.jl:13-76); not in runtests.jl."""
    n = 32
    p = dict(nx=8 * n, ny=n, nz=n, case="threed", location=location, cycle="v", tol=1e-12,
             ndeepest=60, npre=2, npost=2, omega=0.9, maxite=15)
    return Scenario(f"test_rect_{location}", p, _rhs_3d(n, "dipole"), premask=True, mean_removed=True,
                    expect_res=res, atol=atol, expect_ite=ite)


# Every known answer of the reference suite (test/runtests.jl:9-37), plus the
# rectangular pair that the suite does not run.
KNOWN_ANSWERS = [
    tests_jl("test_default", {}, 1.4e-11, 1e-12, 9),
    tests_jl("test_2d_centers", dict(nx=512, ny=512, nz=1, case="twod"), 2.3e-11, 1e-12, 9),
    tests_jl("test_2d_vertices", dict(nx=512, ny=512, nz=1, case="twod", location="vertices"), 9.9e-11, 1e-12, 8),
    test_rp(1024, "centers", "dipole", 1.67e-13, 1e-14, 8),
    test_rp(1024, "vertices", "dipole", 1.639e-13, 1e-14, 8),
    test_3d(128, "centers", "square", 2.55e-13, 1e-14, 6),
    test_3d(128, "vertices", "spherical", 2.60e-13, 1e-14, 6),
    test_topology(32, "vertices", "twod", 2.5e-14, 1e-15, 7),
    test_topology(32, "centers", "twod", 2.7e-14, 1e-15, 7),
    test_topology(32, "vertices", "threed", 3.1e-13, 1e-14, 6),
    test_topology(32, "centers", "threed", 2.7e-13, 1e-13, 6),
]

# Iteration-count-only checks (test/test_RP.jl:16-41); the Julia random
# right-hand sides are unseeded, these use a fixed seed.
ITERATION_ONLY = (
    [test_rp(256, "vertices", c, ite=8) for c in ("dipole", "random", "gradient")]
    + [test_rp(128 * p, "vertices", "dipole", ite=8) for p in range(7, 11)]
    + [test_rp(128 * p, "centers", "random", ite=8, seed=p) for p in range(7, 11)]
)

RECTANGULAR = [
    test_rectangular("centers", 2.6e-13, 1e-14, 6),
    test_rectangular("vertices", 6.9e-13, 1e-14, 6),
]


def _rhs_normal(shape, msk, rng):
    return np.asfortranarray(rng.standard_normal(shape))


# The plain-method benchmark configuration, exactly as stated: 2D cell-centred
# 5-point masked Poisson, 256^2, mask = disk of radius 0.45 N, right-hand
# side N(0,1) from seed 0 on wet cells with the wet mean removed, V-cycle,
# 6 levels, weighted Jacobi omega 0.8 with 2/2 pairs, to 1e-10 relative
# residual: 1e-20 in the reference's squared ratio (src/gmg_solver.jl:29-39).
CONFIG1 = Scenario(
    "config1_256_disk",
    dict(nx=256, ny=256, nz=1, case="twod", location="centers", operator="laplacian", cycle="v", nlevels=6,
         npre=2, npost=2, omega=0.8, ndeepest=20, tol=1e-20, maxite=40),
    _rhs_normal, custom_msk=lambda shape: get_circular_domain(shape, radius=0.45), premask=True,
    mean_removed=True, seed=0)


# Committed oracle solves (tests/golden/make_golden.py): the scenarios whose
# inputs are computed exactly (point charges, gradients; no random right-hand
# side), so that the oracle's result is fixed by IEEE arithmetic alone and is
# the same on every host.
GOLDEN_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_solves.json")


def golden_scenarios():
    """The scenarios whose oracle solve is committed: those with exactly
    computed inputs, plus configuration 1, whose seeded N(0,1) right-hand
    side is committed as a digest (``b_sha256``) so that a change of the
    random stream shows as such."""
    return [sc for sc in KNOWN_ANSWERS + RECTANGULAR + list(ITERATION_ONLY) if "random" not in sc.name] + [CONFIG1]


def field_digest(a) -> str:
    """SHA-256 of a field's FP64 values in column-major order, with -0
    counted as +0 (the comparisons of fields treat the two as equal)."""
    v = np.asarray(a, dtype=np.float64) + 0.0
    return hashlib.sha256(np.ascontiguousarray(v.ravel(order="F")).tobytes()).hexdigest()


def load_golden() -> dict:
    with open(GOLDEN_PATH) as f:
        return json.load(f)


def prepare(mg, sc: Scenario):
    """Replay a scenario's setup on ``mg`` and return the right-hand side.

    ``mg`` must provide: shape(lev), nlevels, get(lev, name), set(lev, name,
    array) and setup_operators(). Mirrors the order of the Julia drivers:
    get_gmg, optional custom mask + setup_operators!, reset_all_levels, rhs,
    optional b .*= msk, optional subtract_mean!.
    """
    shape = mg.shape(1)
    if sc.custom_msk is not None:
        mg.set(1, "msk", sc.custom_msk(shape))
        mg.setup_operators()
    for lev in range(1, mg.nlevels + 1):
        s = mg.shape(lev)
        for f in ("x", "y", "r", "b"):
            mg.set(lev, f, np.zeros(s, order="F"))
    msk = mg.get(1, "msk").astype(np.float64)
    rng = np.random.default_rng(sc.seed)
    b = sc.rhs(shape, msk, rng)
    if sc.premask:
        b *= msk
    if sc.mean_removed:
        subtract_mean(b, msk)
    mg.set(1, "b", b)
    return b


class OracleAdapter:
    """Adapter of the CPU oracle for ``prepare``."""

    def __init__(self, og):
        self.g = og
        self.nlevels = og.nlevels

    def shape(self, lev):
        return self.g.shape(lev)

    def get(self, lev, name):
        return self.g.field(lev, name).copy(order="F")

    def set(self, lev, name, arr):
        self.g.field(lev, name)[...] = arr

    def setup_operators(self):
        self.g.setup_operators()
