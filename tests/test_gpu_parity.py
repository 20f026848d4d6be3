"""CUDA path (libcfmg through its C ABI) against the CPU oracle.

The FP64 form is required to be bit-identical to the oracle pointwise:
every operator (sweep, residual, restriction, prolongation, halo fill) and
the device-side setup coefficients are compared with ``array_equal``, and a
whole solve must reproduce the oracle's iteration count, final x bit for bit
and its residual history to 1e-12 relative (the norms' summation order is
the only difference). Where the scenario's oracle solve is committed
(tests/golden), the solve is also checked against those values.
"""
import math

import numpy as np
import pytest

import fixtures as F
import oracle as O

pytestmark = pytest.mark.gpu

cfmg = pytest.importorskip("cfmg")

HIST_RTOL = 1e-12
# history entries against the oracle's sequential FP64 norm sums: the
# oracle's own summation error on ~1e6 cells reaches ~3e-12
HIST_RTOL_SEQ = 1e-11
GOLDEN = F.load_golden()


class GpuAdapter:
    def __init__(self, mg):
        self.mg = mg
        self.nlevels = mg.nlevels

    def shape(self, lev):
        return self.mg.shape(lev)

    def get(self, lev, name):
        return self.mg.download(lev, name)

    def set(self, lev, name, arr):
        self.mg.upload(lev, name, arr)

    def setup_operators(self):
        cfmg.setup_operators(self.mg)


def gpu_param(p, **kw):
    d = dict(p)
    d.update(kw)
    d.setdefault("verbose", False)
    d["verbose"] = False
    return cfmg.Param(**d)


def both(param_dict, **kw):
    og = O.OracleGmg(dict(param_dict, **kw))
    mg = cfmg.get_gmg(gpu_param(param_dict, **kw))
    return og, mg


CONFIGS = {
    "2d_centers": dict(nx=48, ny=40, nz=1, case="twod"),
    "2d_vertices": dict(nx=48, ny=40, nz=1, case="twod", location="vertices"),
    "2d_centers_xperio": dict(nx=32, ny=24, nz=1, case="twod", topology="xperio"),
    "2d_vertices_xperio": dict(nx=32, ny=24, nz=1, case="twod", location="vertices", topology="xperio"),
    "2d_twolayer": dict(nx=32, ny=32, nz=2, case="twod"),
    "3d_centers": dict(nx=24, ny=16, nz=16, case="threed"),
    "3d_vertices": dict(nx=24, ny=16, nz=16, case="threed", location="vertices"),
    "3d_centers_xperio": dict(nx=16, ny=16, nz=16, case="threed", topology="xperio"),
    "3d_lap9": dict(nx=16, ny=16, nz=16, case="threed", operator="laplacian9"),
    "3d_lap9_vertices": dict(nx=16, ny=16, nz=16, case="threed", operator="laplacian9", location="vertices"),
    "2d_lap9_vertices": dict(nx=64, ny=48, nz=1, case="twod", operator="laplacian9", location="vertices"),
    "2d_lap9_centers": dict(nx=64, ny=48, nz=1, case="twod", operator="laplacian9"),
    "2d_varcoef": dict(nx=48, ny=40, nz=1, case="twod", operator="varcoef"),
    "2d_odd": dict(nx=50, ny=38, nz=1, case="twod", nh=3),
}


def _disk(shape, location):
    msk = F.get_circular_domain(shape, radius=0.45)
    return F.get_mask_at_corners(msk) if location == "vertices" else msk


def _setup_pair(name, custom_mask=True, seed=0):
    p = CONFIGS[name]
    og, mg = both(p)
    if custom_mask and p.get("case") == "twod":
        m = _disk(og.shape(1), p.get("location", "centers"))
        if p.get("operator") == "varcoef":
            rng = np.random.default_rng(seed + 7)
            kap = np.exp(0.5 * rng.standard_normal(og.shape(1))).astype(np.float64)
            kap = np.asfortranarray(kap)
            og.field(1, "kappa")[...] = kap
            mg.upload(1, "kappa", kap)
        og.field(1, "msk")[...] = m
        og.setup_operators()
        mg.upload(1, "msk", m)
        cfmg.setup_operators(mg)
    return og, mg


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_setup_coefficients_bitwise(name):
    og, mg = _setup_pair(name)
    assert og.nlevels == mg.nlevels
    for lev in range(1, og.nlevels + 1):
        for f in ("msk", "diag", "idiag", "Rcoef", "Pcoef", "x", "b", "r"):
            a, b = og.field(lev, f), mg.download(lev, f)
            assert np.array_equal(a, b), (lev, f, np.abs(a.astype(float) - b).max())


def _random_state(og, mg, rng):
    for lev in range(1, og.nlevels + 1):
        shape = og.shape(lev)
        for f in ("x", "b", "y", "r"):
            a = np.asfortranarray(rng.standard_normal(shape))
            og.field(lev, f)[...] = a
            mg.upload(lev, f, a)


def _compare_all(og, mg, what):
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            a, b = og.field(lev, f), mg.download(lev, f)
            assert np.array_equal(a, b), (what, lev, f, np.nanmax(np.abs(a - b)))


@pytest.mark.parametrize("engine", ["engine", "standalone"])
@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_operators_bitwise(name, engine):
    og, mg = _setup_pair(name)
    # small levels run in the coarse-level program engine by default; the
    # standalone variant launches every operator as its own kernel
    mg.set_option("engine_cells", 10**9 if engine == "engine" else 0)
    rng = np.random.default_rng(1)
    _random_state(og, mg, rng)
    L = og.nlevels
    for lev in (1, min(2, L), L):
        og.smooth(lev, 2)
        mg.smoother[lev](mg, lev, 2)
        _compare_all(og, mg, f"smooth{lev}")
        og.residual(lev)
        mg.residual[lev](mg, lev)
        _compare_all(og, mg, f"residual{lev}")
    for lev in range(1, L):
        for field in ("r", "b"):
            og.restrict(lev, field)
            mg.restriction[lev](mg, lev, field)
            _compare_all(og, mg, f"restrict{lev}{field}")
        og.prolong(lev)
        mg.prolongation[lev](mg, lev)
        _compare_all(og, mg, f"prolong{lev}")
    for f in ("x", "r"):
        og.fill(1, f)
        cfmg.fill(mg, 1, f)
    _compare_all(og, mg, "fill")
    for f in ("x", "b", "r"):
        a, b = og.norm(1, f), cfmg.norm(mg, 1, f)
        assert abs(a - b) <= 1e-13 * abs(a), (f, a, b)


@pytest.mark.parametrize("engine_cells", [0, 400, 10**9])
@pytest.mark.parametrize("kind", ["v", "f", "onelev", "twolev", "nlev", "vrec"])
def test_cycles_bitwise(kind, engine_cells):
    og, mg = _setup_pair("2d_centers")
    mg.set_option("engine_cells", engine_cells)  # none / the coarsest levels / all levels in the engine
    rng = np.random.default_rng(2)
    _random_state(og, mg, rng)
    og.cycle(kind)
    cfmg.cycle(mg, kind)
    _compare_all(og, mg, kind)


def _solve_pair(sc, **gpu_kw):
    og = O.OracleGmg(sc.param)
    F.prepare(F.OracleAdapter(og), sc)
    r0 = og.solve()
    mg = cfmg.get_gmg(gpu_param(sc.param, **gpu_kw))
    mg.b_in = F.prepare(GpuAdapter(mg), sc)
    r1 = cfmg.solve(mg, history=True)
    return og, mg, r0, r1


def _exact_ratio(mg):
    """sum(msk r^2)/sum(msk b^2) of the device's final fields, summed exactly."""
    m = mg.download(1, "msk").astype(np.float64).ravel()
    r = mg.download(1, "r").ravel()
    b = mg.download(1, "b").ravel()
    nr = math.fsum(m * r * r) or 1.0
    nb = math.fsum(m * b * b) or 1.0
    return nr / nb


def _check_solve(sc, og, mg, r0, r1):
    (res0, n0, h0), (res1, n1, h1) = r0, r1
    assert n1 == n0
    # pointwise arithmetic is bit-identical: same final solution and residual
    assert np.array_equal(og.x, mg.data[1].x)
    assert np.array_equal(og.field(1, "r"), mg.download(1, "r"))
    # the device norm is a tree sum: within 1e-13 of the exactly rounded
    # ratio; the oracle (like the reference) sums sequentially, which on
    # ~1e6 cells is itself off by up to a few 1e-12
    assert abs(res1 - _exact_ratio(mg)) <= 1e-13 * res1
    np.testing.assert_allclose(h1, h0, rtol=HIST_RTOL_SEQ, atol=0)
    g = GOLDEN.get(sc.name)
    if g is not None:  # the committed oracle solve
        assert F.field_digest(mg.b_in) == g["b_sha256"]
        assert n1 == g["nite"]
        assert F.field_digest(mg.data[1].x) == g["x_sha256"]
        assert F.field_digest(mg.download(1, "r")) == g["r_sha256"]
        np.testing.assert_allclose(h1, g["hist"], rtol=HIST_RTOL_SEQ, atol=0)


@pytest.mark.parametrize("sc", F.KNOWN_ANSWERS + F.RECTANGULAR, ids=lambda s: s.name)
def test_known_answer_solve(sc):
    og, mg, r0, r1 = _solve_pair(sc)
    assert r1[1] == sc.expect_ite
    assert abs(r1[0] - sc.expect_res) <= sc.atol
    _check_solve(sc, og, mg, r0, r1)


@pytest.mark.parametrize("sc", F.ITERATION_ONLY[:3], ids=lambda s: s.name)
def test_iteration_only_solve(sc):
    og, mg, r0, r1 = _solve_pair(sc)
    assert r1[1] == sc.expect_ite
    _check_solve(sc, og, mg, r0, r1)


@pytest.mark.parametrize("host_loop", [0, 1])
def test_config1_plain_method_exact(host_loop):
    """Configuration 1 exactly as stated (256^2 cell-centred 5-point, disk
    0.45 N, seed-0 N(0,1) right-hand side, V-cycle 2/2, 6 levels, omega 0.8,
    1e-10 relative residual) in the FP64 drop-in: the oracle's iteration
    count, x and r bit for bit, and the residual history within 1e-12
    relative (68,644 cells: the sequential sum's own error is far below it),
    also against the committed oracle solve. host_loop 1: one graph launch
    per iteration instead of the device-side loop."""
    sc = F.CONFIG1
    og, mg, r0, r1 = _solve_pair(sc)
    if host_loop:
        mg.set_option("host_loop", 1)
        cfmg.set_to_zero(mg, 1, "x")
        r1 = cfmg.solve(mg, history=True)
    _check_solve(sc, og, mg, r0, r1)
    np.testing.assert_allclose(r1[2], r0[2], rtol=HIST_RTOL, atol=0)
    np.testing.assert_allclose(r1[2], GOLDEN[sc.name]["hist"], rtol=HIST_RTOL, atol=0)
    assert r1[0] <= sc.param["tol"]
