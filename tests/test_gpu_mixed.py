"""Mixed-precision form: FP32 V/F-cycles inside FP64 defect correction.

Its result is checked against the CPU oracle's FP64 solve of the same
problem: the true FP64 residual must meet the tolerance, and the solution
(wet mean removed for the singular cell-centred case) must agree with the
oracle's FP64 solution to the accuracy the tolerance implies.
"""
import numpy as np
import pytest

import fixtures as F
import oracle as O

pytestmark = pytest.mark.gpu
cfmg = pytest.importorskip("cfmg")

CASES = {
    "config1_256_centers_v": (dict(nx=256, ny=256, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8,
                                   nlevels=6), "disk"),
    "config2_512_vertices_lap9_f": (dict(nx=512, ny=512, nz=1, case="twod", location="vertices",
                                         operator="laplacian9", cycle="f", npre=3, npost=3, omega=0.8,
                                         nlevels=7), "disk"),
    "3d_48_centers_v": (dict(nx=48, ny=48, nz=48, case="threed", cycle="v", npre=2, npost=2, omega=0.8), None),
    # 3D vertex-centred (Dirichlet) operators: the 7-point one takes the
    # streaming blocked passes when asked, the 19-point one always runs its
    # one pair of sweeps per call as separate kernels
    "3d_32_vertices_v": (dict(nx=32, ny=32, nz=32, case="threed", location="vertices", cycle="v", npre=2,
                              npost=2, omega=0.8), None),
    "3d_32_vertices_lap9_v": (dict(nx=32, ny=32, nz=32, case="threed", location="vertices",
                                   operator="laplacian9", cycle="v", npre=2, npost=2, omega=0.8), None),
    "2d_xperio_vertices_v": (dict(nx=64, ny=64, nz=1, case="twod", location="vertices", topology="xperio",
                                  cycle="v", npre=2, npost=2, omega=0.9, ndeepest=60), None),
    # ragged 3D: plane and column counts that are no multiple of the sweeps' blocks
    "3d_40x36x26_centers_f": (dict(nx=40, ny=36, nz=26, case="threed", cycle="f", npre=2, npost=2, omega=0.8,
                                   nlevels=3), None),
    # odd row length (tx = 39): no TMA-staged residual pass
    "3d_odd_33x30x20_centers_v": (dict(nx=33, ny=30, nz=20, case="threed", cycle="v", npre=2, npost=2,
                                       omega=0.8, nlevels=3), None),
}


# larger cases for the bit-identity tests only (no oracle solve): several
# waves of tiles per pass, so that an ordering fault between tiles shows
BIG_CASES = {
    "config2_2048_vertices_lap9_f": (dict(nx=2048, ny=2048, nz=1, case="twod", location="vertices",
                                          operator="laplacian9", cycle="f", npre=3, npost=3, omega=0.8,
                                          nlevels=5), "disk"),
    "config1_1024_centers_v": (dict(nx=1024, ny=1024, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8,
                                    nlevels=6), "disk"),
    # 3D 19-point: the streaming pair pass over two tiles in i and j and several k chunks
    "3d_70x44x30_centers_lap9_f": (dict(nx=70, ny=44, nz=30, case="threed", operator="laplacian9", cycle="f",
                                        npre=2, npost=2, omega=0.8, nlevels=3), None),
    # x-periodic, wet everywhere: the blocked passes' tiles wrap across the seam
    "2d_xperio_512_centers_v": (dict(nx=512, ny=256, nz=1, case="twod", topology="xperio", cycle="v", npre=2,
                                     npost=2, omega=0.8, nlevels=5), None),
    # odd widths: no tile takes the aligned vector path
    "2d_odd_301x203_vertices_lap9_f": (dict(nx=301, ny=203, nz=1, case="twod", location="vertices",
                                            operator="laplacian9", cycle="f", npre=3, npost=3, omega=0.8,
                                            nlevels=5), "disk"),
    "2d_odd_301x203_centers_v": (dict(nx=301, ny=203, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8,
                                      nlevels=5), "disk"),
    # two :twod layers (one launch covers both; no fused descent)
    "2d_twolayer_256_centers_v": (dict(nx=256, ny=256, nz=2, case="twod", cycle="v", npre=2, npost=2, omega=0.8,
                                       nlevels=5), "disk"),
}


def _mask(p, shape, kind):
    if kind is None:
        return None
    m = F.get_circular_domain(shape, radius=0.45)
    return F.get_mask_at_corners(m) if p.get("location") == "vertices" else m


def _wet_mean_removed(x, m):
    w = m.astype(bool)
    y = x.copy()
    y[w] -= y[w].mean()
    y[~w] = 0
    return y


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_matches_fp64_oracle(name):
    base, mkind = CASES[name]
    tol = 1e-10
    p = dict(base, tol=tol * tol, maxite=40)  # oracle: squared rule, same threshold
    og = O.OracleGmg(p)
    shape = og.shape(1)
    custom = _mask(base, shape, mkind)
    if custom is not None:
        og.field(1, "msk")[...] = custom
        og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    msk = og.field(1, "msk").copy()
    b = np.asfortranarray(np.random.default_rng(5).standard_normal(shape)) * msk
    F.subtract_mean(b, msk.astype(np.float64))
    og.field(1, "b")[...] = b
    res0, n0, _ = og.solve()

    mg = cfmg.get_gmg(cfmg.Param(**base, tol=tol, maxite=40, residual_norm="l2", precision="mixed", verbose=False))
    if custom is not None:
        mg.oper[1].msk = custom
        cfmg.setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(mg, lev, f)
    assert np.array_equal(mg.download(1, "msk"), msk)
    mg.data[1].b = b
    res1, n1, hist = cfmg.solve(mg, history=True)
    assert res1 <= tol, (res1, hist)
    # the reported residual is the true FP64 one: recompute it on the oracle
    x = mg.data[1].x
    og.field(1, "x")[...] = x
    nb = og.norm(1, "b")
    true_res = og.normresidual(nb) ** 0.5
    assert true_res <= tol * 1.0001, true_res
    assert abs(true_res - res1) <= 1e-6 * res1 + 1e-16
    # iteration count within one of the FP64 form's
    assert abs(n1 - n0) <= 1, (n1, n0)
    # solution agreement with the FP64 oracle
    xo = O.OracleGmg(p)  # fresh solve for x (og.x was overwritten)
    if custom is not None:
        xo.field(1, "msk")[...] = custom
        xo.setup_operators()
    for lev in range(1, xo.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            xo.field(lev, f)[...] = 0.0
    xo.field(1, "b")[...] = b
    xo.solve()
    singular = base.get("location", "centers") == "centers"
    a = _wet_mean_removed(x, msk) if singular else x * msk
    c = _wet_mean_removed(xo.x.copy(), msk) if singular else xo.x * msk
    err = np.linalg.norm(a - c) / np.linalg.norm(c)
    assert err <= 1e-6, err


@pytest.mark.parametrize("name", ["config1_256_centers_v", "config2_512_vertices_lap9_f", "3d_48_centers_v",
                                  "config2_2048_vertices_lap9_f", "config1_1024_centers_v", "2d_xperio_vertices_v",
                                  "2d_xperio_512_centers_v", "2d_odd_301x203_vertices_lap9_f",
                                  "2d_odd_301x203_centers_v", "2d_twolayer_256_centers_v", "3d_32_vertices_v",
                                  "3d_32_vertices_lap9_v", "3d_70x44x30_centers_lap9_f"])
def test_temporal_blocking_is_bit_identical(name):
    """The temporally blocked FP32 smoother (all sweeps of a call in one
    shared-memory pass), and its form whose last pre-smoothing pass also
    forms and restricts the residual, must give the same FP32 fields as one
    kernel per operator, hence the same solve bit for bit."""
    base, mkind = {**CASES, **BIG_CASES}[name]
    out = []
    # packed FP32x2 passes (lean form with and without the fused residual and
    # restriction, with and without the FP64 solution update in the last
    # level-1 pass; first form; 3D: + streaming passes, for the 19-point
    # operator its one-pair pass), scalar passes, one kernel per sweep
    if base.get("case") == "threed":
        runs = ((4, 1, 1), (1, 1, 1), (0, 1, 1))
    else:
        runs = ((5, 1, 1), (5, 1, 0), (5, 0, 1), (3, 1, 1), (1, 1, 1), (0, 1, 1))
    for tb, fuse, upd in runs:
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed",
                                     verbose=False))
        mg.set_option("engine_cells", 2000)  # keep the fine levels out of the engine
        mg.set_option("temporal_blocking", tb)
        mg.set_option("fused_descent", fuse)
        mg.set_option("fused_update", upd)
        shape = mg.shape(1)
        custom = _mask(base, shape, mkind)
        if custom is not None:
            mg.oper[1].msk = custom
            cfmg.setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk").astype(np.float64)
        b = np.asfortranarray(np.random.default_rng(9).standard_normal(shape)) * msk
        F.subtract_mean(b, msk)
        mg.data[1].b = b
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((hist, mg.data[1].x))
    for k in range(1, len(out)):
        assert np.array_equal(out[0][0], out[k][0]), k
        assert np.array_equal(out[0][1], out[k][1]), k


@pytest.mark.parametrize("name", ["config1_256_centers_v", "config2_512_vertices_lap9_f", "3d_48_centers_v"])
def test_integer_residual_matches_fp64_residual(name):
    """The fixed-point level-1 residual (default) against the FP64-arithmetic
    one: same iteration count, residual histories to 1e-4, same solution.
    The FP32 right-hand sides of the two forms differ in the last bit where
    the cell-centred wet mean comes off (after or before the rounding to
    FP32), so the FP32 corrections, and with them the histories, drift
    apart at the 1e-6 level."""
    base, mkind = CASES[name]
    out = {}
    for on in (1, 0):
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed",
                                     verbose=False))
        custom = _mask(base, mg.shape(1), mkind)
        if custom is not None:
            mg.oper[1].msk = custom
            cfmg.setup_operators(mg)
            for lev in range(1, mg.nlevels + 1):
                for f in ("x", "y", "r", "b"):
                    cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk")
        b = np.asfortranarray(np.random.default_rng(9).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk.astype(np.float64))
        mg.data[1].b = b
        mg.set_option("int_residual", on)
        res, n, hist = cfmg.solve(mg, history=True)
        out[on] = (res, n, hist, mg.data[1].x, msk.astype(bool))
    (r1, n1, h1, x1, w), (r0, n0, h0, x0, _) = out[1], out[0]
    assert r1 <= 1e-10 and r0 <= 1e-10 and n1 == n0, (r1, r0, n1, n0)
    np.testing.assert_allclose(h1, h0, rtol=1e-4)
    singular = base.get("location", "centers") == "centers"
    a = _wet_mean_removed(x1, w) if singular else x1 * w
    c = _wet_mean_removed(x0, w) if singular else x0 * w
    assert np.linalg.norm(a - c) <= 1e-8 * np.linalg.norm(c)


@pytest.mark.parametrize("name", ["3d_48_centers_v", "3d_32_vertices_v", "3d_40x36x26_centers_f",
                                  "3d_odd_33x30x20_centers_v"])
def test_staged_residual_matches_strip_residual(name):
    """The TMA-staged 3D residual pass (default) against the row-strip pass:
    per cell the same exact integer residual and FP32 right-hand side; the
    norm's per-thread partial sums are combined in another order, so the
    initial residual agrees to 1e-13, and the histories (through the last
    bit of the wet mean) to 1e-6, with the same iteration count and the
    same solution to 1e-8. An odd row length keeps the strip pass: bit for
    bit."""
    base, mkind = CASES[name]
    out = {}
    for on in (1, 2, 0):  # one and two tile rows per thread; the strip pass
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed",
                                     verbose=False))
        msk = mg.download(1, "msk")
        b = np.asfortranarray(np.random.default_rng(27).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk.astype(np.float64))
        mg.data[1].b = b
        mg.set_option("staged_residual", on)
        res, n, hist = cfmg.solve(mg, history=True)
        out[on] = (res, n, hist, mg.data[1].x, msk.astype(bool), mg.shape(1)[0])
    r0, n0, h0, x0, w, tx = out[0]
    for on in (1, 2):
        r1, n1, h1, x1, _, _ = out[on]
        assert r1 <= 1e-10 and r0 <= 1e-10 and n1 == n0, (on, r1, r0, n1, n0)
        if tx % 2:
            assert np.array_equal(h1, h0) and np.array_equal(x1, x0)
            continue
        np.testing.assert_allclose(h1[0], h0[0], rtol=1e-13)
        np.testing.assert_allclose(h1, h0, rtol=1e-6)
        singular = base.get("location", "centers") == "centers"
        a = _wet_mean_removed(x1, w) if singular else x1 * w
        c = _wet_mean_removed(x0, w) if singular else x0 * w
        assert np.linalg.norm(a - c) <= 1e-8 * np.linalg.norm(c)


@pytest.mark.parametrize("case", ["3d_v", "3d_f", "2d_config2_512", "2d_config1_centers"])
def test_skip_dry_is_bit_identical(case):
    """Skipping groups of dry cells (3D: four-cell sweeps with per-(plane run,
    quad) wet flags, the FP64 update with the dry cells' max |x| taken once,
    the wet-mean shift, the staged residual's dry tile runs, the residual-
    restriction's dry coarse cells; 2D and 3D: the prolongation's dry
    parents, the strip residual's dry tasks) gives the full passes' history
    and solution: on the configuration-3 recipe (coastline cut by a bottom
    topography, most of the box dry), the configuration-2 coastline at 512^2
    and a cell-centred disk."""
    import workloads as W

    if case.startswith("3d"):
        param, vmsk, noise = W.config3(64, 64, 32, nlevels=4)
        param = dict(param, cycle=case[-1])
    elif case == "2d_config2_512":
        param, vmsk, noise = W.config2(512, nlevels=4)
    else:
        base, _ = CASES["config1_256_centers_v"]
        param = dict(base)
        vmsk = None
        noise = None
    out = []
    for skip in (1, 0):
        mg = cfmg.get_gmg(cfmg.Param(**param, tol=1e-10, maxite=60, residual_norm="l2", precision="mixed",
                                     verbose=False))
        mg.set_option("engine_cells", 2000)  # fine levels as standalone kernels
        mg.set_option("skip_dry", skip)
        mg.oper[1].msk = vmsk if vmsk is not None else _mask(param, mg.shape(1), "disk")
        cfmg.setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(mg, lev, f)
        if noise is not None:
            mg.data[1].b = W.rhs(noise, mg.download(1, "msk"))
        else:
            msk = mg.download(1, "msk").astype(np.float64)
            b = np.asfortranarray(np.random.default_rng(31).standard_normal(mg.shape(1))) * msk
            F.subtract_mean(b, msk)
            mg.data[1].b = b
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((res, n, hist, mg.data[1].x))
        mg.close()
    assert out[0][0] <= 1e-10 and out[0][1] == out[1][1] and out[0][0] == out[1][0]
    assert np.array_equal(out[0][2], out[1][2]) and np.array_equal(out[0][3], out[1][3])


@pytest.mark.parametrize("name", ["config1_256_centers_v", "config2_512_vertices_lap9_f", "3d_48_centers_v",
                                  "3d_32_vertices_v", "2d_twolayer_256_centers_v"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_small_smooth_is_bit_identical(name, precision):
    """The coarsest solve run by one block in shared memory (the default for
    small levels) gives the engine's separate sweeps' history and solution
    bit for bit, in the mixed form (FP64 or FP32 coarsest) and the FP64
    drop-in."""
    base, mkind = {**CASES, **BIG_CASES}[name]
    out = []
    for small in (4, 2, 0):  # the coarsest solve only; every call of 2 pairs too; never
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision=precision,
                                     verbose=False))
        mg.set_option("small_smooth", small)
        custom = _mask(base, mg.shape(1), mkind)
        if custom is not None:
            mg.oper[1].msk = custom
            cfmg.setup_operators(mg)
            for lev in range(1, mg.nlevels + 1):
                for f in ("x", "y", "r", "b"):
                    cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk").astype(np.float64)
        b = np.asfortranarray(np.random.default_rng(33).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk)
        mg.data[1].b = b
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((res, n, hist, mg.data[1].x))
    for o in out[1:]:
        assert o[1] == out[0][1] and o[0] == out[0][0]
        assert np.array_equal(o[2], out[0][2]) and np.array_equal(o[3], out[0][3])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solve_graph_matches_host_loop(precision):
    """The whole solve! loop as one graph launch (a while node with the
    stopping test on the device) gives the host-driven loop's history and
    solution bit for bit."""
    base, mkind = CASES["config1_256_centers_v"]
    out = []
    for host in (0, 1):
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision=precision,
                                     verbose=False))
        mg.oper[1].msk = _mask(base, mg.shape(1), mkind)
        cfmg.setup_operators(mg)
        for lev in range(1, mg.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk").astype(np.float64)
        b = np.asfortranarray(np.random.default_rng(3).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk)
        mg.data[1].b = b
        mg.set_option("host_loop", host)
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((res, n, hist, mg.data[1].x))
    assert out[0][1] == out[1][1] and out[0][0] == out[1][0]
    assert np.array_equal(out[0][2], out[1][2])
    assert np.array_equal(out[0][3], out[1][3])


def _profile(mg, cls, lev, precision, fn):
    import ctypes

    from cfmg import _lib

    L = mg._L
    mg._check(L.cfmg_profile(mg.handle, _lib.KERNEL_CLASSES[cls], lev, _lib.PRECISIONS[precision]))
    fn()
    n, ms = ctypes.c_longlong(), ctypes.c_double()
    mg._check(L.cfmg_profile_read(mg.handle, ctypes.byref(n), ctypes.byref(ms)))
    mg._check(L.cfmg_profile(mg.handle, -1, 0, 0))
    return n.value, ms.value


def test_fused_descent_profile_class():
    """Fused descent passes are counted under CFMG_K_DESCENT and the plain
    smoothing passes under CFMG_K_SWEEP; with the fusion off no descent pass
    runs and the level-1 FP32 residual kernel does."""
    base, mkind = CASES["config2_512_vertices_lap9_f"]
    mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed", verbose=False))
    shape = mg.shape(1)
    mg.oper[1].msk = _mask(base, shape, mkind)
    cfmg.setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            cfmg.set_to_zero(mg, lev, f)
    msk = mg.download(1, "msk").astype(np.float64)
    b = np.asfortranarray(np.random.default_rng(5).standard_normal(shape)) * msk
    F.subtract_mean(b, msk)
    mg.data[1].b = b

    def solve():
        cfmg.set_to_zero(mg, 1, "x")
        return cfmg.solve(mg)

    counts = {}
    for fuse in (1, 0):
        mg.set_option("fused_descent", fuse)
        counts[fuse] = {c: _profile(mg, c, 1, "mixed", solve)[0] for c in ("descent", "sweep", "residual")}
    assert counts[1]["descent"] > 0 and counts[1]["sweep"] > 0 and counts[1]["residual"] == 0, counts
    assert counts[0]["descent"] == 0 and counts[0]["residual"] > 0, counts
    assert counts[0]["sweep"] == counts[1]["sweep"] + counts[1]["descent"], counts


def test_fused_update_replaces_the_update_kernel():
    """With the FP64 solution update in the cycle's last level-1
    post-smoothing pass, the separate update kernel (a level-1 conversion
    launch) no longer runs, one fewer per iteration, and the solve is the
    same bit for bit."""
    base, mkind = CASES["config2_512_vertices_lap9_f"]
    mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed", verbose=False))
    shape = mg.shape(1)
    mg.oper[1].msk = _mask(base, shape, mkind)
    cfmg.setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            cfmg.set_to_zero(mg, lev, f)
    msk = mg.download(1, "msk").astype(np.float64)
    b = np.asfortranarray(np.random.default_rng(5).standard_normal(shape)) * msk
    F.subtract_mean(b, msk)
    mg.data[1].b = b
    out = {}
    for upd in (1, 0):
        mg.set_option("fused_update", upd)
        got = {}

        def solve():
            cfmg.set_to_zero(mg, 1, "x")
            got["r"] = cfmg.solve(mg, history=True)

        nconv, _ = _profile(mg, "convert", 1, "mixed", solve)
        out[upd] = (nconv, got["r"], mg.data[1].x)
    (c1, (r1, n1, h1), x1), (c0, (r0, n0, h0), x0) = out[1], out[0]
    assert r1 <= 1e-10 and n1 == n0, (r1, n1, n0)
    assert c0 - c1 == n0, (c0, c1, n0)
    assert np.array_equal(h1, h0)
    assert np.array_equal(x1, x0)


@pytest.mark.parametrize("name", ["config2_512_vertices_lap9_f", "config1_256_centers_v"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dependent_launch_is_bit_identical(name, precision):
    """Kernels launched as programmatic dependents of their predecessor
    (the default) give the plain stream order's history and solution bit
    for bit, in the graph-launched loop and in the host loop."""
    base, mkind = CASES[name]
    out = []
    for dep, host in ((1, 0), (0, 0), (1, 1)):
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision=precision,
                                     verbose=False))
        mg.set_option("dependent_launch", dep)
        mg.set_option("host_loop", host)
        custom = _mask(base, mg.shape(1), mkind)
        if custom is not None:
            mg.oper[1].msk = custom
            cfmg.setup_operators(mg)
            for lev in range(1, mg.nlevels + 1):
                for f in ("x", "y", "r", "b"):
                    cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk").astype(np.float64)
        b = np.asfortranarray(np.random.default_rng(21).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk)
        mg.data[1].b = b
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((res, n, hist, mg.data[1].x))
    for o in out[1:]:
        assert o[1] == out[0][1] and o[0] == out[0][0]
        assert np.array_equal(o[2], out[0][2])
        assert np.array_equal(o[3], out[0][3])



@pytest.mark.parametrize("name", ["3d_48_centers_v", "3d_32_vertices_v", "3d_40x36x26_centers_f",
                                  "3d_odd_33x30x20_centers_v"])
def test_coded_widiag_is_bit_identical(name):
    """The 3D 7-point FP32 sweeps reading omega*idiag as a one-byte code into
    a table (the default where every cell's code reproduces its float) give
    the streamed floats' history and solution bit for bit: in the four-cell
    form (even row length) and in the one-cell form (odd row length). So do
    the forms that come with the codes: the cell-centred residual formed at
    the coarse cells' children and restricted in one pass (fused_descent
    on), and, in the V-cycle, the first level-1 sweep taking x as +0
    without the zeroing pass."""
    base, mkind = CASES[name]
    out = []
    for coded, fuse in ((1, 1), (1, 0), (0, 1)):
        mg = cfmg.get_gmg(cfmg.Param(**base, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed",
                                     verbose=False))
        mg.set_option("engine_cells", 2000)  # fine levels as standalone kernels
        mg.set_option("coded_widiag", coded)
        mg.set_option("fused_descent", fuse)
        custom = _mask(base, mg.shape(1), mkind)
        if custom is not None:
            mg.oper[1].msk = custom
            cfmg.setup_operators(mg)
            for lev in range(1, mg.nlevels + 1):
                for f in ("x", "y", "r", "b"):
                    cfmg.set_to_zero(mg, lev, f)
        msk = mg.download(1, "msk").astype(np.float64)
        b = np.asfortranarray(np.random.default_rng(23).standard_normal(mg.shape(1))) * msk
        F.subtract_mean(b, msk)
        mg.data[1].b = b
        res, n, hist = cfmg.solve(mg, history=True)
        out.append((res, n, hist, mg.data[1].x))
    assert out[0][0] <= 1e-10
    for o in out[1:]:
        assert out[0][1] == o[1] and out[0][0] == o[0]
        assert np.array_equal(out[0][2], o[2]) and np.array_equal(out[0][3], o[3])
