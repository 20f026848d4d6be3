"""Batched engine: many masked solves of uneven sizes in one launch.

Each instance of a small batch (config-4 style: 2D cell-centred 5-point,
disk or noise masks, N(0,1) right-hand sides) must reach the tolerance with
its true FP64 residual, take the same number of cycles as a single-handle
mixed solve of the same problem, and agree with that solution.
"""
import numpy as np
import pytest

import fixtures as F
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu
cfmg = pytest.importorskip("cfmg")


def _param(**kw):
    d = dict(nx=64, ny=64, nz=1, case="twod", location="centers", operator="laplacian", cycle="v", npre=2, npost=2,
             omega=0.8, ndeepest=20, tol=1e-10, maxite=40, residual_norm="l2", precision="mixed", verbose=False)
    d.update(kw)
    return cfmg.Param(**d)


def _setup(g, msk, noise):
    g.oper[1].msk = msk
    cfmg.setup_operators(g)
    for lev in range(1, g.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            cfmg.set_to_zero(g, lev, f)
    m = g.download(1, "msk").astype(np.float64)
    b = np.asfortranarray(noise * m)
    F.subtract_mean(b, m)
    g.data[1].b = b
    return m


@pytest.mark.parametrize("int_res", [1, 0])
@pytest.mark.parametrize("cycle", ["v", "f"])
def test_batch_matches_single_solves(cycle, int_res):
    """int_res: the level-1 residual in 64-bit fixed point (1) or FP64
    arithmetic (0), in the batch and in the single solves alike."""
    probs = W.config4(ninst=10, seed=3, lo=64, hi=288)
    p = _param(cycle=cycle, maxite=100)
    batch = cfmg.Batch(p, [q[0] for q in probs], [q[0] for q in probs], [q[1] for q in probs])
    masks = []
    for i, (n, nlev, msk, noise) in enumerate(probs):
        batch.instance(i).set_option("int_residual", int_res)
        masks.append(_setup(batch.instance(i), msk, noise))
    res, nite, t = batch.solve()
    assert np.all(t > 0)
    for i, (n, nlev, msk, noise) in enumerate(probs):
        g = batch.instance(i)
        x = g.data[1].x
        # the reported residual is the batched solution's own: recomputed in
        # FP64 arithmetic it agrees to the rounding noise of that arithmetic
        # near 1e-10 (|A||x| 2^-53 per cell against r; the fixed-point form
        # is exact for x on its 2^-k grid), 1e-4 relative here
        nb = cfmg.norm(g, 1, "b")
        true = cfmg.normresidual(g, nb) ** 0.5
        assert abs(true - res[i]) <= (1e-4 if int_res else 1e-6) * res[i], (i, true, res[i])
        # single-handle mixed solve of the same problem: same outcome
        s = cfmg.get_gmg(dataclasses_replace(p, nx=n, ny=n, nlevels=nlev))
        s.set_option("int_residual", int_res)
        _setup(s, msk, noise)
        r1, n1 = cfmg.solve(s)
        assert (res[i] <= 1e-10) == (r1 <= 1e-10), (i, res[i], r1)
        assert abs(int(nite[i]) - n1) <= 1, (i, nite[i], n1)
        if r1 <= 1e-10:
            w = masks[i].astype(bool)
            a, c = x[w] - x[w].mean(), s.data[1].x[w] - s.data[1].x[w].mean()
            assert np.linalg.norm(a - c) <= 1e-6 * np.linalg.norm(c)
    assert np.sum(res <= 1e-10) >= 5  # the disks and the smooth coastlines
    # a second solve from zero (graph replay) gives the same answer
    res2, nite2, _ = batch.solve()
    assert np.array_equal(res, res2) and np.array_equal(nite, nite2)


def dataclasses_replace(p, **kw):
    import dataclasses

    return dataclasses.replace(p, **kw)


def test_batch_vertex_9point_matches_single_solves():
    """Vertex-centred 9-point instances (the coastline-style operator of the
    F-cycle configuration): the batched solve agrees with single solves,
    and a second batched solve continuing from the converged x stops at
    once."""
    sizes = [96, 160, 256, 64, 200]
    p = _param(location="vertices", operator="laplacian9", cycle="f", npre=3, npost=3, maxite=60)
    nlev = [int(np.floor(np.log2(n / 8))) + 1 for n in sizes]
    batch = cfmg.Batch(p, sizes, sizes, nlev)
    rng = np.random.default_rng(11)
    probs = []
    for i, n in enumerate(sizes):
        t = n + 6
        cells = F.get_circular_domain((t, t, 1), nh=3, radius=0.45)
        msk = F.get_mask_at_corners(cells)
        noise = np.asfortranarray(rng.standard_normal((t, t, 1)))
        probs.append((msk, noise))
        _setup(batch.instance(i), msk, noise)
    res, nite, _ = batch.solve()
    assert np.all(res <= 1e-10), res
    for i, n in enumerate(sizes):
        g = batch.instance(i)
        s = cfmg.get_gmg(dataclasses_replace(p, nx=n, ny=n, nlevels=nlev[i]))
        _setup(s, *probs[i])
        r1, n1 = cfmg.solve(s)
        assert r1 <= 1e-10 and abs(int(nite[i]) - n1) <= 1, (i, nite[i], n1)
        w = probs[i][0].astype(bool)
        a, c = g.data[1].x[w], s.data[1].x[w]
        assert np.linalg.norm(a - c) <= 1e-6 * np.linalg.norm(c), i
    res2, nite2, _ = batch.solve(from_zero=False)
    assert np.all(nite2 == 0) and np.all(res2 <= 1e-10), (nite2, res2)


def _oracle_solve(p, n, nlev, msk, noise, maxite):
    """The oracle's FP64 solve of one batch instance (same mask, coarse
    hierarchy and right-hand side), to the same 1e-10 in ||r||/||b||, i.e.
    1e-20 in the reference's squared ratio (src/gmg_solver.jl:29-39)."""
    og = O.OracleGmg(dict(nx=n, ny=n, nz=1, case="twod", location=p.location, operator=p.operator, cycle=p.cycle,
                          npre=p.npre, npost=p.npost, omega=p.omega, ndeepest=p.ndeepest, nlevels=nlev,
                          tol=p.tol * p.tol, maxite=maxite))
    og.field(1, "msk")[...] = msk
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    m = og.field(1, "msk").astype(np.float64)
    b = np.asfortranarray(noise * m)
    F.subtract_mean(b, m)
    og.field(1, "b")[...] = b
    res, nite, _ = og.solve()
    return og, res ** 0.5, nite


@pytest.mark.parametrize("cycle", ["v", "f"])
def test_batch_against_oracle(cycle):
    """A config-4-style batch (16 instances, sizes log-uniform in 64..320
    rounded to 32, disk and smoothed-noise coastline masks, N(0,1) right-hand
    sides, mixed precision, 1e-10) against the oracle's FP64 solve of each
    instance: the batched x has a true residual (recomputed by the oracle
    in FP64) at the tolerance, the iteration count is the oracle's within
    one, and the solution is the oracle's to 1e-6 after wet-mean removal."""
    probs = W.config4(ninst=16, seed=5, lo=64, hi=320)
    kinds = {"disk" if q[2][q[0] // 2 + 3, 3, 0] == 0 and q[2][q[0] // 2 + 3, q[0] // 2 + 3, 0] else "noise"
             for q in probs}
    maxite = 150
    p = _param(cycle=cycle, maxite=maxite)
    batch = cfmg.Batch(p, [q[0] for q in probs], [q[0] for q in probs], [q[1] for q in probs])
    for i, (n, nlev, msk, noise) in enumerate(probs):
        _setup(batch.instance(i), msk, noise)
    res, nite, _ = batch.solve()
    converged = 0
    for i, (n, nlev, msk, noise) in enumerate(probs):
        og, ores, onite = _oracle_solve(p, n, nlev, msk, noise, maxite)
        g = batch.instance(i)
        assert np.array_equal(og.field(1, "msk"), g.download(1, "msk")), i
        if ores > 1e-10:  # the oracle does not converge within maxite: neither may the batch
            assert res[i] > 1e-10 and nite[i] == maxite, (i, res[i], nite[i])
            continue
        converged += 1
        assert abs(int(nite[i]) - onite) <= 1, (i, nite[i], onite)
        x = g.data[1].x
        ox = og.x.copy(order="F")
        # the batched solution's true residual, in the oracle's FP64 arithmetic
        og.field(1, "x")[...] = x
        true = og.normresidual(og.norm(1, "b")) ** 0.5
        assert true <= 1e-10 * (1 + 1e-3), (i, true, res[i])
        w = og.field(1, "msk").astype(bool)
        a, c = x[w] - x[w].mean(), ox[w] - ox[w].mean()
        assert np.linalg.norm(a - c) <= 1e-6 * np.linalg.norm(c), (i, np.linalg.norm(a - c) / np.linalg.norm(c))
    assert converged >= 12, converged
    assert len(kinds) == 2


@pytest.mark.parametrize("cycle,location,hi,int_res", [("f", "centers", 512, 1), ("v", "centers", 512, 1),
                                                        ("f", "centers", 128, 1), ("f", "vertices", 320, 1),
                                                        ("f", "centers", 320, 0)])
def test_batch_launch_forms_are_bit_identical(cycle, location, hi, int_res):
    """Four launch forms of the same batched iteration give the same bits:
    the default (coarse levels' steps as one block per instance and run of
    steps, CFMG_BOPT_COARSE_RUNS = 1; fine levels' blocked smoothing in the
    lean packed tiles, k_btb5; work tables interleaved across instances,
    CFMG_BOPT_INTERLEAVE = 1), one launch per coarse step for all instances
    (coarse_runs 0), the scalar blocked tiles (k_btb, the instances'
    temporal_blocking 3), and each instance's chunks listed together
    (interleave 0: the level-1 residual's partial sums keep their slots).
    Each executes the same per-item arithmetic and sums, so the residuals,
    cycle counts and solutions agree exactly. hi = 128: every level of every
    instance is coarse (the whole cycle runs in runs). int_res 0: the FP64
    form of the level-1 residual, whose per-chunk partial sums the
    interleaved table writes to their instance-ordered slots."""
    probs = W.config4(ninst=12, seed=7, lo=64, hi=hi)
    op = "laplacian9" if location == "vertices" else "laplacian"
    p = _param(cycle=cycle, location=location, operator=op, maxite=60)
    out = []
    for runs, tb, inter in ((1, 5, 1), (0, 5, 1), (1, 3, 1), (1, 5, 0)):
        batch = cfmg.Batch(p, [q[0] for q in probs], [q[0] for q in probs], [q[1] for q in probs])
        batch.set_option("coarse_runs", runs)
        batch.set_option("interleave", inter)
        for i, (n, nlev, msk, noise) in enumerate(probs):
            if location == "vertices":
                msk = F.get_mask_at_corners(msk)
            batch.instance(i).set_option("temporal_blocking", tb)
            batch.instance(i).set_option("int_residual", int_res)
            _setup(batch.instance(i), msk, noise)
        res, nite, _ = batch.solve()
        xs = [batch.instance(i).data[1].x.copy() for i in range(len(probs))]
        out.append((res, nite, xs))
        batch.close()
    r1, n1, x1 = out[0]
    for k, (r0, n0, x0) in enumerate(out[1:]):
        assert np.array_equal(n1, n0) and np.array_equal(r1, r0), (k, n1, n0, r1, r0)
        for i in range(len(probs)):
            assert np.array_equal(x1[i], x0[i]), (k, i)
    assert np.all(n1 >= 1) and np.sum(r1 <= 1e-10) >= 3, (n1, r1)
