"""Hand-written adjoint: dL/db and dL/dkappa of L = 1/2 |P x - x*|^2 over the
wet cells, A(kappa) x = b (2D cell-centred variable-coefficient operator,
face coefficient = mean of the two cells).

Checked two ways, as the configuration asks: against central finite
differences along random directions (relative error <= 1e-6, forward
solves to 1e-14), and against the gradient assembled from the CPU
oracle's own FP64 solves (the adjoint system A lam = P g solved by the
oracle's multigrid, the kappa-gradient formula applied in numpy).
"""
import numpy as np
import pytest

import fixtures as F
import oracle as O

pytestmark = pytest.mark.gpu
cfmg = pytest.importorskip("cfmg")

N = 96
BASE = dict(nx=N, ny=N, nz=1, case="twod", location="centers", operator="varcoef", cycle="v", npre=2, npost=2,
            omega=0.8, ndeepest=40)


def _problem(seed=4):
    from scipy.ndimage import gaussian_filter

    t = N + 6
    rng = np.random.default_rng(seed)
    kap = np.exp(0.5 * gaussian_filter(rng.standard_normal((t, t)), 4.0))[:, :, None]
    kap = np.asfortranarray(kap / kap.std() * 0.5 + 1.0)
    msk = F.get_circular_domain((t, t, 1), radius=0.45)
    b = np.asfortranarray(rng.standard_normal((t, t, 1))) * msk
    xstar = np.asfortranarray(rng.standard_normal((t, t, 1))) * msk
    return kap, msk, b, xstar


def _gmg(precision="fp64", tol=1e-14):
    mg = cfmg.get_gmg(cfmg.Param(**BASE, tol=tol, maxite=80, residual_norm="l2", precision=precision,
                                 verbose=False))
    return mg


def _setup(mg, kap, msk):
    mg.oper[1].msk = msk
    mg.oper[1].kappa = kap
    cfmg.setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            cfmg.set_to_zero(mg, lev, f)
    return mg.download(1, "msk").astype(np.float64)


def _loss(mg, kap, msk, b, xstar):
    m = _setup(mg, kap, msk)
    bb = b * m
    F.subtract_mean(bb, m)
    return cfmg.loss_and_grad(mg, bb, xstar * m)


def test_adjoint_matches_central_differences():
    kap, msk, b, xstar = _problem()
    mg = _gmg()
    L0, gb, gk = _loss(mg, kap, msk, b, xstar)
    m = mg.download(1, "msk").astype(np.float64)
    rng = np.random.default_rng(17)
    for k in range(8):
        db = rng.standard_normal(b.shape) * m
        db -= m * (db.sum() / m.sum())
        dk = rng.standard_normal(b.shape) * m * 0.1
        eps = 1e-4
        lp = _loss(mg, kap + eps * dk, msk, b + eps * db, xstar)[0]
        lm = _loss(mg, kap - eps * dk, msk, b - eps * db, xstar)[0]
        fd = (lp - lm) / (2 * eps)
        an = float(np.sum(gb * db) + np.sum(gk * dk))
        assert abs(fd - an) <= 1e-6 * abs(an), (k, fd, an)


def test_adjoint_matches_oracle_fp64_gradient():
    kap, msk, b, xstar = _problem(seed=5)
    mg = _gmg()
    L0, gb, gk = _loss(mg, kap, msk, b, xstar)
    x = mg.data[1].x
    m = mg.download(1, "msk").astype(np.float64)
    # oracle: the same forward x, then A lam = P g with the oracle's multigrid
    p = dict(BASE, tol=1e-30, maxite=60)
    og = O.OracleGmg(p)
    og.field(1, "msk")[...] = msk
    og.field(1, "kappa")[...] = kap
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    w = m.astype(bool)
    px = np.where(w, x, 0.0)
    px[w] -= px[w].mean()
    g = (px - xstar * m) * m
    g[w] -= g[w].mean()
    og.field(1, "b")[...] = g
    og.solve()
    lam = og.x.copy()
    lam[w] -= lam[w].mean()
    lam[~w] = 0
    np.testing.assert_allclose(gb, lam, rtol=0, atol=1e-9 * np.abs(lam).max())
    # kappa gradient from lam and x, face by face
    gko = np.zeros_like(x)
    for sh, ax in ((1, 0), (-1, 0), (1, 1), (-1, 1)):
        xn = np.roll(x, sh, axis=ax)
        ln = np.roll(lam, sh, axis=ax)
        mn = np.roll(m, sh, axis=ax)
        gko += np.where((m > 0) & (mn > 0), 0.5 * (lam - ln) * (x - xn), 0.0)
    np.testing.assert_allclose(gk, gko, rtol=0, atol=1e-9 * np.abs(gko).max())


def test_mixed_adjoint_agrees_with_fp64():
    kap, msk, b, xstar = _problem(seed=6)
    r64 = _loss(_gmg("fp64", 1e-13), kap, msk, b, xstar)
    r32 = _loss(_gmg("mixed", 1e-13), kap, msk, b, xstar)
    assert abs(r32[0] - r64[0]) <= 1e-9 * abs(r64[0])
    for a, c in ((r32[1], r64[1]), (r32[2], r64[2])):
        assert np.linalg.norm(a - c) <= 1e-7 * np.linalg.norm(c)
