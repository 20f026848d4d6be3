"""The 3D cell-centred 7-point configuration (coastline extruded in z, cut by
a bottom topography; V-cycle, Jacobi 2/2) at a reduced size, 64 x 64 x 32
with 5 levels: the FP64 drop-in against the CPU oracle (same solution bit
for bit, residual history to summation order), and the mixed form against
the oracle's FP64 solution."""
import numpy as np
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu
cfmg = pytest.importorskip("cfmg")

TOL = 1e-9


def _problem():
    param, msk, noise = W.config3(64, 64, 32, nlevels=5)
    return param, msk, noise


def _oracle(param, msk, noise):
    og = O.OracleGmg(dict(param, tol=TOL * TOL, maxite=60, verbose=False), setup=False)
    og.field(1, "msk")[...] = msk
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):  # the setup leaves x = msk; both sides start from 0
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    b = W.rhs(noise, og.field(1, "msk"))
    og.field(1, "b")[...] = b
    return og, b


def _gpu(param, msk, b, precision):
    mg = cfmg.get_gmg(cfmg.Param(**param, tol=TOL if precision == "mixed" else TOL * TOL, maxite=60,
                                 residual_norm="l2" if precision == "mixed" else "ref_squared",
                                 precision=precision, verbose=False))
    mg.oper[1].msk = msk
    cfmg.setup_operators(mg)
    for lev in range(1, mg.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            cfmg.set_to_zero(mg, lev, f)
    mg.data[1].b = b
    return mg


def _pair():
    param, msk, noise = _problem()
    og, b = _oracle(param, msk, noise)
    mg = _gpu(param, msk, b, "fp64")
    return og, mg


def test_config3_setup_bitwise():
    og, mg = _pair()
    assert og.nlevels == mg.nlevels
    for lev in range(1, og.nlevels + 1):
        for f in ("msk", "diag", "idiag", "Rcoef", "Pcoef"):
            a, c = og.field(lev, f), mg.download(lev, f)
            bad = np.argwhere(a != c)
            assert bad.size == 0, (lev, f, len(bad), bad[:4].tolist(), a[tuple(bad[0])], c[tuple(bad[0])])


@pytest.mark.parametrize("engine", ["engine", "standalone"])
def test_config3_operators_bitwise(engine):
    og, mg = _pair()
    mg.set_option("engine_cells", 10**9 if engine == "engine" else 0)
    rng = np.random.default_rng(3)
    L = og.nlevels
    for lev in range(1, L + 1):
        for f in ("x", "b", "y", "r"):
            a = np.asfortranarray(rng.standard_normal(og.shape(lev)))
            og.field(lev, f)[...] = a
            mg.upload(lev, f, a)

    def check(what):
        for lev in range(1, L + 1):
            for f in ("x", "y", "r", "b"):
                a, c = og.field(lev, f), mg.download(lev, f)
                bad = np.argwhere(a != c)
                assert bad.size == 0, (what, lev, f, len(bad), bad[:4].tolist())

    for lev in range(1, L + 1):
        og.smooth(lev, 2)
        mg.smoother[lev](mg, lev, 2)
        check(f"smooth{lev}")
        og.residual(lev)
        mg.residual[lev](mg, lev)
        check(f"residual{lev}")
    for lev in range(1, L):
        og.restrict(lev, "r")
        mg.restriction[lev](mg, lev, "r")
        check(f"restrict{lev}")
        og.prolong(lev)
        mg.prolongation[lev](mg, lev)
        check(f"prolong{lev}")


def test_config3_fp64_matches_oracle():
    param, msk, noise = _problem()
    og, b = _oracle(param, msk, noise)
    res0, n0, h0 = og.solve()
    mg = _gpu(param, msk, b, "fp64")
    assert np.array_equal(mg.download(1, "msk"), og.field(1, "msk"))
    res1, n1, h1 = cfmg.solve(mg, history=True)
    assert n1 == n0 and 10 <= n0 < 60, (n0, n1)
    np.testing.assert_allclose(h1, h0, rtol=1e-11, atol=0)
    assert np.array_equal(mg.data[1].x, og.x)


def test_config3_mixed_matches_fp64_oracle():
    param, msk, noise = _problem()
    og, b = _oracle(param, msk, noise)
    og.solve()
    m = og.field(1, "msk").astype(bool)
    xo = og.x.copy()
    mg = _gpu(param, msk, b, "mixed")
    res, n, hist = cfmg.solve(mg, history=True)
    assert res <= TOL, (res, hist)
    x = mg.data[1].x
    # true FP64 residual of the mixed solution, on the oracle
    og.field(1, "x")[...] = x
    true_res = og.normresidual(og.norm(1, "b")) ** 0.5
    assert true_res <= TOL * 1.0001, true_res
    a = x[m] - x[m].mean()
    c = xo[m] - xo[m].mean()
    assert np.linalg.norm(a - c) / np.linalg.norm(c) <= 1e-5
