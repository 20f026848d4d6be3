"""The CPU oracle against every known answer of the reference test suite.

Each case replays one Julia test (file:line in tests/fixtures.py) on the
oracle and checks (res, ite) with the reference's own tolerance. This pins
the oracle before any GPU result is compared with it.
"""
import pytest

import fixtures as F
import oracle as O


GOLDEN = F.load_golden()


def _solve(sc):
    og = O.OracleGmg(sc.param)
    F.prepare(F.OracleAdapter(og), sc)
    return og, og.solve()


def _check_golden(sc, og, res, nite, hist):
    """The committed solve of the scenario (tests/golden), bit for bit."""
    g = GOLDEN.get(sc.name)
    if g is None:
        return
    assert nite == g["nite"] and res == g["res"]
    assert [float(h) for h in hist] == g["hist"]
    assert F.field_digest(og.x) == g["x_sha256"]
    assert F.field_digest(og.field(1, "r")) == g["r_sha256"]


@pytest.mark.parametrize("sc", F.KNOWN_ANSWERS + F.RECTANGULAR, ids=lambda s: s.name)
def test_known_answer(sc):
    og, (res, nite, hist) = _solve(sc)
    assert nite == sc.expect_ite
    assert abs(res - sc.expect_res) <= sc.atol, (res, sc.expect_res)
    assert hist[-1] == res and len(hist) == nite + 1
    _check_golden(sc, og, res, nite, hist)


@pytest.mark.parametrize("sc", F.ITERATION_ONLY, ids=lambda s: s.name)
def test_iteration_count(sc):
    og, (res, nite, hist) = _solve(sc)
    assert nite == sc.expect_ite
    _check_golden(sc, og, res, nite, hist)


def test_golden_file_covers_the_scenarios():
    """The committed solves are those of the current scenarios, with the
    same parameters (regenerate with tests/golden/make_golden.py)."""
    scs = {sc.name: sc for sc in F.golden_scenarios()}
    assert set(GOLDEN) == set(scs)
    for name, sc in scs.items():
        assert GOLDEN[name]["param"] == sc.param, name


def test_level_hierarchy_matches_create_levels():
    # src/gmg_setup.jl:40-64: 64^3 -> 6 levels down to 2^3; 512^2 2D -> 9 levels
    og = O.OracleGmg(dict(nx=64, ny=64, nz=64, case="threed"), setup=False)
    assert og.nlevels == 6 and og.dims(6)[:3] == (2, 2, 2)
    og = O.OracleGmg(dict(nx=512, ny=512, nz=1, case="twod"), setup=False)
    assert og.nlevels == 9 and og.dims(9)[:3] == (2, 2, 1)
    og = O.OracleGmg(dict(nx=256, ny=256, nz=1, case="twod", nlevels=6), setup=False)
    assert og.nlevels == 6 and og.dims(6)[:3] == (8, 8, 1)


def test_default_mask_and_setup_coefficients():
    # 2D centres, 8x8: interior diag = 4 (5-point), corner cells see 2 wet
    # neighbours (Neumann); Rcoef = msk on the coarse level, Pcoef = 1/16.
    og = O.OracleGmg(dict(nx=8, ny=8, nz=1, case="twod"))
    d = og.field(1, "diag")[:, :, 0]
    assert d[5, 5] == 4.0 and d[3, 3] == 2.0 and d[3, 5] == 3.0 and d[0, 0] == 0.0
    assert (og.field(2, "Rcoef") == og.field(2, "msk")).all()
    assert og.field(1, "Pcoef")[5, 5, 0] == 1.0 / 16


def test_field_digest_sees_one_ulp_and_ignores_zero_sign():
    """The digests of the committed solves change with any one-ulp change of
    one cell, not with the sign of a zero, and not with the memory order of
    the array."""
    import numpy as np

    rng = np.random.default_rng(0)
    x = np.asfortranarray(rng.standard_normal((7, 5, 3)))
    x[2, 3, 1] = 0.0
    d = F.field_digest(x)
    y = x.copy(order="F")
    y[4, 1, 2] = np.nextafter(y[4, 1, 2], np.inf)
    assert F.field_digest(y) != d
    z = x.copy(order="F")
    z[2, 3, 1] = -0.0
    assert F.field_digest(z) == d
    assert F.field_digest(np.ascontiguousarray(x)) == d
