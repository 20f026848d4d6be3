"""Error behaviour of the C ABI, as the reference's assertions map to
status codes (src/halo.jl:13, src/gmg_setup.jl:131-155, src/gmg_solver.jl:18
raise AssertionError; libcfmg returns CFMG_ERR_ARG and a message).

Beyond the reference: a call out of order (an operator or solve before the
coefficients exist, an adjoint before a forward solve) is CFMG_ERR_STATE,
and a NaN or Inf in b or in the residual norm ends a solve with
CFMG_ERR_NONFINITE (the reference's loop would stop silently with res =
NaN, or report an infinite |b| as converged). Exhausting maxite is not an
error: solve! returns (res, maxite), as the reference does
(src/gmg_solver.jl:29-41).

The tests without the gpu mark need no device: null handles and bad
descriptors fail before any CUDA call.
"""
import ctypes

import numpy as np
import pytest

import fixtures as F

cfmg = pytest.importorskip("cfmg")
from cfmg import _lib  # noqa: E402

gpu = pytest.mark.gpu


def _codes():
    return _lib.ERR_ARG, _lib.ERR_STATE, _lib.ERR_NONFINITE


# ---------------------------------------------------------------- no GPU
def test_null_handle_is_an_argument_error():
    L = _lib.load()
    res, nite, out = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
    assert L.cfmg_solve(None, ctypes.byref(res), ctypes.byref(nite), None) == _lib.ERR_ARG
    assert L.cfmg_smooth(None, 1, 1) == _lib.ERR_ARG
    assert L.cfmg_residual(None, 1) == _lib.ERR_ARG
    assert L.cfmg_restrict(None, 1, 0) == _lib.ERR_ARG
    assert L.cfmg_prolong(None, 1) == _lib.ERR_ARG
    assert L.cfmg_norm(None, 1, 0, ctypes.byref(out)) == _lib.ERR_ARG
    assert L.cfmg_cycle(None, 0) == _lib.ERR_ARG
    assert L.cfmg_destroy(None) == 0


@pytest.mark.parametrize("bad", [dict(topology="yperio"), dict(cycle="w"), dict(location="edges"),
                                 dict(precision="fp16"), dict(residual_norm="max")])
def test_unknown_symbols_are_argument_errors(bad):
    """The reference asserts on an unknown topology (src/halo.jl:13) or cycle
    (src/gmg_solver.jl:18); the host mirror rejects the symbol before the
    library sees it."""
    with pytest.raises(cfmg.CfmgError) as e:
        cfmg.Param(**bad).desc()
    assert e.value.code == _lib.ERR_ARG


def test_descriptor_codes_out_of_range_are_argument_errors():
    """Codes that pass no Python mapping (a C caller's descriptor) are
    rejected by cfmg_create with a message and no handle."""
    L = _lib.load()
    for field, value in (("topology", 7), ("cycle", 9), ("op", 5), ("precision", 3), ("norm_kind", 4),
                         ("maxite", -1), ("nlevels", -2)):
        d = cfmg.Param().desc()
        setattr(d, field, value)
        h = ctypes.c_void_p()
        assert L.cfmg_create(ctypes.byref(d), ctypes.byref(h)) == _lib.ERR_ARG, field
        assert not h.value and L.cfmg_last_error(None), field


# -------------------------------------------------------------- with GPU
def _small(**kw):
    p = dict(nx=64, ny=64, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8, tol=1e-20, maxite=30,
             verbose=False)
    p.update(kw)
    return cfmg.Param(**p)


def _rhs(mg, seed=0):
    m = mg.download(1, "msk").astype(np.float64)
    b = np.asfortranarray(np.random.default_rng(seed).standard_normal(mg.shape(1))) * m
    F.subtract_mean(b, m)
    return b


@gpu
def test_bad_level_and_field_ids():
    mg = cfmg.get_gmg(_small())
    L, h = mg._L, mg.handle
    n = mg.nlevels
    for lev in (0, n + 1, -3):
        assert L.cfmg_smooth(h, lev, 1) == _lib.ERR_ARG
        assert L.cfmg_residual(h, lev) == _lib.ERR_ARG
        assert b"out of range" in L.cfmg_last_error(h)
    # restriction and prolongation act on lev and lev+1: the coarsest is out
    assert L.cfmg_restrict(h, n, 0) == _lib.ERR_ARG
    assert L.cfmg_prolong(h, n) == _lib.ERR_ARG
    out = ctypes.c_double()
    buf = np.zeros(mg.shape(1), order="F")
    for field in (99, -1):
        assert L.cfmg_norm(h, 1, field, ctypes.byref(out)) == _lib.ERR_ARG
        assert L.cfmg_upload(h, 1, field, buf.ctypes.data_as(ctypes.c_void_p)) == _lib.ERR_ARG
        assert L.cfmg_download(h, 1, field, buf.ctypes.data_as(ctypes.c_void_p)) == _lib.ERR_ARG
        assert L.cfmg_zero(h, 1, field) == _lib.ERR_ARG
        assert L.cfmg_fill(h, 1, field) == _lib.ERR_ARG
    assert L.cfmg_restrict(h, 1, 4) == _lib.ERR_ARG  # diag is not a restrictable field
    assert L.cfmg_norm(h, 1, 9, ctypes.byref(out)) == _lib.ERR_ARG  # the uint8 mask has no FP64 norm
    assert L.cfmg_smooth(h, 1, -1) == _lib.ERR_ARG
    # the handle still works after the rejected calls
    mg.data[1].b = _rhs(mg)
    res, nite = cfmg.solve(mg)
    assert res <= 1e-20 and nite > 0


@gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_calls_out_of_order(precision):
    """An operator or a solve before the coefficients exist, and an adjoint
    before a forward solve, are CFMG_ERR_STATE; after setup the same calls
    succeed."""
    mg = cfmg.Gmg(_small(precision=precision))  # the handle only: no set_default_msk, no setup
    L, h = mg._L, mg.handle
    res, nite = ctypes.c_double(), ctypes.c_int()
    assert L.cfmg_solve(h, ctypes.byref(res), ctypes.byref(nite), None) == _lib.ERR_STATE
    assert b"not set up" in L.cfmg_last_error(h)
    assert L.cfmg_smooth(h, 1, 1) == _lib.ERR_STATE
    assert L.cfmg_cycle(h, 0) == _lib.ERR_STATE
    cfmg.set_default_msk(mg)
    cfmg.setup_operators(mg)
    g = np.zeros(mg.shape(1), order="F")
    gb = np.zeros_like(g)
    assert L.cfmg_adjoint(h, g.ctypes.data_as(ctypes.c_void_p), gb.ctypes.data_as(ctypes.c_void_p), None,
                          ctypes.byref(res), ctypes.byref(nite)) == _lib.ERR_STATE
    assert b"forward" in L.cfmg_last_error(h)
    mg.data[1].b = _rhs(mg)
    r, n = cfmg.solve(mg)
    assert r <= 1e-20 and n > 0
    gb2, _ = cfmg.adjoint(mg, _rhs(mg, 1))
    assert np.isfinite(gb2).all()


@gpu
def test_bound_coefficients_count_as_setup():
    """cfmg_bind_level with coefficients from the caller's own setup (the
    Julia host's path) is a setup; a wrong array size is rejected."""
    ref = cfmg.get_gmg(_small())
    mg = cfmg.Gmg(_small())
    for lev in range(1, ref.nlevels + 1):
        o = ref.oper[lev]
        mg.bind_level(lev, o.diag, o.idiag, o.Rcoef, o.Pcoef, o.msk)
    b = _rhs(ref)
    ref.data[1].b = b
    mg.data[1].b = b
    assert cfmg.solve(mg) == cfmg.solve(ref)
    with pytest.raises(cfmg.CfmgError) as e:
        mg.bind_level(1, diag=np.zeros(10))
    assert e.value.code == _lib.ERR_ARG
    with pytest.raises(cfmg.CfmgError) as e:
        mg.upload(1, "b", np.zeros((5, 5, 1)))
    assert e.value.code == _lib.ERR_ARG


@gpu
@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("host_loop", [0, 1])
def test_nonfinite_b_ends_the_solve(bad, precision, host_loop):
    mg = cfmg.get_gmg(_small(precision=precision, residual_norm="l2", tol=1e-10))
    mg.set_option("host_loop", host_loop)
    b = _rhs(mg)
    b[30, 30, 0] = bad
    mg.data[1].b = b
    L, h = mg._L, mg.handle
    res, nite = ctypes.c_double(), ctypes.c_int()
    hist = (ctypes.c_double * 31)()
    rc = L.cfmg_solve(h, ctypes.byref(res), ctypes.byref(nite), hist)
    assert rc == _lib.ERR_NONFINITE, (rc, res.value, nite.value)
    assert nite.value == 0 and b"non-finite" in L.cfmg_last_error(h)
    # a clean b afterwards solves normally on the same handle
    mg.data[1].b = _rhs(mg)
    cfmg.set_to_zero(mg, 1, "x")
    r, n = cfmg.solve(mg)
    assert r <= 1e-10 and n > 0


@gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_maxite_exhaustion_returns_res_and_maxite(precision):
    """solve! stops at maxite with the residual of that iteration and no
    error (src/gmg_solver.jl:29-41); the FP64 form's history is the
    oracle's."""
    import oracle as O

    p = _small(precision=precision, maxite=3, tol=1e-30)
    mg = cfmg.get_gmg(p)
    b = _rhs(mg)
    mg.data[1].b = b
    res, nite, hist = cfmg.solve(mg, history=True)
    assert nite == 3 and res > 1e-30 and len(hist) == 4 and hist[-1] == res
    og = O.OracleGmg(dict(nx=64, ny=64, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8, tol=1e-30,
                          maxite=3))
    og.field(1, "b")[...] = b
    r0, n0, h0 = og.solve()
    assert n0 == 3
    np.testing.assert_allclose(hist, h0, rtol=1e-12 if precision == "fp64" else 1e-4)


@gpu
def test_batch_errors():
    """A batch with an instance that was never set up is CFMG_ERR_STATE; an
    instance whose b holds a NaN stops with CFMG_ERR_NONFINITE while the
    others converge."""
    p = _small(precision="mixed", residual_norm="l2", tol=1e-10, maxite=40)
    sizes = [64, 96, 128]
    batch = cfmg.Batch(p, sizes, sizes)
    L = batch._L
    res = np.zeros(3)
    nite = np.zeros(3, dtype=np.int32)
    rc = L.cfmg_batch_solve(batch._b, 1, res.ctypes.data_as(ctypes.c_void_p), nite.ctypes.data_as(ctypes.c_void_p),
                            None)
    assert rc == _lib.ERR_STATE and b"not set up" in L.cfmg_batch_last_error(batch._b)
    for i, n in enumerate(sizes):
        g = batch.instance(i)
        cfmg.set_default_msk(g)
        cfmg.setup_operators(g)
        for lev in range(1, g.nlevels + 1):
            for f in ("x", "y", "r", "b"):
                cfmg.set_to_zero(g, lev, f)
        b = _rhs(g, i)
        if i == 1:
            b[20, 20, 0] = np.nan
        g.data[1].b = b
    rc = L.cfmg_batch_solve(batch._b, 1, res.ctypes.data_as(ctypes.c_void_p), nite.ctypes.data_as(ctypes.c_void_p),
                            None)
    assert rc == _lib.ERR_NONFINITE and b"instance 1" in L.cfmg_batch_last_error(batch._b)
    assert res[0] <= 1e-10 and res[2] <= 1e-10 and not np.isfinite(res[1]) and nite[1] == 0


@gpu
def test_solve_tol_sets_the_rule_per_call():
    """cfmg_solve_tol(h, tol, maxite, norm_kind, ...): the stopping rule per
    call (the graphs are rebuilt when it changes, the history buffer grows
    with maxite); each solve matches the oracle's solve! with that rule."""
    import oracle as O

    mg = cfmg.get_gmg(_small(tol=1e-20, maxite=30))
    b = _rhs(mg)
    mg.data[1].b = b
    base = dict(nx=64, ny=64, nz=1, case="twod", cycle="v", npre=2, npost=2, omega=0.8)
    for tol, maxite, kind in ((1e-20, 30, "ref_squared"), (1e-8, 30, "ref_squared"), (1e-24, 60, "ref_squared"),
                              (1e-6, 4, "ref_squared"), (1e-10, 30, "l2")):
        cfmg.set_to_zero(mg, 1, "x")
        res, nite, hist = cfmg.solve(mg, history=True, tol=tol, maxite=maxite, residual_norm=kind)
        og = O.OracleGmg(dict(base, tol=tol * tol if kind == "l2" else tol, maxite=maxite))
        og.field(1, "b")[...] = b
        r0, n0, h0 = og.solve()
        assert nite == n0 and len(hist) == n0 + 1, (tol, maxite, kind, nite, n0)
        np.testing.assert_allclose(hist ** 2 if kind == "l2" else hist, h0, rtol=1e-11)
        assert np.array_equal(mg.data[1].x, og.x)


@gpu
def test_adjoint_solve_matches_adjoint():
    mg = cfmg.get_gmg(_small(tol=1e-20, maxite=30))
    mg.data[1].b = _rhs(mg)
    cfmg.solve(mg)
    g = np.asfortranarray(_rhs(mg, 3))
    gb, _ = cfmg.adjoint(mg, g)
    gb2 = np.empty_like(gb)
    L = mg._L
    assert L.cfmg_adjoint_solve(mg.handle, g.ctypes.data_as(ctypes.c_void_p), gb2.ctypes.data_as(ctypes.c_void_p),
                                None) == 0
    assert np.array_equal(gb, gb2)
