"""cfmg_norm_noalloc: the masked norm for callers that cannot allocate.

Some users of this library hold their fields in device memory that another
allocator owns (a Julia CuArray pool, a PyTorch caching allocator) or run
under a fixed device-memory budget, and cannot let the library call
cudaMalloc where they need a reduction. cfmg_norm_noalloc keeps its partial
sums in a static device array instead. This test calls it through the C ABI
on a handle's own device field, twice in a row (the scratch array is shared
by both calls), and compares each result with the handle-based cfmg_norm,
which uses scratch the handle allocated. It needs only a GPU, so it passes
alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
cfmg = pytest.importorskip("cfmg")
torch = pytest.importorskip("torch")

RTOL = 1e-13  # two tree sums of the same values in different orders


def test_norm_noalloc_matches_handle_norm_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    stream = torch.cuda.Stream()
    # 1006 x 706 = 710,236 elements: 11 chunks of the static scratch
    mg = cfmg.get_gmg(cfmg.Param(nx=1000, ny=700, nz=1, case="twod", verbose=False))
    mg.set_stream(stream.cuda_stream)
    L = mg._L
    shape = mg.shape(1)
    n = shape[0] * shape[1] * shape[2]
    rng = np.random.default_rng(11)
    msk = rng.integers(0, 3, size=shape).astype(np.uint8)  # 0, 1 and 2 weights
    mg.oper[1].msk = msk
    xp, mp, out = mg.field_ptr(1, "x"), mg.field_ptr(1, "msk"), mg.field_ptr(2, "y")
    for call in range(2):
        x = np.asfortranarray(rng.standard_normal(shape) * (10.0 ** call))
        mg.data[1].x = x
        expected = cfmg.norm(mg, 1, "x")
        rc = L.cfmg_norm_noalloc(ctypes.c_void_p(xp), ctypes.c_void_p(mp), ctypes.c_longlong(n),
                                 ctypes.c_void_p(out), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.cfmg_last_error(None)
        got = mg.download(2, "y").ravel(order="F")[0]
        assert abs(got - expected) <= RTOL * abs(expected), (call, got, expected)
        exact = float(np.sum(msk.astype(np.float64) * x * x))
        assert abs(got - exact) <= 1e-12 * exact


def test_norm_noalloc_rejects_oversize():
    L = cfmg._lib.load()
    rc = L.cfmg_norm_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_longlong(268435456 + 1),
                             ctypes.c_void_p(16), None)
    assert rc == cfmg._lib.ERR_ARG
    assert b"exceeds the static scratch limit" in L.cfmg_last_error(None)


def test_norm_noalloc_rejects_negative_n():
    L = cfmg._lib.load()
    rc = L.cfmg_norm_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_longlong(-1), ctypes.c_void_p(16), None)
    assert rc == cfmg._lib.ERR_ARG
    assert b"negative n" in L.cfmg_last_error(None)
