"""Accuracy of the fixed-point level-1 residual (the mixed loop's integer
form) against FP64 arithmetic, both measured against the exact residual of
the same FP64 x (rational arithmetic).

A config-4 coastline instance is solved by the CPU oracle to ~1e-10. Near
convergence r is small against |A||x|. FP64 evaluation of b - A x rounds
at 2^-53 |x| per operation, while the fixed-point evaluation represents x
on a 2^-k grid (k = 58 - E, max(|x|, |b|) < 2^E) and is otherwise exact.
The fixed-point sum of r^2 must therefore be the closer one. This is the
property the GPU's k_resid_int* kernels rely on; this test restates their
arithmetic in Python integers.
"""
import math
from fractions import Fraction

import numpy as np

import oracle as O
import workloads as W


def test_fixed_point_residual_is_closer_to_exact_than_fp64():
    n, nlev, msk, noise = W.config4(12)[9]  # a 512^2 noise-coastline instance
    p = dict(nx=n, ny=n, nz=1, nh=3, case="twod", location="centers", operator="laplacian", cycle="v",
             nlevels=nlev, npre=2, npost=2, omega=0.8, ndeepest=20, tol=1e-20, maxite=40)
    og = O.OracleGmg(p, setup=False)
    og.msk[...] = msk
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0
    b = W.rhs(noise, og.msk)
    og.b[...] = b
    nb = og.norm(1, "b")
    for _ in range(40):
        og.cycle("v")
        if math.sqrt(og.normresidual(nb)) < 1e-10:
            break
    x = og.x.ravel(order="F")
    d = og.field(1, "diag").ravel(order="F")
    m = og.msk.ravel(order="F")
    r64 = og.field(1, "r").ravel(order="F")
    bf = b.ravel(order="F")
    n1 = og.shape(1)[0]
    k = 58 - math.frexp(max(np.abs(x).max(), np.abs(bf).max()))[1]
    scale = 2 ** k

    def fix(v):
        return round(Fraction(float(v)) * scale)

    # a band of rows keeps the rational arithmetic quick
    lo = n1 * (n1 // 2 - 20)
    hi = n1 * (n1 // 2 + 20)
    ex = fp = fx = Fraction(0)
    for I in range(lo, hi):
        if m[I] != 1:
            continue
        fr = [Fraction(float(v)) for v in (x[I], x[I - 1], x[I + 1], x[I - n1], x[I + n1])]
        r = Fraction(float(d[I])) * fr[0] + Fraction(float(bf[I])) - (fr[1] + fr[2] + fr[3] + fr[4])
        ex += r * r
        fp += Fraction(float(r64[I])) ** 2
        R = int(d[I]) * fix(x[I]) + fix(bf[I]) - (fix(x[I - 1]) + fix(x[I + 1]) + fix(x[I - n1]) + fix(x[I + n1]))
        fx += Fraction(R, scale) ** 2
    err_fp = abs(float((fp - ex) / ex))
    err_fx = abs(float((fx - ex) / ex))
    assert err_fx < err_fp / 4, (err_fx, err_fp)


def _bits(v):
    import struct

    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _to_fix_branching(v, k):
    """round(v 2^k) as first defined: a left shift for sh >= 0, else round
    half up on the magnitude; zero and subnormal v give 0."""
    u = _bits(v)
    ex = (u >> 52) & 0x7FF
    m = (u & 0x000FFFFFFFFFFFFF) | 0x0010000000000000
    sh = ex - 1075 + k
    if sh >= 0:
        r = m << sh
    else:
        s = -sh
        r = (((m >> (s - 1)) + 1) >> 1) if s <= 64 else 0
    r = r if ex else 0
    return -r if u >> 63 else r


def _to_fix_branchfree(v, k):
    """The kernels' form (ops_dev.cuh to_fix): M = m << 10, t = clamp(10 -
    sh, 1, 64), r = ((M >> (t-1)) + 1) >> 1."""
    u = _bits(v)
    ex = (u >> 52) & 0x7FF
    M = ((u & 0x000FFFFFFFFFFFFF) | 0x0010000000000000) << 10
    t = min(max(1085 - ex - k, 1), 64)
    r = (((M >> (t - 1)) + 1) >> 1) if ex else 0
    return -r if u >> 63 else r


def test_branch_free_conversion_matches_definition():
    """The branch-free fixed-point conversion of the integer residual
    kernels gives round(v 2^k) exactly as the branching definition over the
    whole range they use (|v| 2^k < 2^58), ties, subnormals and zeros
    included, and matches the exact rational rounding."""
    rng = np.random.default_rng(7)
    for E in range(-60, 61, 7):
        k = 58 - E
        vals = list(rng.uniform(-1, 1, 400) * 2.0 ** E)
        vals += list(rng.standard_normal(100) * 2.0 ** (E - rng.integers(1, 90, 100)))
        vals += [0.0, -0.0, 2.0 ** (E - 1), -(2.0 ** (E - 1)), 2.0 ** E * (1 - 2.0 ** -53), 5e-324, -5e-324,
                 2.0 ** (E - 59), 3 * 2.0 ** (E - 60), -3 * 2.0 ** (E - 60)]  # the last three: ties and a half
        for v in vals:
            v = float(v)
            if abs(v) >= 2.0 ** E:
                continue
            a, c = _to_fix_branching(v, k), _to_fix_branchfree(v, k)
            assert a == c, (v, k, a, c)
            exact = Fraction(v) * Fraction(2) ** k
            if _bits(v) & 0x7FF0000000000000:  # normal: round half away from zero
                ref = math.floor(abs(exact) + Fraction(1, 2))
                assert c == (ref if v >= 0 else -ref), (v, k, c, ref)
