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
