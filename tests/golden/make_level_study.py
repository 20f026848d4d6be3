"""Writes config2_levels.json: the CPU oracle's per-cycle contraction
factors of the configuration-2 F-cycle by level count.

Configuration 2 is the 4096^2 vertex-centred 2D 9-point masked Laplacian
on a smoothed-noise coastline (sigma = 32 cells, 30 % land; seeds and
recipe in tests/workloads.py), F-cycle, Jacobi 3/3, omega 0.8. For each
level count, the oracle runs a fixed number of F-cycles from x = 0 and
records the residual history; the factor of cycle k is
sqrt(hist[k] / hist[k-1]), the contraction of ||r||_2.

The reference derives coarse masks by thresholding the restricted coverage
(compute_msk_dev, src/gmg_setup.jl:322-366). On this coastline that splits
the connected ocean into pieces once a coarse cell spans more than about
16 fine cells, and the F-cycle stops converging: the factors settle below 1
up to 5 levels and above 1 from 6 levels on, which is why the benchmark
runs 5 levels instead of the configuration's 10.

    CFMG_ORACLE_THREADS=8 python tests/golden/make_level_study.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle as O  # noqa: E402
import workloads as W  # noqa: E402

PATH = os.path.join(HERE, "config2_levels.json")
LEVELS = (3, 4, 5, 6, 7, 8, 10)
CYCLES = 6


def factors(n: int, nlevels: int, cycles: int, wet_mask=None, noise=None):
    """(history, per-cycle factors) of `cycles` oracle F-cycles on the
    configuration-2 problem of size n with `nlevels` levels."""
    param, vmsk, nz = W.config2(n, nlevels=nlevels)
    if wet_mask is not None:
        vmsk, nz = wet_mask, noise
    og = O.OracleGmg(dict(param, tol=0.0, maxite=cycles))
    og.field(1, "msk")[...] = vmsk
    og.setup_operators()
    for lev in range(1, og.nlevels + 1):
        for f in ("x", "y", "r", "b"):
            og.field(lev, f)[...] = 0.0
    og.field(1, "b")[...] = W.rhs(nz, og.field(1, "msk"))
    _, _, hist = og.solve()
    hist = [float(h) for h in hist]
    return hist, [(hist[k] / hist[k - 1]) ** 0.5 for k in range(1, len(hist))]


def main():
    out = {"n": 4096, "cycle": "f", "npre": 3, "npost": 3, "omega": 0.8, "cycles": CYCLES, "by_levels": {}}
    _, vmsk, noise = W.config2(4096)
    for nl in LEVELS:
        hist, f = factors(4096, nl, CYCLES, vmsk, noise)
        out["by_levels"][str(nl)] = {"hist": hist, "factors": f}
        print(nl, ["%.3f" % v for v in f], flush=True)
    with open(PATH, "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
