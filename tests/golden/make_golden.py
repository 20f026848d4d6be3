"""Writes oracle_solves.json: the CPU oracle's solves of the scenarios of
``fixtures.golden_scenarios()`` (the reference suite's known-answer cases,
the rectangular pair, the iteration-count cases with exactly computed
right-hand sides, and the plain-method configuration 1 with its seeded
N(0,1) right-hand side).

Per scenario: the iteration count, the final residual ratio, the residual
history of every iteration, and SHA-256 digests of the right-hand side and
of the final level-1 x and r
(``fixtures.field_digest``). The oracle's pointwise arithmetic and its
sequential norms are plain IEEE FP64 operations on exactly representable
inputs, so the values do not depend on the host.

    python tests/golden/make_golden.py
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import fixtures as F  # noqa: E402
import oracle as O  # noqa: E402


def solve(sc):
    og = O.OracleGmg(sc.param)
    b = F.prepare(F.OracleAdapter(og), sc)
    res, nite, hist = og.solve()
    x = og.x
    return {
        "b_sha256": F.field_digest(b),
        "param": sc.param,
        "nite": int(nite),
        "res": float(res),
        "hist": [float(h) for h in hist],
        "x_sha256": F.field_digest(x),
        "r_sha256": F.field_digest(og.field(1, "r")),
        "x_abs_sum": math.fsum(abs(float(v)) for v in x.ravel(order="F")),
    }


def main():
    out = {}
    for sc in F.golden_scenarios():
        out[sc.name] = solve(sc)
        print(sc.name, out[sc.name]["nite"], out[sc.name]["res"], flush=True)
    with open(F.GOLDEN_PATH, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
