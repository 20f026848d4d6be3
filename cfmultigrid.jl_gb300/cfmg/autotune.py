"""Schedule autotuner for batched solves.

The batched configuration leaves the cycle schedule open. This tuner picks
it by measurement: it builds a small stratified sample of the batch
(instances spread over the size range), solves it once with every candidate
schedule, and keeps the one with the least device time. It does not stop
at the first iteration count. The choice is cached in a JSON file keyed by
the problem signature, so later runs skip the trials.

A candidate is (cycle, npre, npost, omega). Every candidate must reach the
tolerance on every sample instance, or it is discarded.
"""
from __future__ import annotations

import dataclasses
import json
import os
import time
from typing import Callable, Sequence

import numpy as np

CANDIDATES = [
    ("v", 2, 2, 0.8),
    ("v", 3, 3, 0.8),
    ("f", 2, 2, 0.8),
    ("v", 2, 2, 0.9),
    ("f", 1, 1, 0.9),
]

_CACHE = os.environ.get("CFMG_TUNE_CACHE", os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json"))


def _signature(param, sizes) -> str:
    s = np.asarray(sizes)
    return (f"{param.case}/{param.location}/{param.operator}/tol={param.tol:g}/"
            f"n={len(s)}/min={s.min()}/max={s.max()}/mean={int(s.mean())}")


def _load():
    try:
        with open(_CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d):
    try:
        with open(_CACHE, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def tune(param, sizes: Sequence[int], make_sample: Callable[[object, Sequence[int]], object], sample: int = 24,
         candidates=CANDIDATES, use_cache: bool = True):
    """Return (best param, report). ``make_sample(param, idx)`` builds a
    ready-to-solve cfmg.Batch of the instances ``idx`` with ``param``."""
    sig = _signature(param, sizes)
    cache = _load() if use_cache else {}
    if sig in cache:
        c = cache[sig]
        return dataclasses.replace(param, cycle=c["cycle"], npre=c["npre"], npost=c["npost"],
                                   omega=c["omega"]), {"cached": True, **c}
    order = np.argsort(sizes)
    idx = [int(order[k]) for k in np.linspace(0, len(sizes) - 1, min(sample, len(sizes))).round().astype(int)]
    trials = []
    for cyc, npre, npost, omega in candidates:
        p = dataclasses.replace(param, cycle=cyc, npre=npre, npost=npost, omega=omega)
        batch = make_sample(p, idx)
        batch.solve()  # builds programs and graphs
        t = time.perf_counter()
        res, nite, _ = batch.solve()
        dt = time.perf_counter() - t
        ok = bool(np.all(res <= param.tol))
        trials.append({"cycle": cyc, "npre": npre, "npost": npost, "omega": omega, "seconds": dt, "ok": ok,
                       "max_cycles": int(nite.max())})
        batch.close()
    good = [t for t in trials if t["ok"]] or trials
    best = min(good, key=lambda t: t["seconds"])
    if use_cache:
        cache[sig] = best
        _store(cache)
    p = dataclasses.replace(param, cycle=best["cycle"], npre=best["npre"], npost=best["npost"], omega=best["omega"])
    return p, {"cached": False, "best": best, "trials": trials}
