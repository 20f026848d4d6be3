"""Schedule and tile-form autotuner for batched solves.

The batched configuration leaves the cycle schedule open. This tuner picks
it by measurement: it builds a small stratified sample of the batch
(instances spread over the size range), solves it once with every candidate
schedule and every tile form of the blocked smoothing passes, and keeps the
pair with the least device time. It does not stop at the first iteration
count. The choice is cached in a JSON file keyed by the problem signature,
so later runs skip the trials.

A schedule is (cycle, npre, npost, omega). A tile form is the value of the
instances' ``temporal_blocking`` option: 5, the lean packed tiles (8 x 6
rows of FP32 pairs, two CTAs per SM), or 1, the scalar tiles (128 x 72, one
CTA per SM); both give the same bits, so the form changes only the time.
Every candidate must reach the tolerance on every sample instance, or it is
discarded; when none does, the caller's own schedule is kept and the report
says so.

The cache lives outside the package: $CFMG_TUNE_CACHE if set, else
$XDG_CACHE_HOME/cfmg/tuned.json (default ~/.cache/cfmg/tuned.json).
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

# tile forms of the blocked passes (the instances' temporal_blocking value)
FORMS = (5, 1)
DEFAULT_FORM = 5


def _cache_path() -> str:
    if os.environ.get("CFMG_TUNE_CACHE"):
        return os.environ["CFMG_TUNE_CACHE"]
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "cfmg", "tuned.json")


def _signature(param, sizes) -> str:
    s = np.asarray(sizes)
    return (f"{param.case}/{param.location}/{param.operator}/tol={param.tol:g}/"
            f"n={len(s)}/min={s.min()}/max={s.max()}/mean={int(s.mean())}")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d):
    try:
        os.makedirs(os.path.dirname(_cache_path()), exist_ok=True)
        with open(_cache_path(), "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def apply_form(batch, form: int) -> None:
    """Give every instance of ``batch`` the tile form ``form`` (before the
    batch's first solve, which builds its launches)."""
    for k in range(batch.n):
        batch.instance(k).set_option("temporal_blocking", int(form))


def tune(param, sizes: Sequence[int], make_sample: Callable[[object, Sequence[int]], object], sample: int = 24,
         candidates=CANDIDATES, forms=FORMS, use_cache: bool = True):
    """Return (best param, report); report["form"] is the chosen tile form,
    to be set on the full batch with ``apply_form`` before it is solved.
    ``make_sample(param, idx)`` builds a ready-to-solve cfmg.Batch of the
    instances ``idx`` with ``param``."""
    sig = _signature(param, sizes)
    cache = _load() if use_cache else {}
    if sig in cache:
        c = cache[sig]
        form = int(c.get("form", DEFAULT_FORM))
        return dataclasses.replace(param, cycle=c["cycle"], npre=c["npre"], npost=c["npost"],
                                   omega=c["omega"]), {"cached": True, "form": form, **c}
    order = np.argsort(sizes)
    idx = [int(order[k]) for k in np.linspace(0, len(sizes) - 1, min(sample, len(sizes))).round().astype(int)]
    trials = []
    for cyc, npre, npost, omega in candidates:
        p = dataclasses.replace(param, cycle=cyc, npre=npre, npost=npost, omega=omega)
        for form in forms:
            batch = make_sample(p, idx)
            apply_form(batch, form)
            batch.solve()  # builds programs and graphs
            t = time.perf_counter()
            res, nite, _ = batch.solve()
            dt = time.perf_counter() - t
            ok = bool(np.all(res <= param.tol))
            trials.append({"cycle": cyc, "npre": npre, "npost": npost, "omega": omega, "form": int(form),
                           "seconds": dt, "ok": ok, "max_cycles": int(nite.max())})
            batch.close()
    good = [t for t in trials if t["ok"]]
    if not good:  # no candidate converged on the sample: keep the caller's schedule, do not cache
        return param, {"cached": False, "best": None, "form": DEFAULT_FORM, "trials": trials,
                       "note": "no candidate reached the tolerance on every sample instance"}
    best = min(good, key=lambda t: t["seconds"])
    if use_cache:
        cache[sig] = best
        _store(cache)
    p = dataclasses.replace(param, cycle=best["cycle"], npre=best["npre"], npost=best["npost"], omega=best["omega"])
    return p, {"cached": False, "best": best, "form": best["form"], "trials": trials}
