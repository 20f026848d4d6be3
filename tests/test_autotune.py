"""Batch autotuner logic (cfmg/autotune.py) on the CPU, with a stand-in for
the batched solver: the tuner must try every (schedule, tile form) pair,
keep only pairs that converge on every sample instance, take the fastest of
those, apply the form to every instance before the first solve, and cache
the choice outside the package directory."""
import dataclasses
import json
import os

import numpy as np
import pytest

from cfmg import autotune


@dataclasses.dataclass
class _P:
    case: str = "twod"
    location: str = "centers"
    operator: str = "laplacian"
    tol: float = 1e-10
    cycle: str = "v"
    npre: int = 2
    npost: int = 2
    omega: float = 0.8


class _Clock:
    t = 0.0

    def __call__(self):
        return self.t


class _Inst:
    def __init__(self):
        self.opts = {}

    def set_option(self, name, value):
        self.opts[name] = value


class _Batch:
    """solve() advances the clock by cost(schedule, form) and converges
    unless the schedule is in `fail`."""

    def __init__(self, p, idx, clock, cost, fail, log):
        self.p, self.n, self.clock, self.cost, self.fail, self.log = p, len(idx), clock, cost, fail, log
        self.inst = [_Inst() for _ in idx]
        self.solved = False

    def instance(self, k):
        assert not self.solved, "the form must be set before the first solve"
        return self.inst[k]

    def solve(self):
        self.solved = True
        forms = {i.opts.get("temporal_blocking") for i in self.inst}
        assert len(forms) == 1
        form = forms.pop()
        key = (self.p.cycle, self.p.npre, self.p.npost, self.p.omega)
        self.clock.t += self.cost(key, form)
        self.log.append((key, form))
        bad = key in self.fail
        res = np.full(self.n, 1e-3 if bad else 1e-11)
        return res, np.full(self.n, 200 if bad else 20), np.zeros(self.n)

    def close(self):
        pass


def _run(monkeypatch, tmp_path, cost, fail=()):
    clock, log = _Clock(), []
    monkeypatch.setattr(autotune.time, "perf_counter", clock)
    monkeypatch.setenv("CFMG_TUNE_CACHE", str(tmp_path / "tuned.json"))
    sizes = list(np.linspace(64, 1024, 100).astype(int))
    make = lambda p, idx: _Batch(p, idx, clock, cost, set(fail), log)
    p, rep = autotune.tune(_P(), sizes, make)
    return p, rep, log


def test_tunes_schedule_and_form_together(monkeypatch, tmp_path):
    # fastest overall: F(2,2) with the scalar tiles; V(2,2,0.8) is faster but
    # does not converge and must not be chosen
    def cost(key, form):
        base = {("v", 2, 2, 0.8): 0.5, ("f", 2, 2, 0.8): 1.0}.get(key, 2.0)
        return base * (0.9 if (key[0] == "f" and form == 1) else 1.0)

    p, rep, log = _run(monkeypatch, tmp_path, cost, fail=[("v", 2, 2, 0.8)])
    assert (p.cycle, p.npre, p.npost, p.omega) == ("f", 2, 2, 0.8)
    assert rep["form"] == 1 and rep["best"]["form"] == 1
    tried = {(k, f) for k, f in log}
    assert tried == {(c, f) for c in autotune.CANDIDATES for f in autotune.FORMS}
    assert all(not t["ok"] for t in rep["trials"] if t["cycle"] == "v" and t["npre"] == 2 and t["omega"] == 0.8)


def test_no_converging_candidate_keeps_caller_schedule(monkeypatch, tmp_path):
    p, rep, _ = _run(monkeypatch, tmp_path, lambda k, f: 1.0, fail=autotune.CANDIDATES)
    assert p == _P() and rep["best"] is None and rep["form"] == autotune.DEFAULT_FORM
    assert not os.path.exists(tmp_path / "tuned.json")  # nothing cached


def test_cache_outside_package_and_reused(monkeypatch, tmp_path):
    cost = lambda k, f: 1.0 if (k[0] == "f" and f == 5) else 2.0
    p1, rep1, log1 = _run(monkeypatch, tmp_path, cost)
    cache = tmp_path / "tuned.json"
    assert cache.exists()
    pkg = os.path.dirname(os.path.abspath(autotune.__file__))
    assert not os.path.abspath(autotune._cache_path()).startswith(pkg)
    entry = next(iter(json.loads(cache.read_text()).values()))
    assert entry["form"] == 5
    p2, rep2, log2 = _run(monkeypatch, tmp_path, cost)
    assert log2 == [] and rep2["cached"] and rep2["form"] == rep1["form"] == 5
    assert (p2.cycle, p2.npre) == (p1.cycle, p1.npre)


def test_default_cache_path_is_user_cache(monkeypatch):
    monkeypatch.delenv("CFMG_TUNE_CACHE", raising=False)
    monkeypatch.setenv("XDG_CACHE_HOME", "/tmp/xdg-test")
    assert autotune._cache_path() == os.path.join("/tmp/xdg-test", "cfmg", "tuned.json")


def test_apply_form_sets_every_instance():
    class B:
        n = 3
        inst = [_Inst() for _ in range(3)]

        def instance(self, k):
            return self.inst[k]

    b = B()
    autotune.apply_form(b, 1)
    assert all(i.opts["temporal_blocking"] == 1 for i in b.inst)
