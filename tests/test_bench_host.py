"""Host logic of bench.py (no GPU): argument defaults, the switches that
only go with --quick, and the clock summary that decides whether a run
saw throttling."""
import sys

import pytest

import bench


def _parse(*argv):
    old = sys.argv
    sys.argv = ["bench.py", *argv]
    try:
        return bench.parse()
    finally:
        sys.argv = old


def test_step_defaults():
    assert _parse().steps == 30  # config 2, our arm: long enough for the clock sampler
    assert _parse("--impl", "reference").steps == 5
    assert _parse("--workload", "config3").steps == 5
    assert _parse("--steps", "7").steps == 7


def test_earlier_forms_only_with_quick():
    a = _parse("--quick", "--host-loop", "--no-fuse", "--tb", "3", "--no-int")
    assert a.no_fuse and a.tb == 3 and a.no_int
    for flags in (("--no-fuse",), ("--tb", "1"), ("--no-int",), ("--quick", "--workload", "config3", "--no-fuse")):
        with pytest.raises(SystemExit):
            _parse(*flags)


def _summary(tmp_path, lines):
    p = tmp_path / "clocks.csv"
    p.write_text("".join(line + "\n" for line in lines))
    c = bench.Clocks(0)
    c.path = str(p)
    return c.summary()


def test_clock_summary(tmp_path):
    ok = "0, 2070, 2070, 850.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
    capped = "0, 1980, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    hot = "0, 1500, 2070, 1300.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    s = _summary(tmp_path, [ok, ok, capped])
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    s = _summary(tmp_path, [ok, hot])
    assert "hw_thermal_slowdown" in s["reasons"] and s["samples"] == 2
    assert _summary(tmp_path, [])["reasons"] == ["unsampled"]
