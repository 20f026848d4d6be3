"""C ABI checks that need no GPU: the library loads and exports every entry
point that include/cfmg.h declares; descriptor validation fails cleanly."""
import ctypes
import os
import re

import pytest

cfmg = pytest.importorskip("cfmg")
from cfmg import _lib  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cfmg_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_table():
    assert _declared("cfmg.h") == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for name in _declared("cfmg.h"):
        assert hasattr(L, name), name


def test_internal_symbols_hidden():
    # kernels and helpers are built with -fvisibility=hidden: only cfmg_* is public
    out = os.popen(f"nm -D --defined-only {_lib.LIB_PATH}").read()
    public = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert public and all(s.startswith("cfmg_") for s in public), public[:10]


def test_desc_default_is_reference_param():
    L = _lib.load()
    d = _lib.Desc()
    assert L.cfmg_desc_default(ctypes.byref(d)) == 0
    p = cfmg.Param()
    ref = p.desc()
    for f, _ in _lib.Desc._fields_:
        assert getattr(d, f) == getattr(ref, f), f


@pytest.mark.parametrize("bad", [dict(nh=1), dict(case="fourd"), dict(omega=2.5), dict(nx=0),
                                 dict(operator="varcoef", case="threed")])
def test_create_rejects_bad_param(bad):
    L = _lib.load()
    try:
        d = cfmg.Param(**bad).desc()
    except cfmg.CfmgError:
        return
    h = ctypes.c_void_p()
    rc = L.cfmg_create(ctypes.byref(d), ctypes.byref(h))
    assert rc != 0 and not h.value
    assert L.cfmg_last_error(None)


def _defines(prefix):
    src = open(os.path.join(ROOT, "include", "cfmg.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(" + prefix + r"[A-Z0-9_]+)\s+(\d+)", src)}


def test_option_and_class_tables_match_header():
    """The Python names of the option, batch-option and kernel-class codes
    are the header's #define values (a mismatch would set the wrong knob)."""
    opts = _defines("CFMG_OPT_")
    assert {("CFMG_OPT_" + k.upper()): v for k, v in _lib.OPTIONS.items()} == opts
    classes = _defines("CFMG_K_")
    assert {("CFMG_K_" + k.upper()): v for k, v in _lib.KERNEL_CLASSES.items()} == classes
    bopts = _defines("CFMG_BOPT_")
    assert {("CFMG_BOPT_" + k.upper()): v for k, v in _lib.BATCH_OPTIONS.items()} == bopts
