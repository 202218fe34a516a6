"""The C ABI library loads and exports every entry point include/annongpu.h declares
(no compute calls: this runs without a GPU)."""

import ctypes as ct
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "annongpu.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ann_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    return ct.CDLL(os.path.join(ROOT, "annongpu_gb300", "libannongpu.so"))


def test_header_declares_entry_points():
    names = declared()
    assert "ann_tdvp_eval" in names and "ann_sr_step" in names and len(names) > 50


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from annongpu_gb300 import _lib
    missing = [n for n in declared() if n not in _lib._SIGS]
    assert not missing, missing


def test_error_reporting_without_device(lib):
    lib.ann_last_error.restype = ct.c_char_p
    assert lib.ann_version() >= 10000
    # argument validation happens before any device work
    out = ct.c_void_p()
    rc = lib.ann_ens_create_exact(40, ct.byref(out))
    assert rc == 1
    assert b"exact summation" in lib.ann_last_error()


def test_factor_trace_levels_without_device(lib):
    """ann_set_factor_trace takes 0 (off), 1 (panel pairs) or 2 (also between the panel
    kernels); anything else is rejected before any device work."""
    lib.ann_last_error.restype = ct.c_char_p
    for level in (0, 1, 2, 0):
        assert lib.ann_set_factor_trace(level) == 0
    assert lib.ann_set_factor_trace(3) == 1
    assert b"factor trace level" in lib.ann_last_error()
    assert lib.ann_set_factor_trace(-1) == 1
    n = ct.c_uint(7)
    assert lib.ann_get_factor_trace(None, 0, ct.byref(n)) == 0 and n.value == 0
