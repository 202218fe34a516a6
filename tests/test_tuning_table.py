"""Tuning table of the autotuner through the C ABI (host-side only, no GPU work):
set, get, dump and clear, and the Python save/load helpers' table form."""

import ctypes as ct

import pytest

ann = pytest.importorskip("annongpu_gb300")


def test_table_round_trip():
    ann.set_tuning({}, clear=True)
    assert ann.tuning_table() == {}
    ann.set_tuning({"dev0/rbm_mc.wpb/N64.M128.U4.P0.made1": 4, "dev0/chol.update/n9216": 1})
    v, found = ct.c_int(), ct.c_int()
    ann._lib.call("ann_tuning_get", b"dev0/rbm_mc.wpb/N64.M128.U4.P0.made1", ct.byref(v), ct.byref(found))
    assert found.value == 1 and v.value == 4
    ann._lib.call("ann_tuning_get", b"dev0/absent", ct.byref(v), ct.byref(found))
    assert found.value == 0
    assert ann.tuning_table() == {"dev0/rbm_mc.wpb/N64.M128.U4.P0.made1": 4, "dev0/chol.update/n9216": 1}
    ann.set_tuning({}, clear=True)
    assert ann.tuning_table() == {}


def test_empty_key_is_rejected():
    with pytest.raises(ann.AnnError, match="empty tuning key"):
        ann._lib.call("ann_tuning_set", b"", 1)
