"""C-ABI library: loads, exports every symbol include/g6gpu.h declares, and its
host-only model tables equal the oracle's.  No device work here."""
import ctypes
import os
import re

import numpy as np

import genesis6_gb300 as g6
from genesis6_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "g6gpu.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(g6_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = g6.lib()
    declared = _declared()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(_capi.SYMBOLS) == declared


def test_model_tables_match_oracle(orc):
    for m in ("TIP4P", "TIP5P", "ST2", "SPCE"):
        a = g6.model_info(m)
        b = orc.model_info(m)
        assert a["nsite"] == b["nsite"]
        assert np.array_equal(a["body"], b["body"])
        assert np.array_equal(a["param"], b["param"])
        assert a["mass"] == b["mass"] and np.array_equal(a["inertia"], b["inertia"])


def test_status_strings_and_bad_model():
    L = g6.lib()
    assert L.g6_status_string(0) == b"ok"
    ns = ctypes.c_int()
    assert L.g6_model_info(99, ctypes.byref(ns), None, None, None) == _capi.G6_ERR_ARG


def test_null_context_is_rejected():
    L = g6.lib()
    assert L.g6_system(None, 1, 1, 0, 1, None, None) == _capi.G6_ERR_ARG
    assert L.g6_force(None, None, None, None, None) == _capi.G6_ERR_ARG
