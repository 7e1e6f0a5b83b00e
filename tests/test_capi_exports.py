"""The C-ABI library loads and exports every entry point include/panslbm_gb300.h declares
(no compute call: runs without a GPU)."""
import ctypes
import os
import re

import pytest

from panslbm2_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:int|long long|const char \*|double)\s*\*?\s*(pl_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    assert "pl_create" in names and "pl_solve" in names and len(names) >= 25


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_capi.LIB_PATH):
        pytest.skip("CUDA library not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(_capi.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_capi.EXPORTS) <= set(declared())
