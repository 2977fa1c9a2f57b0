"""CPU-side checks of the C-ABI library: it builds, loads, and exports every
symbol that include/*.h declares (no compute calls: no GPU here)."""
import ctypes as C
import os

import pytest

from oops_gb300 import _lib
from oops_gb300 import build as b


def test_library_builds_and_exports_header_symbols():
    path = b.build()
    assert os.path.exists(path)
    L = C.CDLL(path)
    names = _lib.header_symbols()
    assert "main_cache_" in names and "main_mkl_" in names and "oops_expv_block" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_api_without_gpu_calls():
    L = _lib.lib()
    assert L.oops_expv_status() == 0
    assert L.oops_expv_error() == b""
