"""CPU-side checks of the C-ABI library: it builds, loads, and exports every
symbol that include/*.h declares; the drop-in entry points turn bad
arguments into a status before any device work (no compute calls: no GPU
here)."""
import ctypes as C
import os

import numpy as np
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


def _terms(nbody, positions, dims, spin_dim):
    from oops_gb300.expv import KronTerms
    nb = np.array(nbody, np.uint64)
    poff = np.concatenate([[0], np.cumsum(nb)]).astype(np.uint64)
    plist = np.array(positions, np.uint64)
    dlist = np.array(dims, np.uint64)
    moff = np.concatenate([[0], np.cumsum(dlist * dlist)]).astype(np.uint64)
    mats = np.ones(int(moff[-1]), np.complex128)
    return KronTerms(np.ones(len(nbody)), nb, poff, plist, dlist, moff, mats, np.array(spin_dim, np.uint64))


@pytest.mark.parametrize("terms,code,text", [
    (lambda: _terms([3], [0, 1, 2], [2, 2, 2], [2, 2, 2]), -4, "more than two bodies"),
    (lambda: _terms([2], [0, 3], [2, 2], [2, 2, 2]), -1, "position/dimension"),
    (lambda: _terms([1], [0], [3], [2, 2]), -1, "position/dimension"),
    (lambda: _terms([1], [0], [2], [2, 0]), -1, "spin dimension 0"),
])
@pytest.mark.parametrize("symbol", ["main_cache_", "main_mkl_"])
def test_drop_in_rejects_bad_term_lists_with_a_status(terms, code, text, symbol):
    """The drop-in entry points keep the reference's void signatures but
    never stop the process: term lists the reference's Fortran would stop
    on, or mis-read, come back as a status (oops_expv_status /
    oops_expv_error) before any device work (so this runs on the CPU)."""
    from oops_gb300 import expv
    t = terms()
    N = int(np.prod(t.spin_dim)) or 1
    with pytest.raises(_lib.OopsError) as e:
        expv.main_cache(t, np.ones(N, np.complex128), [1e-6], m=min(30, max(1, N - 1)),
                        use_mkl_symbol=symbol == "main_mkl_")
    assert e.value.code == code and text in str(e.value)


def test_drop_in_null_argument_is_a_status_not_a_crash():
    L = _lib.lib()
    L.main_cache_(*([None] * 24))
    assert L.oops_expv_status() == -1 and b"null" in L.oops_expv_error()
    L.main_mkl_(*([None] * 22))
    assert L.oops_expv_status() == -1
