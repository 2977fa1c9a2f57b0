"""CPU-side checks of the C-ABI library: it builds, loads, and exports every
symbol that include/*.h declares; the drop-in and CCE entry points turn
bad arguments into a status and message before any device work (no
compute calls: no GPU here)."""
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


def _params(pulse_num=1, nT=11):
    from oops_gb300 import cce
    return cce.CCEParams.make(np.array([0.0, 0.0, 0.05]), np.zeros(3), np.zeros(3), pulse_num, nT, 1e-5)


# any non-null address: every case below returns before the buffers are used
FAKE = C.c_void_p(0x1000)


@pytest.mark.parametrize("k,pulse_num,nT,prec,code,text", [
    (0, 1, 11, 0, -3, "cluster size"), (7, 1, 11, 0, -3, "cluster size"),
    (3, 0, 11, 0, -3, "pulse_num"), (3, 65, 11, 0, -3, "pulse_num"),
    (3, 1, 0, 0, -3, "nT"), (3, 1, 11, 9, -1, "precision"),
])
def test_cce_entry_points_check_their_arguments(k, pulse_num, nT, prec, code, text):
    """oops_cce_coherence and oops_cce_coherence_liouville reject cluster
    sizes, pulse counts, time grids and precisions outside their ranges with
    a status and message, before any device work; no clusters is a no-op."""
    from oops_gb300 import cce
    L = cce.L_()
    p = _params(pulse_num, nT)
    assert L.oops_cce_coherence(FAKE, 10, FAKE, 5, k, C.byref(p), prec, FAKE, None) == code
    assert text in L.oops_last_error().decode()
    if prec == 0:
        bath = cce.CCEBath.make(1e4)
        assert L.oops_cce_coherence_liouville(FAKE, 10, FAKE, 5, k, C.byref(p), C.byref(bath), FAKE,
                                              None) == code
        assert text in L.oops_last_error().decode()


def test_cce_entry_points_null_pointers_and_empty_batches():
    from oops_gb300 import cce
    L = cce.L_()
    p = _params()
    assert L.oops_cce_coherence(None, 10, FAKE, 5, 3, C.byref(p), 0, FAKE, None) == -1
    assert L.oops_cce_coherence(FAKE, 10, FAKE, 0, 3, C.byref(p), 0, FAKE, None) == 0
    for rate in (-1.0, float("nan"), float("inf")):
        bath = cce.CCEBath.make(rate)
        assert L.oops_cce_coherence_liouville(FAKE, 10, FAKE, 5, 3, C.byref(p), C.byref(bath), FAKE,
                                              None) == -1
    out = np.zeros(22)
    for order in (0, 7):
        assert L.oops_ensemble_cce(10, FAKE, 5.0, order, C.byref(p), 0, out.ctypes.data, None, None,
                                   None, 0, None) == -1
        assert "max_order" in L.oops_last_error().decode()
