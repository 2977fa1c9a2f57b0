"""Python front end of the expv C-ABI (include/oops_expv.h).

``KronTerms`` is the flattened SumKronProd that the reference's
``MatExpVector::runInexplicitGPU`` hands to ``main_cache_``
(src/source/math/MatExp.cpp:367-420).  ``main_cache`` calls the drop-in with
host arrays exactly as that C++ caller does; ``Hamiltonian`` and
``expv_block`` expose the device-resident block API.  Device memory is held in
torch tensors; all compute runs in liboops_gb300.so.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import ExpvStats, OopsError, check, lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class KronTerms:
    coeff: np.ndarray        # float64 [nterm]      (MULTIPLIER is double)
    nbody: np.ndarray        # uint64  [nterm]
    pos_offset: np.ndarray   # uint64  [nterm+1]    0-based prefix sums of nbody
    pos_list: np.ndarray     # uint64  [total_nbody]
    dim_list: np.ndarray     # uint64  [total_nbody]
    mat_offset: np.ndarray   # uint64  [total_nbody+1]
    mats: np.ndarray         # complex128, column-major body matrices
    spin_dim: np.ndarray     # uint64  [nspin]

    @property
    def nterm(self):
        return int(self.coeff.size)

    @property
    def nspin(self):
        return int(self.spin_dim.size)

    @property
    def dim(self):
        return int(np.prod(self.spin_dim.astype(np.int64)))

    @classmethod
    def coerce(cls, t):
        """Accept any object with the same fields (e.g. a test-side copy)."""
        if isinstance(t, cls):
            return t
        return cls(*(np.ascontiguousarray(getattr(t, f)) for f in
                     ("coeff", "nbody", "pos_offset", "pos_list", "dim_list", "mat_offset",
                      "mats", "spin_dim")))

    def arrays(self):
        return (np.ascontiguousarray(self.coeff, np.float64),
                np.ascontiguousarray(self.nbody, np.uint64),
                np.ascontiguousarray(self.pos_offset, np.uint64),
                np.ascontiguousarray(self.pos_list, np.uint64),
                np.ascontiguousarray(self.dim_list, np.uint64),
                np.ascontiguousarray(self.mat_offset, np.uint64),
                np.ascontiguousarray(self.mats, np.complex128),
                np.ascontiguousarray(self.spin_dim, np.uint64))


def main_cache(terms, v, tlist, m=30, tol=1e-12, k=10, use_mkl_symbol=False):
    """Call main_cache_ (or main_mkl_) with host buffers, like
    MatExpVector::runInexplicitGPU does; returns the N x tn result."""
    t = KronTerms.coerce(terms)
    coeff, nbody, poff, plist, dlist, moff, mats, sdim = t.arrays()
    v = np.ascontiguousarray(v, np.complex128)
    ta = np.ascontiguousarray(tlist, np.float64)
    N = t.dim
    w = np.zeros((ta.size, N), np.complex128)
    s = lambda x: C.byref(C.c_size_t(int(x)))
    nspin, nterm, ndim = C.c_size_t(t.nspin), C.c_size_t(t.nterm), C.c_size_t(N)
    pos_idx, mat_idx = C.c_size_t(int(poff[-1]) if poff.size else 0), C.c_size_t(mats.size)
    kk, tn, mm, itr = C.c_size_t(k), C.c_size_t(ta.size), C.c_size_t(m), C.c_size_t(0)
    tl = C.c_double(tol)
    wlen = C.c_size_t(w.size)
    L = lib()
    szp = C.POINTER(C.c_size_t)
    dp = C.POINTER(C.c_double)
    args_head = [C.byref(nspin), C.byref(nterm), coeff.ctypes.data_as(dp),
                 nbody.ctypes.data_as(szp), poff.ctypes.data_as(szp), plist.ctypes.data_as(szp),
                 dlist.ctypes.data_as(szp), moff.ctypes.data_as(szp), _p(mats), C.byref(ndim),
                 sdim.ctypes.data_as(szp), _p(v), C.byref(pos_idx), C.byref(mat_idx), C.byref(kk)]
    if use_mkl_symbol:
        L.main_mkl_(*args_head, C.byref(tn), ta.ctypes.data_as(dp), C.byref(mm), C.byref(tl),
                    C.byref(itr), _p(w), C.byref(wlen))
    else:
        mtpb = C.c_size_t(256)
        mgs = (C.c_size_t * 3)(2147483647, 65535, 65535)
        L.main_cache_(*args_head, C.byref(mtpb), mgs, C.byref(tn), ta.ctypes.data_as(dp),
                      C.byref(mm), C.byref(tl), C.byref(itr), _p(w), C.byref(wlen))
    rc = L.oops_expv_status()
    if rc != 0:
        raise OopsError(rc, L.oops_expv_error().decode())
    return w.T.copy()


class Hamiltonian:
    """Device-resident Kronecker Hamiltonian (oops_ham handle)."""

    def __init__(self, terms):
        t = KronTerms.coerce(terms)
        self._arrays = t.arrays()
        coeff, nbody, poff, plist, dlist, moff, mats, sdim = self._arrays
        h = C.c_void_p()
        check(lib().oops_ham_create(t.nspin, t.nterm, _p(coeff), _p(nbody), _p(poff), _p(plist),
                                    _p(dlist), _p(moff), _p(mats), _p(sdim), C.byref(h)))
        self._h = h
        self.dim = int(lib().oops_ham_dim(h))

    def close(self):
        if getattr(self, "_h", None):
            lib().oops_ham_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def apply(self, x, alpha=1.0, out=None, stream=None):
        """y = alpha * H x for a torch complex128 CUDA tensor of shape (N,) or
        (N, nvec) (row-major: vectors interleaved), nvec a power of two."""
        import torch
        if not (x.is_cuda and x.dtype == torch.complex128 and x.is_contiguous()):
            raise OopsError(-1, "x must be a contiguous complex128 CUDA tensor")
        nvec = 1 if x.dim() == 1 else x.shape[1]
        y = torch.empty_like(x) if out is None else out
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        a = complex(alpha)
        check(lib().oops_ham_apply(self._h, a.real, a.imag, C.c_void_p(x.data_ptr()),
                                   C.c_void_p(y.data_ptr()), nvec, C.c_void_p(st)))
        return y


def expv_block(ham: Hamiltonian, V, T, m=30, tol=1e-12, k=10, stream=None):
    """W[tt, :, b] = exp(-i H T[tt, b]) V[:, b].  V: torch complex128 CUDA
    (N, nvec) row-major; T: (tn, nvec) increasing per column.  Returns a torch
    tensor (tn, N, nvec) and column 0's counters."""
    import torch
    if not (V.is_cuda and V.dtype == torch.complex128 and V.is_contiguous()):
        raise OopsError(-1, "V must be a contiguous complex128 CUDA tensor")
    if V.dim() == 1:
        V = V.reshape(-1, 1)
    N, nvec = V.shape
    T = np.asarray(T, np.float64)
    if T.ndim == 1:
        T = np.repeat(T[:, None], nvec, axis=1)
    tn = T.shape[0]
    ta = np.ascontiguousarray(T.T)  # column b's times contiguous
    W = torch.empty((tn, N, nvec), dtype=torch.complex128, device=V.device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    stats = ExpvStats()
    check(lib().oops_expv_block(ham.handle, C.c_void_p(V.data_ptr()), nvec, tn, _p(ta), m, tol,
                                k, C.c_void_p(W.data_ptr()), C.byref(stats), C.c_void_p(st)))
    return W, stats
