"""ctypes binding of liboops_gb300.so (the C-ABI declared in include/*.h).

The library is built in-tree (oops_gb300/build.py).  Loading fails loudly when
it is missing or when no CUDA device is present for a compute call: there is
no CPU path in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "liboops_gb300.so")
HEADERS = [os.path.join(ROOT, "include", f) for f in ("oops_expv.h", "oops_cce.h")]

_lib = None

vp = C.c_void_p
sz = C.c_size_t
szp = C.POINTER(C.c_size_t)
dp = C.POINTER(C.c_double)

OOPS_OK = 0
STATUS_NAMES = {0: "OOPS_OK", -1: "OOPS_ERR_ARG", -3: "OOPS_ERR_SIZE",
                -4: "OOPS_ERR_UNSUPPORTED", -5: "OOPS_ERR_CUDA", -6: "OOPS_ERR_NOMEM",
                -7: "OOPS_ERR_NUMERIC", -8: "OOPS_ERR_TIMEOUT"}


class OopsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class ExpvStats(C.Structure):
    _fields_ = [("nmult", C.c_long), ("nexph", C.c_long), ("nscale", C.c_long),
                ("nstep", C.c_long), ("nreject", C.c_long), ("ibrkflag", C.c_long),
                ("mbrkdwn", C.c_long), ("anorm", C.c_double), ("step_min", C.c_double),
                ("step_max", C.c_double), ("x_error", C.c_double), ("s_error", C.c_double),
                ("hump", C.c_double)]


def header_symbols():
    """Function names declared in include/*.h."""
    names = []
    for h in HEADERS:
        if not os.path.exists(h):
            continue
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt):
            name = m.group(1)
            if name in ("if", "sizeof", "defined") or name.isupper():
                continue
            prefix = txt[:m.start()].rstrip()
            if prefix.endswith(("typedef", "#define")):
                continue
            names.append(name)
    seen, out = set(), []
    for n in names:
        if n not in seen and (n.startswith("oops_") or n.endswith("_")):
            seen.add(n)
            out.append(n)
    return out


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OopsError(-5, f"{LIB_PATH} is missing: run oops_gb300/build.py (nvcc) first")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    drop = [szp, szp, dp, szp, szp, szp, szp, szp, vp, szp, szp, vp, szp, szp, szp]
    L.main_cache_.restype = None
    L.main_cache_.argtypes = drop + [szp, szp, szp, dp, szp, dp, szp, vp, szp]
    L.main_mkl_.restype = None
    L.main_mkl_.argtypes = drop + [szp, dp, szp, dp, szp, vp, szp]
    L.oops_expv_status.restype = C.c_int
    L.oops_expv_error.restype = C.c_char_p
    L.oops_last_status.restype = C.c_int
    L.oops_last_error.restype = C.c_char_p
    L.oops_ham_create.restype = C.c_int
    L.oops_ham_create.argtypes = [sz, sz, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(vp)]
    L.oops_ham_destroy.restype = C.c_int
    L.oops_ham_destroy.argtypes = [vp]
    L.oops_ham_dim.restype = sz
    L.oops_ham_dim.argtypes = [vp]
    L.oops_ham_apply.restype = C.c_int
    L.oops_ham_apply.argtypes = [vp, C.c_double, C.c_double, vp, vp, sz, vp]
    L.oops_expv_block.restype = C.c_int
    L.oops_expv_block.argtypes = [vp, vp, sz, sz, vp, sz, C.c_double, sz, vp,
                                  C.POINTER(ExpvStats), vp]
    _declare_cce(L)


def _declare_cce(L):
    if not hasattr(L, "oops_cce_batch_create"):
        return
    L.oops_cce_batch_create.restype = C.c_int
    L.oops_cce_batch_destroy.restype = C.c_int
    L.oops_cce_batch_destroy.argtypes = [vp]


def check(rc):
    if rc != OOPS_OK:
        msg = lib().oops_last_error()
        raise OopsError(rc, msg.decode() if msg else "")
    return rc
