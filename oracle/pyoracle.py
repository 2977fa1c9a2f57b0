"""ctypes front end of the CPU oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs may import this module; the product package never does.

The term-list format is the one ``MatExpVector::runInexplicit`` flattens a
``SumKronProd`` into (src/source/math/MatExp.cpp:216-270) and hands to
``main_mkl_`` / ``main_cache_``: real coefficients, body counts, 0-based
position offsets, spin positions, body dimensions, matrix offsets and the
column-major body matrices.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

c_size_p = C.POINTER(C.c_size_t)
c_double_p = C.POINTER(C.c_double)


def build() -> str:
    """Compile liboracle.so (and the reference matvec pin when the reference
    tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref = os.path.join(HERE, "build_ref.sh")
    subprocess.run(["sh", ref], check=True, stdout=subprocess.DEVNULL)
    return os.path.join(HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        src = os.path.join(HERE, "oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = C.CDLL(path)
        _declare(_LIB)
    return _LIB


def ref_lib():
    """The reference's own hamvec_func3.cpp, if oracle/_ref was built."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libref_hamvec.so")
        if not os.path.exists(path):
            return None
        _REF = C.CDLL(path)
    return _REF


class ExpvStats(C.Structure):
    _fields_ = [("anorm", C.c_double), ("nmult", C.c_long), ("nexph", C.c_long),
                ("nscale", C.c_long), ("nstep", C.c_long), ("nreject", C.c_long),
                ("ibrkflag", C.c_long), ("mbrkdwn", C.c_long), ("step_min", C.c_double),
                ("step_max", C.c_double), ("x_error", C.c_double), ("s_error", C.c_double),
                ("hump", C.c_double), ("tbrkdwn", C.c_double), ("t_now", C.c_double),
                ("iflag", C.c_int)]


def _declare(L):
    vp = C.c_void_p
    L.orc_dlaran.restype = C.c_double
    L.orc_dlaran.argtypes = [C.POINTER(C.c_int)]
    L.orc_kron_mode.argtypes = [C.c_size_t, C.c_size_t, C.c_size_t, vp, vp]
    L.orc_hamvec.argtypes = [C.c_size_t, C.c_size_t, vp, vp, vp, vp, vp, vp, vp,
                             C.c_size_t, vp, vp, vp, vp]
    L.orc_padm.restype = C.c_int
    L.orc_padm.argtypes = [C.c_int, C.c_int, C.c_double, vp, C.c_int, vp,
                           C.POINTER(C.c_int)]
    L.orc_expv.restype = C.c_int
    L.orc_expv.argtypes = [C.c_size_t, C.c_size_t, vp, vp, vp, vp, vp, vp, vp,
                           C.c_size_t, vp, vp, C.c_size_t, C.c_size_t, vp,
                           C.c_size_t, C.c_double, vp, C.POINTER(ExpvStats)]
    L.orc_expv_block.restype = C.c_int
    L.orc_expv_block.argtypes = [C.c_size_t, C.c_size_t, vp, vp, vp, vp, vp, vp,
                                 vp, C.c_size_t, vp, vp, C.c_size_t, C.c_size_t,
                                 C.c_size_t, vp, C.c_size_t, C.c_double, vp]
    L.orc_dipole.argtypes = [vp, vp, C.c_double, C.c_double, vp]
    L.orc_nv_states.argtypes = [vp, vp, vp]
    L.orc_cluster_hamiltonian.restype = C.c_size_t
    L.orc_cluster_hamiltonian.argtypes = [C.c_size_t, vp, C.c_double, vp, vp,
                                          C.c_double, vp, vp, vp, vp, vp, vp, vp, vp]
    L.orc_dense_hamiltonian.argtypes = [C.c_size_t, C.c_size_t, vp, vp, vp, vp, vp,
                                        vp, vp, vp, vp]
    L.orc_cpmg_intervals.argtypes = [C.c_int, vp]
    L.orc_coherence_hilbert.argtypes = [C.c_size_t, vp, vp, C.c_int, C.c_size_t,
                                        C.c_double, vp]
    L.orc_coherence_state.argtypes = [C.c_size_t, vp, vp, C.c_int, C.c_size_t, C.c_double,
                                      C.c_size_t, vp]
    L.orc_coherence_liouville.argtypes = [C.c_size_t, vp, vp, C.c_int, C.c_size_t,
                                          C.c_double, C.c_double, vp, vp, vp]
    L.orc_enumerate.restype = vp
    L.orc_enumerate.argtypes = [C.c_size_t, vp, C.c_double, C.c_int]
    L.orc_enum_count.restype = C.c_size_t
    L.orc_enum_count.argtypes = [vp, C.c_int]
    L.orc_enum_cluster.argtypes = [vp, C.c_int, C.c_size_t, vp]
    L.orc_enum_parents.restype = C.c_size_t
    L.orc_enum_parents.argtypes = [vp, C.c_int, C.c_size_t, vp, C.c_size_t]
    L.orc_enum_subclusters.restype = C.c_size_t
    L.orc_enum_subclusters.argtypes = [vp, C.c_int, C.c_size_t, vp, C.c_size_t]
    L.orc_enum_free.argtypes = [vp]
    L.orc_cce_reduce.argtypes = [vp, C.c_int, C.c_size_t, vp, vp, vp, vp]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# term lists
# --------------------------------------------------------------------------
@dataclass
class KronTerms:
    """A flattened SumKronProd (MatExp.cpp:216-270)."""
    coeff: np.ndarray        # float64 [nterm]
    nbody: np.ndarray        # uint64 [nterm]
    pos_offset: np.ndarray   # uint64 [nterm+1]
    pos_list: np.ndarray     # uint64 [total_nbody]
    dim_list: np.ndarray     # uint64 [total_nbody]
    mat_offset: np.ndarray   # uint64 [total_nbody+1]
    mats: np.ndarray         # complex128 [total_dim]
    spin_dim: np.ndarray     # uint64 [nspin]

    @property
    def nterm(self):
        return int(self.coeff.size)

    @property
    def nspin(self):
        return int(self.spin_dim.size)

    @property
    def dim(self):
        return int(np.prod(self.spin_dim.astype(np.int64)))

    @staticmethod
    def from_list(spin_dim, terms):
        """terms: list of (coeff, [(pos, matrix), ...])."""
        coeff, nbody, pos, dims, mats, moff = [], [], [], [], [], [0]
        for c, bodies in terms:
            coeff.append(float(c))
            nbody.append(len(bodies))
            for p, M in bodies:
                M = np.asarray(M, dtype=np.complex128)
                pos.append(int(p))
                dims.append(M.shape[0])
                mats.append(M.reshape(-1, order="F"))
                moff.append(moff[-1] + M.size)
        poff = np.concatenate([[0], np.cumsum(nbody)]).astype(np.uint64)
        return KronTerms(np.asarray(coeff, np.float64), np.asarray(nbody, np.uint64), poff,
                         np.asarray(pos, np.uint64), np.asarray(dims, np.uint64),
                         np.asarray(moff, np.uint64),
                         np.concatenate(mats).astype(np.complex128) if mats else
                         np.zeros(0, np.complex128),
                         np.asarray(spin_dim, np.uint64))


# --------------------------------------------------------------------------
# wrappers
# --------------------------------------------------------------------------
def dlaran_sequence(n, seed=(0, 0, 0, 5)):
    s = (C.c_int * 4)(*seed)
    return np.array([lib().orc_dlaran(s) for _ in range(n)]), tuple(s)


def kron_mode(m, s, n, A, x):
    x = np.ascontiguousarray(x, np.complex128).copy()
    A = np.asfortranarray(A, np.complex128).reshape(-1, order="F").copy()
    lib().orc_kron_mode(m, s, n, _p(A), _p(x))
    return x


def hamvec(t: KronTerms, v, coeffz=None):
    v = np.ascontiguousarray(v, np.complex128)
    cz = t.coeff.astype(np.complex128) if coeffz is None else np.asarray(coeffz, np.complex128)
    w = np.zeros_like(v)
    wm = np.zeros_like(v)
    lib().orc_hamvec(t.nspin, t.nterm, _p(cz), _p(t.nbody), _p(t.pos_offset), _p(t.pos_list),
                     _p(t.dim_list), _p(t.mat_offset), _p(t.mats), v.size, _p(t.spin_dim),
                     _p(v), _p(w), _p(wm))
    return w


def ref_hamvec(t: KronTerms, v, coeffz=None):
    """Run the reference's own hamvec_func3_ (oracle/_ref), or None."""
    R = ref_lib()
    if R is None:
        return None
    v = np.ascontiguousarray(v, np.complex128)
    cz = t.coeff.astype(np.complex128) if coeffz is None else np.asarray(coeffz, np.complex128)
    nspin = C.c_int(t.nspin)
    nterm = C.c_int(t.nterm)
    dims = t.spin_dim.astype(np.uint64)
    mlst = np.array([int(np.prod(dims[:i].astype(np.int64))) for i in range(t.nspin)], np.uint64)
    nlst = np.array([int(np.prod(dims[i + 1:].astype(np.int64))) for i in range(t.nspin)], np.uint64)
    vlen = C.c_size_t(v.size)
    w = np.zeros_like(v)
    wm = np.zeros_like(v)
    R.hamvec_func3_(C.byref(nspin), C.byref(nterm), _p(cz), _p(t.nbody), _p(t.pos_offset),
                    _p(t.pos_list), _p(t.dim_list), _p(t.mat_offset), _p(t.mats), C.byref(vlen),
                    _p(dims), _p(mlst), _p(nlst), _p(v), _p(w), _p(wm))
    return w


def padm(H, t=1.0, ideg=6):
    H = np.asfortranarray(H, np.complex128)
    m = H.shape[0]
    E = np.zeros((m, m), np.complex128, order="F")
    ns = C.c_int(0)
    rc = lib().orc_padm(ideg, m, float(t), _p(H), m, _p(E), C.byref(ns))
    if rc != 0:
        raise RuntimeError(f"orc_padm failed: {rc}")
    return E, ns.value


def expv(t: KronTerms, v, tlist, m=30, tol=1e-12, klim=10):
    v = np.ascontiguousarray(v, np.complex128)
    tl = np.ascontiguousarray(tlist, np.float64)
    n = t.dim
    w = np.zeros((tl.size, n), np.complex128)
    st = ExpvStats()
    rc = lib().orc_expv(t.nspin, t.nterm, _p(t.coeff), _p(t.nbody), _p(t.pos_offset),
                        _p(t.pos_list), _p(t.dim_list), _p(t.mat_offset), _p(t.mats), n,
                        _p(t.spin_dim), _p(v), klim, tl.size, _p(tl), m, tol, _p(w),
                        C.byref(st))
    if rc != 0:
        raise RuntimeError(f"orc_expv failed: {rc}")
    return w.T.copy(), st     # n x tn, column tt = w(ta[tt])


def expv_block(t: KronTerms, V, T, m=30, tol=1e-12, klim=10):
    """V: n x nvec, T: tn x nvec (per-column times). Returns n x tn x nvec."""
    V = np.asfortranarray(V, np.complex128)
    T = np.asfortranarray(T, np.float64)
    n, nvec = V.shape
    tn = T.shape[0]
    W = np.zeros((n, tn, nvec), np.complex128, order="F")
    rc = lib().orc_expv_block(t.nspin, t.nterm, _p(t.coeff), _p(t.nbody), _p(t.pos_offset),
                              _p(t.pos_list), _p(t.dim_list), _p(t.mat_offset), _p(t.mats),
                              n, _p(t.spin_dim), _p(V), nvec, klim, tn, _p(T), m, tol, _p(W))
    if rc != 0:
        raise RuntimeError(f"orc_expv_block failed: {rc}")
    return W


def dipole(c1, c2, g1, g2):
    c1 = np.asarray(c1, np.float64)
    c2 = np.asarray(c2, np.float64)
    out = np.zeros(9)
    lib().orc_dipole(_p(c1), _p(c2), g1, g2, _p(out))
    return out


def nv_states(B):
    B = np.asarray(B, np.float64)
    ev = np.zeros(3)
    sv = np.zeros(9)
    lib().orc_nv_states(_p(B), _p(ev), _p(sv))
    return ev, sv.reshape(3, 3)


GAMMA_C13 = 6.728284e7
GAMMA_NVE = -1.760859708e11


def cluster_hamiltonian(coords, B, center, sv, g=GAMMA_C13, gc=GAMMA_NVE) -> KronTerms:
    coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 3)
    k = coords.shape[0]
    cap = 9 * k * (k - 1) // 2 + 12 * k + 1
    coeff = np.zeros(cap)
    nbody = np.zeros(cap, np.uint64)
    pidx = np.zeros(cap + 1, np.uint64)
    plist = np.zeros(2 * cap, np.uint64)
    dlist = np.zeros(2 * cap, np.uint64)
    moff = np.zeros(2 * cap + 1, np.uint64)
    mats = np.zeros(8 * cap, np.complex128)
    B = np.asarray(B, np.float64)
    cc = np.asarray(center, np.float64)
    sv = np.asarray(sv, np.float64)
    nt = lib().orc_cluster_hamiltonian(k, _p(coords), g, _p(B), _p(cc), gc, _p(sv), _p(coeff),
                                       _p(nbody), _p(pidx), _p(plist), _p(dlist), _p(moff),
                                       _p(mats))
    nb = int(pidx[nt])
    return KronTerms(coeff[:nt].copy(), nbody[:nt].copy(), pidx[:nt + 1].copy(),
                     plist[:nb].copy(), dlist[:nb].copy(), moff[:nb + 1].copy(),
                     mats[:4 * nb].copy(), np.full(k, 2, np.uint64))


def dense_hamiltonian(t: KronTerms):
    D = t.dim
    H = np.zeros((D, D), np.complex128, order="F")
    lib().orc_dense_hamiltonian(t.nspin, t.nterm, _p(t.coeff), _p(t.nbody), _p(t.pos_offset),
                                _p(t.pos_list), _p(t.dim_list), _p(t.mat_offset), _p(t.mats),
                                _p(t.spin_dim), _p(H))
    return H


def cpmg_intervals(n):
    f = np.zeros(n + 1)
    lib().orc_cpmg_intervals(n, _p(f))
    return f


def coherence_hilbert(H0, H1, pulse_num, nT, dt):
    H0 = np.asfortranarray(H0, np.complex128)
    H1 = np.asfortranarray(H1, np.complex128)
    L = np.zeros(nT)
    lib().orc_coherence_hilbert(H0.shape[0], _p(H0), _p(H1), pulse_num, nT, dt, _p(L))
    return L


def coherence_state(H0, H1, pulse_num, nT, dt, b):
    """Single-sample observable of basis state b (orc_coherence_state)."""
    H0 = np.asfortranarray(H0, np.complex128)
    H1 = np.asfortranarray(H1, np.complex128)
    L = np.zeros(nT)
    lib().orc_coherence_state(H0.shape[0], _p(H0), _p(H1), pulse_num, nT, dt, int(b), _p(L))
    return L


def bath_field(coords, state, cluster, g=GAMMA_C13):
    """Mean dipolar field on each spin of `cluster` from the bath spins outside
    it in product state `state` (0: up, 1: down along z): DipolarField with the
    cluster masked out (SpinInteraction.cpp:150-165; dipole_field, misc.cpp:
    50-57).  Returns (k, 3) in rad/s."""
    coords = np.asarray(coords, np.float64)
    out = np.zeros((len(cluster), 3))
    inside = set(int(c) for c in cluster)
    for s, i in enumerate(cluster):
        for j in range(len(coords)):
            if j in inside:
                continue
            t9 = np.zeros(9)
            lib().orc_dipole(_p(np.ascontiguousarray(coords[i])), _p(np.ascontiguousarray(coords[j])),
                             g, g, _p(t9))
            m = -0.5 if state[j] else 0.5
            out[s] += t9.reshape(3, 3) @ np.array([0.0, 0.0, m])
    return out


def coherence_liouville(k, H0, H1, pulse_num, nT, dt, dephase_rate=0.0,
                        axis=(0.0, 0.0, 1.0), pol=(0.0, 0.0, 0.0)):
    H0 = np.asfortranarray(H0, np.complex128)
    H1 = np.asfortranarray(H1, np.complex128)
    ax = np.asarray(axis, np.float64)
    po = np.asarray(pol, np.float64)
    L = np.zeros(nT)
    lib().orc_coherence_liouville(k, _p(H0), _p(H1), pulse_num, nT, dt, dephase_rate,
                                  _p(ax), _p(po), _p(L))
    return L


class Enumeration:
    """Cluster sets per order, as cDepthFirstPathTracing builds them."""

    def __init__(self, coords, cutoff, max_order):
        L = lib()
        self.coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 3)
        self.max_order = int(max_order)
        self._h = L.orc_enumerate(self.coords.shape[0], _p(self.coords), float(cutoff),
                                  self.max_order)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_enum_free(self._h)
            self._h = None

    def count(self, order):
        return int(lib().orc_enum_count(self._h, order))

    def clusters(self, order):
        n = self.count(order)
        out = np.zeros((n, order + 1), np.uint64)
        buf = np.zeros(order + 1, np.uint64)
        for i in range(n):
            lib().orc_enum_cluster(self._h, order, i, _p(buf))
            out[i] = buf
        return out

    def parents(self, order, idx):
        buf = np.zeros(4096, np.uint64)
        n = lib().orc_enum_parents(self._h, order, idx, _p(buf), buf.size)
        return buf[:n].copy()

    def subclusters(self, order, idx):
        buf = np.zeros(2 * 65536, np.uint64)
        n = lib().orc_enum_subclusters(self._h, order, idx, _p(buf), 65536)
        return [tuple(int(x) for x in buf[2 * i:2 * i + 2]) for i in range(n)]

    def reduce(self, Lraw, nT):
        """Lraw: list per order of (nT x count) arrays."""
        raw = [np.asfortranarray(a, np.float64) for a in Lraw]
        til = [np.zeros_like(a, order="F") for a in raw]
        each = np.zeros((nT, self.max_order), order="F")
        cum = np.zeros((nT, self.max_order), order="F")
        rp = (C.c_void_p * self.max_order)(*[a.ctypes.data for a in raw])
        tp = (C.c_void_p * self.max_order)(*[a.ctypes.data for a in til])
        lib().orc_cce_reduce(self._h, self.max_order, nT, rp, tp, _p(each), _p(cum))
        return til, each, cum
