"""Python front end of the batched CCE C-ABI (include/oops_cce.h).

Mirrors the reference's application layer: ``Clusters`` is cSpinCluster built
by cDepthFirstPathTracing (src/source/spin/SpinCluster/SpinClusterAlgorithm.cpp),
``nv_states`` is NVCenter::make_espin_hamiltonian (src/source/app/
DefectCenter.cpp:32-45), ``cluster_coherence`` is EnsembleCCE::cluster_evolution
for a whole batch of clusters (src/source/app/ensemble_cce.cpp:33-55) and
``ensemble_cce`` the full EnsembleCCE run with the CCE reduction
(src/source/app/cce.cpp:54-189).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib

GAMMA_C13 = 6.728284e7          # SpinData.cpp:4
GAMMA_NVE = -1.760859708e11     # SpinData.cpp:8
PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_SIMT = 2


class CCEParams(C.Structure):
    _fields_ = [("B", C.c_double * 3), ("center", C.c_double * 3), ("gamma_center", C.c_double),
                ("gamma_bath", C.c_double), ("sv0", C.c_double * 3), ("sv1", C.c_double * 3),
                ("pulse_num", C.c_int), ("nT", C.c_size_t), ("dt", C.c_double),
                ("fp64_below", C.c_double), ("fp64_max_k", C.c_int)]

    @classmethod
    def make(cls, B, sv0, sv1, pulse_num, nT, dt, center=(0.0, 0.0, 0.0),
             gamma_center=GAMMA_NVE, gamma_bath=GAMMA_C13, fp64_below=0.0, fp64_max_k=0):
        p = cls()
        p.B[:] = [float(x) for x in B]
        p.center[:] = [float(x) for x in center]
        p.gamma_center = gamma_center
        p.gamma_bath = gamma_bath
        p.sv0[:] = [float(x) for x in sv0]
        p.sv1[:] = [float(x) for x in sv1]
        p.pulse_num = int(pulse_num)
        p.nT = int(nT)
        p.dt = float(dt)
        p.fp64_below = float(fp64_below)
        p.fp64_max_k = int(fp64_max_k)
        return p


class CCEBath(C.Structure):
    """Bath terms of the Liouville-space path (oops_cce_bath): pure dephasing
    of every bath spin along an axis and the initial bath polarisation
    (EnsembleCCE::set_parameters, src/source/app/ensemble_cce.cpp:16-18).
    The defaults are the EnsNVeBath / EnsNVLattice application defaults
    (src/application/EnsNVeBath.cpp:133-135)."""
    _fields_ = [("dephasing_rate", C.c_double), ("dephasing_axis", C.c_double * 3),
                ("polarization", C.c_double * 3)]

    @classmethod
    def make(cls, dephasing_rate=1e4, dephasing_axis=(1.0, 1.0, 1.0),
             polarization=(0.0, 0.0, 0.0)):
        b = cls()
        b.dephasing_rate = float(dephasing_rate)
        b.dephasing_axis[:] = [float(x) for x in dephasing_axis]
        b.polarization[:] = [float(x) for x in polarization]
        return b


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _declare(L):
    vp = C.c_void_p
    if getattr(L, "_cce_declared", False):
        return
    L.oops_clusters_enumerate.restype = C.c_int
    L.oops_clusters_enumerate.argtypes = [C.c_size_t, vp, C.c_double, C.c_int, C.POINTER(vp)]
    L.oops_clusters_destroy.argtypes = [vp]
    L.oops_clusters_count.restype = C.c_size_t
    L.oops_clusters_count.argtypes = [vp, C.c_int]
    L.oops_clusters_indices.restype = C.c_int
    L.oops_clusters_indices.argtypes = [vp, C.c_int, vp]
    L.oops_clusters_subcluster_total.restype = C.c_size_t
    L.oops_clusters_subcluster_total.argtypes = [vp, C.c_int]
    L.oops_clusters_subclusters.restype = C.c_int
    L.oops_clusters_subclusters.argtypes = [vp, C.c_int, vp, vp]
    L.oops_nv_states.restype = C.c_int
    L.oops_nv_states.argtypes = [vp, vp, vp]
    L.oops_cce_coherence.restype = C.c_int
    L.oops_cce_coherence.argtypes = [vp, C.c_size_t, vp, C.c_size_t, C.c_int,
                                     C.POINTER(CCEParams), C.c_int, vp, vp]
    L.oops_ensemble_cce.restype = C.c_int
    L.oops_ensemble_cce.argtypes = [C.c_size_t, vp, C.c_double, C.c_int, C.POINTER(CCEParams),
                                    C.c_int, vp, vp, vp, vp, C.c_size_t, vp]
    L.oops_cce_coherence_liouville.restype = C.c_int
    L.oops_cce_coherence_liouville.argtypes = [vp, C.c_size_t, vp, C.c_size_t, C.c_int,
                                               C.POINTER(CCEParams), C.POINTER(CCEBath), vp, vp]
    L.oops_ensemble_cce_bath.restype = C.c_int
    L.oops_ensemble_cce_bath.argtypes = [C.c_size_t, vp, C.c_double, C.c_int, C.POINTER(CCEParams),
                                         C.POINTER(CCEBath), vp, vp, vp, vp, C.c_size_t, vp]
    L.oops_cce_reduce.restype = C.c_int
    L.oops_cce_reduce.argtypes = [C.c_int, vp, C.c_size_t, vp, vp, vp, vp, vp, vp, vp]
    L.oops_profile_enable.restype = C.c_int
    L.oops_profile_enable.argtypes = [C.c_int]
    L.oops_profile_read_eig.restype = C.c_int
    L.oops_profile_read_eig.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_long)]
    L.oops_profile_corrected.restype = C.c_int
    L.oops_profile_corrected.argtypes = [C.c_int, C.POINTER(C.c_long)]
    L.oops_cce_coherence_state.restype = C.c_int
    L.oops_cce_coherence_state.argtypes = [vp, C.c_size_t, vp, vp, C.c_size_t, C.c_int,
                                           C.POINTER(CCEParams), C.c_int, vp, vp]
    L.oops_bath_state_from_seed.restype = C.c_int
    L.oops_bath_state_from_seed.argtypes = [C.c_uint, C.c_size_t, vp]
    L.oops_single_sample_cce_device.restype = C.c_int
    L.oops_single_sample_cce_device.argtypes = [vp, C.c_size_t, vp, C.c_int, vp, vp,
                                                C.POINTER(CCEParams), C.c_int, vp, vp, vp, vp,
                                                vp, vp, vp]
    L.oops_single_sample_cce.restype = C.c_int
    L.oops_single_sample_cce.argtypes = [C.c_size_t, vp, vp, C.c_double, C.c_int,
                                         C.POINTER(CCEParams), C.c_int, vp, vp, vp, vp,
                                         C.c_size_t, vp]
    L.oops_cce_export_mat.restype = C.c_int
    L.oops_cce_export_mat.argtypes = [C.c_char_p, C.c_int, C.c_size_t, vp, vp, vp, vp, vp, vp]
    L.oops_cce_release_plans.restype = C.c_int
    L.oops_cce_release_plans.argtypes = []
    L.oops_profile_liouville.restype = C.c_int
    L.oops_profile_liouville.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double),
                                         C.POINTER(C.c_long), C.POINTER(C.c_double)]
    L.oops_liouville_launches.restype = C.c_long
    L.oops_liouville_launches.argtypes = []
    L.oops_profile_read.restype = C.c_int
    L.oops_profile_read.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_long),
                                    C.POINTER(C.c_double)]
    L._cce_declared = True


def L_():
    L = lib()
    _declare(L)
    return L


class Clusters:
    """Connected clusters of a bath up to max_order spins (order o: o+1 spins)."""

    def __init__(self, coords, cutoff, max_order):
        self.coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 3)
        self.max_order = int(max_order)
        h = C.c_void_p()
        check(L_().oops_clusters_enumerate(self.coords.shape[0], _p(self.coords), float(cutoff),
                                           self.max_order, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            L_().oops_clusters_destroy(self._h)
            self._h = None

    def count(self, order):
        return int(L_().oops_clusters_count(self._h, order))

    def clusters(self, order):
        n = self.count(order)
        out = np.zeros((n, order + 1), np.uint32)
        if n:
            check(L_().oops_clusters_indices(self._h, order, _p(out)))
        return out

    def subclusters(self, order):
        n = self.count(order)
        tot = int(L_().oops_clusters_subcluster_total(self._h, order))
        off = np.zeros(n + 1, np.uint64)
        pairs = np.zeros(max(1, 2 * tot), np.uint32)
        check(L_().oops_clusters_subclusters(self._h, order, _p(off), _p(pairs)))
        return off, pairs[:2 * tot].reshape(-1, 2)


def nv_states(B):
    B = np.ascontiguousarray(B, np.float64)
    ev = np.zeros(3)
    sv = np.zeros(9)
    check(L_().oops_nv_states(_p(B), _p(ev), _p(sv)))
    return ev, sv.reshape(3, 3)


def cluster_coherence(coords_dev, clusters_dev, k, params: CCEParams, precision=PREC_FP64,
                      out=None, stream=None, tuned=True):
    """L_C(t) for a batch of k-spin clusters.  coords_dev: torch float64 CUDA
    (nbath, 3); clusters_dev: torch int32 CUDA (ncl, k).  Returns torch
    float64 CUDA (ncl, nT).  tuned: use the autotuner's cached launch shape
    for this workload shape (oops_gb300.tune), else leave the current one."""
    import torch
    ncl = clusters_dev.shape[0]
    if tuned:
        from . import tune
        tune.apply(k, precision, params.pulse_num, ncl, params.nT)
    if out is None:
        out = torch.empty((ncl, int(params.nT)), dtype=torch.float64, device=coords_dev.device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(L_().oops_cce_coherence(C.c_void_p(coords_dev.data_ptr()), coords_dev.shape[0],
                                  C.c_void_p(clusters_dev.data_ptr()), ncl, int(k),
                                  C.byref(params), int(precision), C.c_void_p(out.data_ptr()),
                                  C.c_void_p(st)))
    return out


def cluster_coherence_liouville(coords_dev, clusters_dev, k, params: CCEParams, bath: CCEBath,
                                out=None, stream=None):
    """L_C(t) of a batch of k-spin clusters (k <= 6) in Liouville space with
    bath dephasing and polarisation (EnsembleCCE::cluster_evolution as the
    reference runs it, src/source/app/ensemble_cce.cpp:33-113), FP64.
    Arguments as cluster_coherence."""
    import torch
    ncl = clusters_dev.shape[0]
    if out is None:
        out = torch.empty((ncl, int(params.nT)), dtype=torch.float64, device=coords_dev.device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(L_().oops_cce_coherence_liouville(
        C.c_void_p(coords_dev.data_ptr()), coords_dev.shape[0], C.c_void_p(clusters_dev.data_ptr()),
        ncl, int(k), C.byref(params), C.byref(bath), C.c_void_p(out.data_ptr()), C.c_void_p(st)))
    return out


def bath_state_from_seed(seed, nbath):
    """The bath product state SingleSampleCCE::prepare_bath_state draws
    (src/source/app/single_sample_cce.cpp:35-46): srand(seed), rand() % 2 per
    spin (0: up, 1: down along z), with glibc's rand() restated."""
    out = np.zeros(int(nbath), np.uint8)
    check(L_().oops_bath_state_from_seed(int(seed) & 0xffffffff, out.size, _p(out)))
    return out


def cluster_coherence_state(coords_dev, state_dev, clusters_dev, k, params: CCEParams,
                            precision=PREC_FP64, out=None, stream=None):
    """Single-sample L_C(t) of a batch of k-spin clusters (SingleSampleCCE::
    cluster_evolution, src/source/app/single_sample_cce.cpp:48-127).
    state_dev: torch uint8 CUDA (nbath,); other arguments as cluster_coherence."""
    import torch
    ncl = clusters_dev.shape[0]
    if out is None:
        out = torch.empty((ncl, int(params.nT)), dtype=torch.float64, device=coords_dev.device)
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(L_().oops_cce_coherence_state(
        C.c_void_p(coords_dev.data_ptr()), coords_dev.shape[0], C.c_void_p(state_dev.data_ptr()),
        C.c_void_p(clusters_dev.data_ptr()), ncl, int(k), C.byref(params), int(precision),
        C.c_void_p(out.data_ptr()), C.c_void_p(st)))
    return out


def single_sample_cce(coords, state, cutoff, max_order, params: CCEParams, precision=PREC_FP64,
                      want_clusters=False, stream=None):
    """Whole single-sample CCE run (SingleSampleCCE + the CCE reduction) with
    host buffers.  Returns as ensemble_cce."""
    coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 3)
    state = np.ascontiguousarray(state, np.uint8)
    if state.size != coords.shape[0]:
        raise ValueError("one state byte per bath spin")
    nT = int(params.nT)
    cum = np.zeros((max_order, nT))
    each = np.zeros((max_order, nT))
    counts = np.zeros(max_order, np.uint64)
    cl_buf, cl_len = None, 0
    if want_clusters:
        cl = Clusters(coords, cutoff, max_order)
        cl_buf = np.zeros(max(1, sum(cl.count(o) for o in range(max_order)) * nT))
        cl_len = cl_buf.size
    st = C.c_void_p(stream) if stream is not None else None
    check(L_().oops_single_sample_cce(coords.shape[0], _p(coords), _p(state), float(cutoff),
                                      int(max_order), C.byref(params), int(precision), _p(cum),
                                      _p(each), _p(counts),
                                      _p(cl_buf) if cl_buf is not None else None, cl_len, st))
    res = (cum.T.copy(), each.T.copy(), counts.astype(np.int64))
    if want_clusters:
        per, off = [], 0
        for o in range(max_order):
            n = int(counts[o])
            per.append(cl_buf[off:off + n * nT].reshape(n, nT).copy())
            off += n * nT
        res = res + (per,)
    return res


def ensemble_cce(coords, cutoff, max_order, params: CCEParams, precision=PREC_FP64,
                 want_clusters=False, stream=None, bath: CCEBath | None = None):
    """Whole EnsembleCCE run through the C-ABI with host buffers.  With a
    ``bath`` (CCEBath) the clusters run in Liouville space with dephasing and
    polarisation (oops_ensemble_cce_bath: FP64, max_order <= 6).
    Returns (final_cum (nT, max_order), final_each, counts[, cluster_L list])."""
    coords = np.ascontiguousarray(coords, np.float64).reshape(-1, 3)
    nT = int(params.nT)
    cum = np.zeros((max_order, nT))
    each = np.zeros((max_order, nT))
    counts = np.zeros(max_order, np.uint64)
    cl_buf = None
    cl_len = 0
    if want_clusters:
        cl = Clusters(coords, cutoff, max_order)
        tot = sum(cl.count(o) for o in range(max_order))
        cl_buf = np.zeros(max(1, tot * nT))
        cl_len = cl_buf.size
    st = C.c_void_p(stream) if stream is not None else None
    if bath is None:
        check(L_().oops_ensemble_cce(coords.shape[0], _p(coords), float(cutoff), int(max_order),
                                     C.byref(params), int(precision), _p(cum), _p(each), _p(counts),
                                     _p(cl_buf) if cl_buf is not None else None, cl_len, st))
    else:
        check(L_().oops_ensemble_cce_bath(coords.shape[0], _p(coords), float(cutoff),
                                          int(max_order), C.byref(params), C.byref(bath), _p(cum),
                                          _p(each), _p(counts),
                                          _p(cl_buf) if cl_buf is not None else None, cl_len, st))
    res = (cum.T.copy(), each.T.copy(), counts.astype(np.int64))
    if want_clusters:
        per, off = [], 0
        for o in range(max_order):
            n = int(counts[o])
            per.append(cl_buf[off:off + n * nT].reshape(n, nT).copy())
            off += n * nT
        res = res + (per,)
    return res


class DeviceBath:
    """A bath's geometry resident on the device: coordinates, every order's
    cluster index lists and closures (the part of a run that depends only on
    the bath, the cutoff and the order; a serving process keeps these across
    jobs).  limit: keep at most this many clusters per order (a profiling
    case)."""

    def __init__(self, coords, cutoff, max_order, device="cuda", limit=0):
        import torch
        self.max_order = int(max_order)
        cl = Clusters(coords, cutoff, max_order)
        self.counts = [cl.count(o) for o in range(self.max_order)]
        if limit:
            # keep only the first `limit` clusters of every order (closures of
            # the kept clusters point to lower orders, which are kept in full
            # only as far as they fall under the limit: a profiling case)
            self.counts = [min(c, limit) for c in self.counts]
        self.coords = torch.from_numpy(np.ascontiguousarray(coords, np.float64)).to(device)
        self.idx, self.off, self.pairs = [], [], []
        self.h2d_bytes = self.coords.numel() * 8
        for o in range(self.max_order):
            rows = cl.clusters(o).astype(np.int32)[:self.counts[o]]
            off, pairs = cl.subclusters(o)
            if limit:
                keep_off, keep_pairs = [0], []
                for j in range(self.counts[o]):
                    for a, b in pairs[int(off[j]):int(off[j + 1])]:
                        if b < self.counts[a]:
                            keep_pairs.append((a, b))
                    keep_off.append(len(keep_pairs))
                off = np.asarray(keep_off, np.uint64)
                pairs = np.asarray(keep_pairs, np.uint32).reshape(-1, 2)
            self.idx.append(torch.from_numpy(rows).to(device))
            self.off.append(torch.from_numpy(off.astype(np.int64)).to(device))
            self.pairs.append(torch.from_numpy(pairs.astype(np.int32).reshape(-1).copy()
                                               if pairs.size else np.zeros(2, np.int32)).to(device))
            self.h2d_bytes += rows.nbytes + off.nbytes + pairs.nbytes

    @property
    def device_bytes(self):
        return int(self.coords.numel() * 8 + sum(t.numel() * t.element_size()
                                                 for t in self.idx + self.off + self.pairs))


class DeviceRun:
    """A CCE run with bath, cluster lists and closures resident on the device
    (the serving / bench form): step() computes every cluster's coherence and
    the reduction without host traffic.  geometry: an existing DeviceBath of
    the same bath, cutoff and order to run on (nothing is enumerated or
    uploaded again)."""

    def __init__(self, coords, cutoff, max_order, params: CCEParams, precision=PREC_FP64,
                 device="cuda", limit=0, bath: CCEBath | None = None, state=None, geometry=None):
        import torch
        self.torch = torch
        self.params = params
        self.precision = precision
        self.bath = bath
        self.state = None if state is None else torch.from_numpy(
            np.ascontiguousarray(state, np.uint8)).to(device)
        self.max_order = int(max_order)
        self.nT = int(params.nT)
        geo = geometry if geometry is not None else DeviceBath(coords, cutoff, max_order, device, limit)
        if geo.max_order != self.max_order:
            raise ValueError("geometry was built for another CCE order")
        self.geometry = geo
        self.counts = list(geo.counts)
        self.coords, self.idx, self.off, self.pairs = geo.coords, geo.idx, geo.off, geo.pairs
        self.h2d_bytes = geo.h2d_bytes
        dev = self.coords.device
        self.L, self.til = [], []
        for o in range(self.max_order):
            self.L.append(torch.empty((max(1, self.counts[o]), self.nT), dtype=torch.float64,
                                      device=dev))
            self.til.append(torch.empty_like(self.L[-1]))
        self.each = torch.empty((self.max_order, self.nT), dtype=torch.float64, device=dev)
        self.cum = torch.empty_like(self.each)

    @property
    def n_clusters(self):
        return int(sum(self.counts))

    def apply_tuning(self):
        """The autotuner's cached launch shapes for this run's size classes."""
        from . import tune
        for o, n in enumerate(self.counts):
            if n:
                tune.apply(o + 1, self.precision, self.params.pulse_num, n, self.nT)

    def step(self, stream=None):
        """One whole run (every cluster's coherence + the reduction) through
        oops_ensemble_cce_device: the size classes run concurrently on streams
        forked from `stream`, one host synchronisation at the end."""
        torch = self.torch
        self.apply_tuning()
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        n = self.max_order
        ptr = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])
        counts = (C.c_size_t * n)(*self.counts)
        if self.state is not None:
            # single-sample run (oops_single_sample_cce_device): concurrent
            # size classes, one synchronisation
            check(L_().oops_single_sample_cce_device(
                C.c_void_p(self.coords.data_ptr()), C.c_size_t(self.coords.shape[0]),
                C.c_void_p(self.state.data_ptr()), n, counts, ptr(self.idx), C.byref(self.params),
                int(self.precision), ptr(self.L), ptr(self.til), ptr(self.off), ptr(self.pairs),
                C.c_void_p(self.each.data_ptr()), C.c_void_p(self.cum.data_ptr()), C.c_void_p(st)))
            return self.cum
        if self.bath is not None:
            # Liouville path: the classes one after another (each waits for
            # its exponentials' scaling exponents), then the reduction
            for o in reversed(range(n)):
                if self.counts[o]:
                    cluster_coherence_liouville(self.coords, self.idx[o][:self.counts[o]], o + 1,
                                                self.params, self.bath, out=self.L[o], stream=st)
            check(L_().oops_cce_reduce(n, counts, self.nT, ptr(self.L), ptr(self.til), ptr(self.off),
                                       ptr(self.pairs), C.c_void_p(self.each.data_ptr()),
                                       C.c_void_p(self.cum.data_ptr()), C.c_void_p(st)))
            return self.cum
        check(L_().oops_ensemble_cce_device(
            C.c_void_p(self.coords.data_ptr()), C.c_size_t(self.coords.shape[0]), n, counts, ptr(self.idx),
            C.byref(self.params), int(self.precision), ptr(self.L), ptr(self.til), ptr(self.off),
            ptr(self.pairs), C.c_void_p(self.each.data_ptr()), C.c_void_p(self.cum.data_ptr()),
            C.c_void_p(st)))
        return self.cum

    def reduce_curves(self, Ls, stream=None):
        """The CCE reduction (oops_cce_reduce) of the given raw cluster curves
        (one torch float64 CUDA tensor per order, counts[o] x nT) with this
        run's closures; returns a copy of the cumulative curves (max_order x
        nT).  Overwrites this run's raw and reduced curve buffers."""
        torch = self.torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        n = self.max_order
        for o in range(n):
            if self.counts[o]:
                self.L[o][:self.counts[o]].copy_(Ls[o][:self.counts[o]])
        ptr = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])
        counts = (C.c_size_t * n)(*self.counts)
        check(L_().oops_cce_reduce(n, counts, self.nT, ptr(self.L), ptr(self.til), ptr(self.off),
                                   ptr(self.pairs), C.c_void_p(self.each.data_ptr()),
                                   C.c_void_p(self.cum.data_ptr()), C.c_void_p(st)))
        return self.cum.clone()

    def make_graph(self):
        """Capture the run into a CUDA graph (oops_cce_graph_create); step_graph()
        replays it.  The run's device buffers stay owned by this object."""
        self.close_graph()
        self.apply_tuning()
        n = self.max_order
        ptr = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])
        counts = (C.c_size_t * n)(*self.counts)
        g = C.c_void_p()
        check(L_().oops_cce_graph_create(
            C.c_void_p(self.coords.data_ptr()), C.c_size_t(self.coords.shape[0]), n, counts,
            ptr(self.idx), C.byref(self.params), int(self.precision), ptr(self.L), ptr(self.til),
            ptr(self.off), ptr(self.pairs), C.c_void_p(self.each.data_ptr()),
            C.c_void_p(self.cum.data_ptr()), C.byref(g)))
        self._graph = g
        return self

    def step_graph(self, stream=None):
        """One whole run as one graph launch (make_graph first)."""
        if getattr(self, "_graph", None) is None:
            raise RuntimeError("make_graph() first")
        st = stream if stream is not None else self.torch.cuda.current_stream().cuda_stream
        check(L_().oops_cce_graph_launch(self._graph, C.c_void_p(st)))
        return self.cum

    def close_graph(self):
        g = getattr(self, "_graph", None)
        if g is not None:
            L_().oops_cce_graph_destroy(g)
            self._graph = None

    def __del__(self):
        try:
            self.close_graph()
        except Exception:
            pass

    def launches_per_step(self):
        """Kernels of this library per step: per non-empty size class the
        assembly/eigensolver, overlap and coherence kernels (and the phase
        steps in the mixed modes); per order the tilde and the two product
        kernels; one initialisation."""
        nz = sum(1 for c in self.counts if c)
        per_class = 3 if self.precision == PREC_FP64 else 4
        return per_class * nz + 1 + 3 * self.max_order


def profile_enable(on=True):
    check(L_().oops_profile_enable(1 if on else 0))


def profile_corrected(k):
    n = C.c_long()
    check(L_().oops_profile_corrected(int(k), C.byref(n)))
    return n.value


def profile_read(k):
    ms, n, fl = C.c_double(), C.c_long(), C.c_double()
    check(L_().oops_profile_read(int(k), C.byref(ms), C.byref(n), C.byref(fl)))
    return ms.value, n.value, fl.value


def profile_read_eig(k):
    """(ms, launches) of the eigensolver phase of clusters of k spins since
    profile_enable."""
    ms, n = C.c_double(), C.c_long()
    check(L_().oops_profile_read_eig(int(k), C.byref(ms), C.byref(n)))
    return ms.value, n.value


def profile_liouville(k, phase):
    """(ms, launches, FP64 flop) of one phase of the Liouville path for
    clusters of k spins since profile_enable: 0 exponentials and powers,
    1 outer recurrences, 2 middle passes."""
    ms, n, fl = C.c_double(), C.c_long(), C.c_double()
    check(L_().oops_profile_liouville(int(k), int(phase), C.byref(ms), C.byref(n), C.byref(fl)))
    return ms.value, n.value, fl.value


def liouville_launches():
    """Kernels launched by the Liouville path since profile_enable."""
    return int(L_().oops_liouville_launches())


def export_mat(path, time_list, final_cum, final_each, cluster_L=None, cluster_til=None):
    """Write a run's results as the MAT-file CCE::export_mat_file writes
    (src/source/app/cce.cpp:191-234) through oops_cce_export_mat.
    final_cum / final_each: (nT, max_order); cluster_L / cluster_til: one
    (n_clusters, nT) array per order (cluster-major, as ensemble_cce returns
    them), or None."""
    t = np.ascontiguousarray(time_list, np.float64)
    nT = t.size
    cum = np.asfortranarray(final_cum, np.float64)
    each = np.asfortranarray(final_each, np.float64)
    K = cum.shape[1]
    if cum.shape != (nT, K) or each.shape != (nT, K):
        raise ValueError("final curves must be (nT, max_order)")

    def per_order(arrs):
        if arrs is None:
            return None, []
        keep = [np.ascontiguousarray(a, np.float64).reshape(-1, nT) for a in arrs]
        return (C.c_void_p * K)(*[a.ctypes.data if a.size else None for a in keep]), keep

    src = cluster_L if cluster_L is not None else cluster_til
    counts = (C.c_size_t * K)(*([np.asarray(a).reshape(-1, nT).shape[0] for a in src]
                                if src is not None else [0] * K))
    pl, keep_l = per_order(cluster_L)
    pt, keep_t = per_order(cluster_til)
    check(L_().oops_cce_export_mat(str(path).encode(), K, nT, counts, pl, pt, _p(each), _p(cum), _p(t)))


def release_plans():
    """Free the calling thread's ensemble_cce run plan (oops_cce_release_plans)."""
    check(L_().oops_cce_release_plans())
