"""oops_cce_coherence_noalloc: the cluster-coherence entry point for callers
that cannot allocate device memory during a run (their allocator reserved the
device memory up front, or their serving loop must not let cudaMalloc/cudaFree
synchronise the device).  It draws its scratch from a static 32 MiB device
array in the library.

Called through the C-ABI and checked against oops_cce_coherence, which
allocates its own scratch, on two calls in a row (the array keeps the previous
call's contents, so the second call checks that nothing stale leaks through),
with the tolerances the other parity tests use.  Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import OopsError, cce, configs  # noqa: E402
from oops_gb300._lib import check  # noqa: E402


def _noalloc(coords, clusters, k, params, precision, out):
    L = cce.L_()
    fn = L.oops_cce_coherence_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int,
                   C.POINTER(cce.CCEParams), C.c_int, C.c_void_p, C.c_void_p]
    st = torch.cuda.current_stream().cuda_stream
    return fn(C.c_void_p(coords.data_ptr()), coords.shape[0], C.c_void_p(clusters.data_ptr()),
              clusters.shape[0], k, C.byref(params), precision, C.c_void_p(out.data_ptr()),
              C.c_void_p(st))


def _bath():
    w = configs.cce4_hahn()
    cl = cce.Clusters(w.coords, w.cutoff, 5)
    _, sv = cce.nv_states(w.B)
    return w, cl, sv, torch.from_numpy(w.coords).cuda()


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("precision,tol", [(cce.PREC_FP64, 1e-10), (cce.PREC_MIXED, 1e-6),
                                           (cce.PREC_MIXED_SIMT, 1e-6)])
def test_noalloc_matches_allocating_entry_point_twice(k, precision, tol):
    """Two calls in a row (different batches) against oops_cce_coherence; the
    static array keeps the first call's contents, so the second call checks
    that nothing stale leaks through.  For k <= 4 this path runs the block
    kernels, which the allocating entry point does not use at those sizes."""
    w, cl, sv, coords = _bath()
    rows_all = cl.clusters(k - 1)
    batches = [rows_all[:61], rows_all[-37:]]
    for rows in batches:
        p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, 101, 4e-5)
        idx = torch.from_numpy(rows.astype(np.int32)).cuda()
        ref = cce.cluster_coherence(coords, idx, k, p, precision).cpu().numpy()
        out = torch.full((rows.shape[0], 101), np.nan, dtype=torch.float64, device="cuda")
        check(_noalloc(coords, idx, k, p, precision, out))
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= tol


def test_noalloc_honours_fp64_max_k_and_rejects_fp64_below():
    w, cl, sv, coords = _bath()
    rows = cl.clusters(2)[:40]
    idx = torch.from_numpy(rows.astype(np.int32)).cuda()
    # fp64_max_k = 3: the three-spin clusters of a mixed call run in FP64
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, 101, 4e-5, fp64_max_k=3)
    ref = cce.cluster_coherence(coords, idx, 3, p, cce.PREC_FP64).cpu().numpy()
    out = torch.full((rows.shape[0], 101), np.nan, dtype=torch.float64, device="cuda")
    check(_noalloc(coords, idx, 3, p, cce.PREC_MIXED, out))
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-10
    # fp64_below > 0 in a mixed mode: a status, not a silent mixed result
    p2 = cce.CCEParams.make(w.B, sv[0], sv[1], 1, 101, 4e-5, fp64_below=0.5)
    out.fill_(np.nan)
    for prec in (cce.PREC_MIXED, cce.PREC_MIXED_SIMT):
        assert _noalloc(coords, idx, 3, p2, prec, out) == -4
    assert torch.isnan(out).all()
    # ... and ignored in FP64, where it has nothing to recompute
    check(_noalloc(coords, idx, 3, p2, cce.PREC_FP64, out))
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-10


def test_noalloc_rejects_batches_beyond_the_static_scratch():
    w = configs.cce6_cpmg8()
    cl = cce.Clusters(w.coords, w.cutoff, 6)
    _, sv = cce.nv_states(w.B)
    coords = torch.from_numpy(w.coords).cuda()
    rows = cl.clusters(5)[:1000]   # 1000 six-spin clusters need ~190 MiB of scratch
    idx = torch.from_numpy(rows.astype(np.int32)).cuda()
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 8, 11, 1e-4)
    out = torch.empty((rows.shape[0], 11), dtype=torch.float64, device="cuda")
    rc = _noalloc(coords, idx, 6, p, cce.PREC_MIXED, out)
    assert rc == -3
    with pytest.raises(OopsError):
        check(rc)
    # a batch that fits still runs after the rejection
    small = idx[:20].contiguous()
    out2 = torch.empty((20, 11), dtype=torch.float64, device="cuda")
    check(_noalloc(coords, small, 6, p, cce.PREC_MIXED, out2))
    # the static-scratch path runs six-spin clusters on CUDA cores: compare with
    # the allocating entry point's CUDA-core mode
    ref = cce.cluster_coherence(coords, small, 6, p, cce.PREC_MIXED_SIMT).cpu().numpy()
    assert np.abs(out2.cpu().numpy() - ref).max() <= 1e-6
