"""Serving loop: continuous batching over CUDA streams.  Each request's result
is the same alone and in the mix (the kernels are deterministic per request,
so the tolerance is tight), and admission respects slots and the HBM budget."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import cce, serve  # noqa: E402


def _small(n, seed):
    reqs = serve.make_requests(n, rate=1000.0, seed=seed, orders=(2, 4))
    for r in reqs:
        r.radius = min(r.radius, 25.0)
        r.nT = min(r.nT, 101)
    return reqs


@pytest.mark.parametrize("precision", [cce.PREC_FP64, cce.PREC_MIXED])
def test_result_alone_equals_result_in_the_mix(precision):
    reqs = _small(6, 77)
    mixed = serve.Server(slots=3, precision=precision).run(reqs, time_scale=0.0)
    assert len(mixed) == len(reqs)
    by_id = {r.rid: r for r in mixed}
    alone_srv = serve.Server(slots=1, precision=precision)
    for r in reqs:
        alone = alone_srv.run([r], time_scale=0.0)[0]
        assert np.abs(alone.L - by_id[r.rid].L).max() <= 1e-12
        assert alone.L.shape == (r.nT, r.order)


def test_admission_budget_serialises_large_jobs():
    reqs = _small(4, 78)
    res = serve.Server(slots=4, hbm_budget=1, precision=cce.PREC_MIXED).run(reqs, time_scale=0.0)
    # with a 1-byte budget every job runs alone: admissions never overlap
    spans = sorted((r.admitted, r.done) for r in res)
    for (a0, d0), (a1, d1) in zip(spans, spans[1:]):
        assert a1 >= d0 - 1e-3
    stats = serve.latency_stats(res)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0


def test_geometry_stays_resident_across_jobs():
    """A second job on a bath already served reuses its device-resident
    geometry (no enumeration, no upload) and gives the same curve."""
    reqs = _small(3, 79)
    srv = serve.Server(slots=2, precision=cce.PREC_MIXED)
    first = {r.rid: r.L for r in srv.run(reqs, time_scale=0.0)}
    assert srv.geometry.misses == 3 and srv.geometry.hits == 0
    again = {r.rid: r.L for r in srv.run(reqs, time_scale=0.0)}
    assert srv.geometry.hits == 3
    for rid in first:
        assert np.array_equal(first[rid], again[rid])
