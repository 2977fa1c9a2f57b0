"""Host-side logic of the serving loop (no GPU): request generation follows
the serving config's distributions; footprints grow with the cluster count;
the scheduler (Server.run over a fake device) serves every request once,
keeps to its slots and HBM budget, runs a job larger than the budget alone,
and reports a failed job after the others have finished; the geometry
cache counts hits and misses and evicts the least recently used bath."""
import numpy as np

from oops_gb300 import serve


def test_request_stream_distributions():
    reqs = serve.make_requests(4096, rate=20.0, seed=5005)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    gaps = np.diff(arr)
    assert abs(gaps.mean() - 1 / 20.0) < 0.005
    rad = np.array([r.radius for r in reqs])
    ab = np.array([r.abundance for r in reqs])
    assert rad.min() >= 20 and rad.max() <= 40
    assert ab.min() >= 0.003 and ab.max() <= 0.05
    assert abs(np.log(ab).mean() - 0.5 * (np.log(0.003) + np.log(0.05))) < 0.05
    assert {r.order for r in reqs} == {2, 4, 6}
    assert {r.pulse_num for r in reqs} == {1, 2, 4, 8}
    nts = [r.nT for r in reqs]
    assert min(nts) >= 201 and max(nts) <= 501
    # same seed, same stream
    again = serve.make_requests(4096, rate=20.0, seed=5005)
    assert [r.seed for r in again] == [r.seed for r in reqs]


def test_footprint_and_cutoff_scaling():
    assert serve.footprint_bytes([10, 5], 201) < serve.footprint_bytes([10, 50], 201)
    r = serve.make_requests(1, 1.0, seed=1)[0]
    r.abundance = 0.011
    assert abs(r.cutoff - serve.BASE_CUTOFF[r.order]) < 1e-12
    r.abundance = 0.011 * 8
    assert abs(r.cutoff - serve.BASE_CUTOFF[r.order] / 2) < 1e-12


class _FakeCuda:
    @staticmethod
    def synchronize(device=None):
        pass


class _FakeTorch:
    cuda = _FakeCuda


class _FakeServer(serve.Server):
    """Server.run's scheduler over a fake device: each job "runs" by sleeping
    and records how many jobs and how many footprint bytes were in flight."""

    def __init__(self, slots, budget, counts_of, run_s=0.02, fail=()):
        self.torch = _FakeTorch
        self.device = 0
        self.slots = slots
        self.budget = budget
        self.streams = list(range(slots))
        self.counts_of = counts_of
        self.run_s = run_s
        self.fail = set(fail)
        self.lock = __import__("threading").Lock()
        self.active = self.in_use = 0
        self.max_active = 0
        self.overlaps = []          # (rid, bytes in flight when it started)
        self.big_alone = []

    def _prepare(self, r):
        return None, self.counts_of(r)

    def _run_job(self, r, geo, stream):
        import time
        need = serve.footprint_bytes(self.counts_of(r), r.nT)
        with self.lock:
            self.active += 1
            self.in_use += need
            self.max_active = max(self.max_active, self.active)
            self.overlaps.append((r.rid, self.in_use))
            if need > self.budget:
                self.big_alone.append(self.active == 1)
        time.sleep(self.run_s)
        with self.lock:
            self.active -= 1
            self.in_use -= need
        if r.rid in self.fail:
            raise ValueError("planted failure")
        return np.full((r.nT, r.order), float(r.rid))


def _requests(n, rate=400.0):
    reqs = serve.make_requests(n, rate=rate, seed=77)
    for r in reqs:
        r.nT = 201
    return reqs


def test_scheduler_keeps_slots_and_budget():
    """Every request is served once; no more jobs than slots run at a time,
    and the footprints in flight never exceed the budget."""
    counts_of = lambda r: [50 * (1 + r.rid % 3), 20]
    reqs = _requests(24)
    budget = 2 * serve.footprint_bytes([150, 20], 201)
    srv = _FakeServer(slots=3, budget=budget, counts_of=counts_of)
    res = srv.run(reqs, time_scale=1.0)
    assert sorted(r.rid for r in res) == list(range(24))
    assert srv.max_active <= 3
    assert all(b <= budget for _, b in srv.overlaps)
    assert [r.done for r in res] == sorted(r.done for r in res)
    for r in res:
        assert r.latency >= 0 and r.admitted >= r.arrival - 1e-6
        assert np.all(r.L == r.rid)


def test_scheduler_runs_a_job_larger_than_the_budget_alone():
    counts_of = lambda r: [5000, 5000] if r.rid == 3 else [10, 5]
    budget = serve.footprint_bytes([100, 50], 201)
    srv = _FakeServer(slots=4, budget=budget, counts_of=counts_of)
    res = srv.run(_requests(8), time_scale=1.0)
    assert len(res) == 8
    assert srv.big_alone == [True]


def test_scheduler_reports_a_failed_job_after_the_others_finish():
    import pytest
    srv = _FakeServer(slots=2, budget=1 << 40, counts_of=lambda r: [10, 5], fail=(5,))
    with pytest.raises(RuntimeError, match="request 5 failed"):
        srv.run(_requests(10), time_scale=1.0)
    assert srv.active == 0 and srv.in_use == 0


def test_geometry_cache_hits_and_evicts_least_recently_used(monkeypatch):
    """GeometryCache keeps baths keyed by seed and cluster parameters, counts
    hits and misses, and drops the least recently used beyond its budget
    (always keeping the newest)."""
    made = []

    class FakeBath:
        def __init__(self, coords, cutoff, order, device=None):
            self.device_bytes = 100
            made.append((len(coords), cutoff, order))

    monkeypatch.setattr(serve.cce, "DeviceBath", FakeBath)
    reqs = serve.make_requests(4, 1.0, seed=9)
    for r in reqs:
        r.radius = 15.0
    cache = serve.GeometryCache(budget=250)
    a, b, c = (cache.get(r) for r in reqs[:3])     # three misses; the first is evicted
    assert (cache.hits, cache.misses) == (0, 3)
    assert cache.bytes == 200 and len(cache.entries) == 2
    assert cache.get(reqs[2]) is c and cache.get(reqs[1]) is b
    assert cache.hits == 2
    assert cache.get(reqs[0]) is not a               # rebuilt after eviction
    assert cache.misses == 4
    assert serve.GeometryCache.key(reqs[2]) not in cache.entries   # least recently used went
    tiny = serve.GeometryCache(budget=10)
    tiny.get(reqs[3])
    assert len(tiny.entries) == 1                    # the newest entry stays even over budget
