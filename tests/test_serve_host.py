"""Host-side logic of the serving loop (no GPU): request generation follows
the serving config's distributions; footprints grow with the cluster count."""
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
