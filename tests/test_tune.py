"""The autotuner (oops_gb300/tune.py, oops_tune_* in include/oops_cce.h).

CPU: the on-disk cache (keys, shape buckets, round trip, per-device entries,
merging with other writers, unreadable files) and the C-ABI's argument
checks.  GPU: tuning a class of clusters records launch shapes that give
bit-identical results and are no slower than the defaults when timed again,
and the product entry points consult the cache.
"""
import json

import numpy as np
import pytest

from oops_gb300 import tune


def test_shape_key_buckets_counts_and_time_points():
    assert tune.shape_key(4, 1, 8, 143, 401) == "k4|p1|n8|c256|t512"
    assert tune.shape_key(4, 1, 8, 129, 257) == tune.shape_key(4, 1, 8, 256, 512)
    assert tune.shape_key(4, 1, 8, 128, 256) != tune.shape_key(4, 1, 8, 129, 256)
    assert tune.shape_key(6, 0, 1, 1, 1) == "k6|p0|n1|c1|t1"


def test_cache_round_trip_and_device_separation(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    assert tune.load(path) == {}
    tune.record("GB300|sm152", "k4|p1|n1|c256|t512", {"eig_per_sm": 4, "ms": 1.0}, path=path)
    tune.record("GB300|sm152", "k5|p1|n1|c256|t512", {"tslice_mult": 2, "ms": 2.0}, path=path)
    tune.record("OTHER|sm100", "k4|p1|n1|c256|t512", {"eig_per_sm": 1, "ms": 3.0}, path=path)
    with open(path) as f:
        on_disk = json.load(f)
    assert on_disk["GB300|sm152"]["k4|p1|n1|c256|t512"]["eig_per_sm"] == 4
    tune._cache = None  # force a re-read
    c = tune.load(path)
    assert tune.lookup("GB300|sm152", "k5|p1|n1|c256|t512", c)["tslice_mult"] == 2
    assert tune.lookup("OTHER|sm100", "k4|p1|n1|c256|t512", c)["eig_per_sm"] == 1
    assert tune.lookup("GB300|sm152", "k6|p1|n1|c256|t512", c) is None


def test_record_keeps_entries_other_processes_wrote(tmp_path):
    """A tuner that loaded the cache earlier does not drop what another
    process recorded since: record() merges into the file on disk."""
    path = str(tmp_path / "tune.json")
    tune._cache = None
    tune.record("GB300|sm152", "k4|p1|n1|c256|t512", {"eig_per_sm": 4}, path=path)
    assert tune.load(path)["GB300|sm152"]
    other = {"GB300|sm152": {"k6|p1|n8|c65536|t512": {"coh_per_sm": 2}}}   # another process's save
    with open(path, "w") as f:
        json.dump(other, f)
    tune.record("GB300|sm152", "k5|p1|n1|c256|t512", {"tslice_mult": 2}, path=path)
    with open(path) as f:
        on_disk = json.load(f)
    assert set(on_disk["GB300|sm152"]) == {"k6|p1|n8|c65536|t512", "k5|p1|n1|c256|t512"}
    assert not any(p.name.endswith(".tmp") for p in tmp_path.iterdir())


@pytest.mark.parametrize("content", ["", "{not json", "[1, 2]", '{"GB300|sm152": 3}'])
def test_unreadable_cache_reads_as_empty(tmp_path, content):
    path = str(tmp_path / "tune.json")
    with open(path, "w") as f:
        f.write(content)
    tune._cache = None
    assert tune.load(path) == {}
    c = tune.record("GB300|sm152", "k4|p1|n1|c256|t512", {"eig_per_sm": 1}, path=path)
    assert c == {"GB300|sm152": {"k4|p1|n1|c256|t512": {"eig_per_sm": 1}}}
    tune._cache = None


def test_tune_set_checks_its_arguments():
    L = tune._lib()
    assert L.oops_tune_set(3, 4, 1) == -1      # no such parameter
    assert L.oops_tune_set(0, 7, 1) == -1      # cluster size out of range
    assert L.oops_tune_set(0, 4, 65) == -1     # value out of range


@pytest.mark.gpu
def test_tuned_launch_shape_is_exact_and_no_slower(tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    from oops_gb300 import cce, configs
    monkeypatch.setenv("OOPS_TUNE_CACHE", str(tmp_path / "tune.json"))
    tune._cache = None
    w = configs.cce4_hahn()
    cl = cce.Clusters(w.coords, w.cutoff, 5)
    _, sv = cce.nv_states(w.B)
    coords = torch.from_numpy(w.coords).cuda()
    idx = torch.from_numpy(cl.clusters(4).astype(np.int32)).cuda()   # 128 five-spin clusters
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 2, 101, 4e-5)
    tune.reset()
    ref = cce.cluster_coherence(coords, idx, 5, p, cce.PREC_MIXED, tuned=False).clone()
    vals, d_ms, t_ms = tune.tune_class(coords, idx, 5, p, cce.PREC_MIXED, reps=3)
    assert t_ms <= d_ms
    # the entry point consults the cache: same launch shape, same results
    got = cce.cluster_coherence(coords, idx, 5, p, cce.PREC_MIXED)
    for name in tune.PARAMS:
        if name in vals:
            assert tune.get_param(name, 5) == vals[name]
    assert torch.equal(got, ref)
    # timed again, interleaved: the tuned shape is no slower than the default
    def timed(use_tuned):
        if use_tuned:
            tune.apply(5, cce.PREC_MIXED, 2, idx.shape[0], 101)
        else:
            tune.reset(5)
        return tune._time_call(lambda: cce.cluster_coherence(coords, idx, 5, p, cce.PREC_MIXED,
                                                             out=got, tuned=False), 3)
    dd, tt = [], []
    for _ in range(3):
        dd.append(timed(False))
        tt.append(timed(True))
    assert np.median(tt) <= 1.05 * np.median(dd)
    tune.reset()
