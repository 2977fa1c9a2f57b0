"""The project's autotuner: launch shapes of the batched CCE kernels and the
Krylov dimension of the expv drop-in, measured on the device in use and kept
in an on-disk cache.

The reference fixes its launch geometry from the device limits
(src/expv/source/get_grid.cu:43-125) and its Krylov parameters in the
MatExpVector constructor (src/source/math/MatExp.cpp:98-100: m = 30,
tol = 1e-12).  Here:

* per cluster size k, the eigensolver's CTAs per SM, the block coherence
  kernels' CTAs per SM and the time-slice multiplier (oops_tune_set) are
  chosen by timing every candidate on the caller's clusters with CUDA events;
  a tuned value changes the launch shape only, never the results;
* the Krylov dimension m in {20, 30, 40} (bounded by the cluster dimension)
  is chosen by timing the first output step of a block propagation.

The cache is a JSON file ($OOPS_TUNE_CACHE, else
~/.cache/oops_gb300/tune.json) keyed by the device name and SM count and the
workload shape (cluster size, precision, pulse count, and the cluster count
and time-point count rounded to powers of two).  cce.cluster_coherence and
cce.DeviceRun consult it before they launch (apply()).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import time

PARAMS = {"eig_per_sm": 0, "coh_per_sm": 1, "tslice_mult": 2}
CANDIDATES = {"eig_per_sm": (1, 2, 4, 8), "coh_per_sm": (1, 2, 4, 8), "tslice_mult": (1, 2, 4, 8)}
KRYLOV_M = (20, 30, 40)

_cache = None
_cache_path = None


def cache_path():
    p = os.environ.get("OOPS_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "oops_gb300", "tune.json")


def _lib():
    from .cce import L_
    L = L_()
    if not getattr(L, "_tune_declared", False):
        L.oops_tune_set.restype = C.c_int
        L.oops_tune_set.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oops_tune_get.restype = C.c_int
        L.oops_tune_get.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int)]
        L._tune_declared = True
    return L


def set_param(name, k, value):
    from ._lib import check
    check(_lib().oops_tune_set(PARAMS[name], int(k), int(value)))
    try:
        _applied[(device_key(), name, int(k))] = int(value)
    except Exception:  # no device to key on: the next apply() sets it again
        pass


def get_param(name, k):
    from ._lib import check
    v = C.c_int()
    check(_lib().oops_tune_get(PARAMS[name], int(k), C.byref(v)))
    return v.value


def reset(k=None):
    for kk in ([k] if k else range(1, 7)):
        for name in PARAMS:
            set_param(name, kk, 0)


_dkeys = {}


def device_key(device=None):
    import torch
    idx = torch.cuda.current_device() if device is None else torch.device("cuda", device).index
    if idx not in _dkeys:
        p = torch.cuda.get_device_properties(idx)
        _dkeys[idx] = f"{p.name}|sm{p.multi_processor_count}"
    return _dkeys[idx]


def _bucket(n):
    return 1 << max(0, int(math.ceil(math.log2(max(1, int(n))))))


def shape_key(k, precision, pulse_num, ncl, nT):
    return f"k{int(k)}|p{int(precision)}|n{int(pulse_num)}|c{_bucket(ncl)}|t{_bucket(nT)}"


def load(path=None):
    """The cache as a dict (empty when the file does not exist)."""
    global _cache, _cache_path
    path = path or cache_path()
    if _cache is not None and _cache_path == path:
        return _cache
    _cache, _cache_path = _read(path), path
    return _cache


def save(cache, path=None):
    """Write the cache atomically: a private temporary file renamed over the
    cache, so a reader never sees a partial file and two writers never share
    the temporary."""
    path = path or cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    global _cache, _cache_path
    _cache, _cache_path = cache, path


def lookup(dkey, skey, cache=None):
    cache = load() if cache is None else cache
    return cache.get(dkey, {}).get(skey)


def _read(path):
    """The cache file's content; {} when it is missing or not a cache."""
    try:
        with open(path) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return {}
    if not isinstance(d, dict):
        return {}
    return {k: v for k, v in d.items() if isinstance(v, dict)}


def record(dkey, skey, values, cache=None, path=None):
    """Add one entry and save.  Without `cache` the entry is merged into the
    file as it is now on disk, so entries that other processes recorded since
    this one loaded the cache are kept."""
    path = path or cache_path()
    base = _read(path) if cache is None else cache
    cache = {d: dict(v) for d, v in base.items()}
    cache.setdefault(dkey, {})[skey] = values
    save(cache, path)
    return cache


_applied = {}


def apply(k, precision, pulse_num, ncl, nT, device=None):
    """Set the cached launch shape of this workload shape on the current
    device (the defaults when nothing is cached).  Returns the values.  The
    library is only called when a value changes."""
    dkey = device_key(device)
    vals = lookup(dkey, shape_key(k, precision, pulse_num, ncl, nT)) or {}
    for name in PARAMS:
        v = int(vals.get(name, 0))
        if _applied.get((dkey, name, k)) != v:
            set_param(name, k, v)
            _applied[(dkey, name, k)] = v
    return vals


def _time_call(fn, reps):
    import torch
    fn()  # warm-up (module load, first allocations)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ts.sort()
    return ts[len(ts) // 2]


def tune_class(coords_dev, clusters_dev, k, params, precision, reps=3, path=None):
    """Time every candidate of every launch parameter (one parameter at a
    time, the others at their best so far) for one batch of k-spin clusters
    and record the winners in the cache.  Returns (values, default_ms,
    tuned_ms)."""
    from . import cce
    ncl = int(clusters_dev.shape[0])
    nT = int(params.nT)
    out = None

    def run():
        nonlocal out
        out = cce.cluster_coherence(coords_dev, clusters_dev, k, params, precision, out=out,
                                    tuned=False)

    reset(k)
    default_ms = _time_call(run, reps)
    best = {}
    best_ms = default_ms
    for name in PARAMS:
        choice = 0
        for v in CANDIDATES[name]:
            set_param(name, k, v)
            ms = _time_call(run, reps)
            if ms < best_ms:
                best_ms, choice = ms, v
        set_param(name, k, choice)
        if choice:
            best[name] = choice
    best["ms"] = best_ms
    best["default_ms"] = default_ms
    record(device_key(), shape_key(k, precision, params.pulse_num, ncl, nT), best, path=path)
    return best, default_ms, best_ms


def krylov_key(N, nvec):
    return f"krylov|N{int(N)}|v{int(nvec)}"


def tune_krylov_m(ham, V, t_first, tol=1e-12, k=10, path=None):
    """Krylov dimension for a Hamiltonian of this size and this block width:
    the m in {20, 30, 40} (m < N) whose first output step is fastest; cached
    per device and (N, nvec)."""
    import torch
    from .expv import expv_block
    N, nvec = V.shape[0], (V.shape[1] if V.dim() > 1 else 1)
    cands = [m for m in KRYLOV_M if m < N] or [max(1, N - 1)]
    # untimed call at the largest m first: the handle's workspace grows to its
    # final size, so no candidate's time includes the allocation
    expv_block(ham, V, [t_first], m=max(cands), tol=tol, k=k)
    best = None
    for m in cands:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        expv_block(ham, V, [t_first], m=m, tol=tol, k=k)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if best is None or el < best[1]:
            best = (m, el)
    record(device_key(), krylov_key(N, nvec), {"m": best[0], "s": best[1]}, path=path)
    return best[0]


def krylov_m(N, nvec, default=30):
    """The cached Krylov dimension for (N, nvec) on this device, else the
    reference's default (bounded by N - 1)."""
    v = lookup(device_key(), krylov_key(N, nvec))
    m = int(v["m"]) if v else default
    return max(1, min(m, N - 1))
