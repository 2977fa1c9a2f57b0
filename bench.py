#!/usr/bin/env python3
"""Benchmark of the GB300 CCE hot path.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--workload cce2|cce4|cce6] [--precision fp64|mixed]

A step is one whole ensemble-CCE pass over the workload: every enumerated
cluster's coherence curve L_C(t) (one "cluster-propagation" each) plus the CCE
reduction, with the bath, cluster lists and closures resident in HBM.  The
headline value is cluster-propagations/s; e2e repeats the metric through the
reference-facing C-ABI call (oops_ensemble_cce) with host buffers: enumeration,
host->device copies, compute and device->host copies inside the timed region.

--impl reference times the reference's own CPU algorithm for the same
workload: the reference's application does not build as shipped (Fortran
Pade and Krylov drivers, MKL, armadillo, MPI) and its sources do not travel
with this repository, so its dense Pade + power propagation
(PiecewiseFullMatrixVectorEvolution + MatExp::pade_exp_mat, restated in the
C oracle) runs on bounded samples of the workload's clusters on all host
cores: untimed warm-up steps, then --steps timed steps of a fixed number of
clusters each.  The oracle is used only on that leg and for cpu_baseline.

Multi-GPU: clusters are independent but the reduction needs every
sub-cluster, and each box has one GPU, so N>1 runs N independent replicas
(one per rank); value = all ranks' cluster-propagations / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cluster-propagations/s vs plain FP64 GPU at max|ΔL|≤1e-6; serve p50/p99 ms"
UNIT = "cluster-propagations/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cce6",
                    choices=["cce2", "cce4", "cce6", "c4", "serve", "dephasing", "single"])
    ap.add_argument("--serve-requests", type=int, default=1024)
    ap.add_argument("--serve-rate", type=float, default=0.5, help="Poisson arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=1e9,
                    help="arrival-time cap of the mixed-precision run; later arrivals are dropped")
    ap.add_argument("--serve-fp64", type=int, default=8,
                    help="requests (of at most four spins per cluster) in the FP64 comparison")
    ap.add_argument("--c4-points", type=int, default=3,
                    help="c4: output times of the 100-point grid integrated in the timed run")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--plain-seconds", type=float, default=20.0)
    # profiling helpers: shrink the workload to a small case of the same kernels
    ap.add_argument("--limit-clusters", type=int, default=0,
                    help="keep at most this many clusters per order (profiling)")
    ap.add_argument("--nt", type=int, default=0, help="override the time-point count (profiling)")
    ap.add_argument("--accuracy", default="on", choices=["on", "off"],
                    help="off: skip the FP64 comparison run (profiling)")
    ap.add_argument("--graph", default="on", choices=["on", "off"],
                    help="replay the device-resident run as one CUDA graph in the timed region")
    ap.add_argument("--fp64-below", type=float, default=0.0,
                    help="mixed precision: recompute clusters whose L_C drops below this in FP64")
    ap.add_argument("--fp64-max-k", type=int, default=0,
                    help="mixed precision: clusters of up to this many spins run in FP64")
    return ap.parse_args()


def kernel_name(k, prec, pulse_num):
    """The coherence kernel that runs clusters of k spins at this precision."""
    from oops_gb300 import cce
    T = "double" if prec == cce.PREC_FP64 else "float"
    if k >= 5 and prec == cce.PREC_MIXED and (pulse_num == 1 or pulse_num % 2 == 0):
        return f"k_coherence_tc{1 << k} (tcgen05)"
    if k <= 4:
        return f"k_coherence_warp<{k},{T}>"
    return f"k_coherence<{k},{T}>"


# ncu sm__pipe_fp64_cycles_active of k_assemble_eig<k> on the CCE-6 case
# with 1216 clusters per size class (profiles/assemble_eig6_cce6_small.md)
EIG_FP64_PIPE_NCU = {6: 0.467, 5: 0.638, 4: 0.705, 3: 0.640}

# ncu dram__bytes_read.sum + dram__bytes_write.sum of the tensor-core
# coherence kernels on 1216 clusters x 51 time points, per cluster
# (profiles/coherence_tc_cce6_1216.md): k_coherence_tc64 42,477,312 B,
# k_coherence_tc32 11,307,264 B
COHERENCE_DRAM_BYTES_PER_CLUSTER_NCU = {6: 42477312 / 1216, 5: 11307264 / 1216}

# FMA-chain probe on a GB300 of this pool (152 SMs, 1987 MHz): CUDA-core rates
FP32_SIMT_PEAK = 69.85
FP64_PEAK = 1.19


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    except Exception:
        return 1900.0, 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


_T0 = time.perf_counter()


def progress(msg):
    """One line on stderr per phase (the JSON line goes to stdout)."""
    sys.stderr.write(f"[bench {time.perf_counter() - _T0:8.1f} s] {msg}\n")
    sys.stderr.flush()


def max_over_ranks(x, dist, device):
    """The largest x over all ranks (the job's time is its slowest rank's);
    x itself on a single process."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        import torch
        if args.impl == "ours":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:  # the reference arm runs on the host cores only
            dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def workload(name, nt=0):
    from oops_gb300 import configs
    w = configs.WORKLOADS[name]()
    if nt:
        w.name += f"_nT{nt}"
        w.nT = nt
    return w


def systematic_orders(n, offset, counts):
    """Cluster orders of an n-cluster sample that follow `counts` (clusters
    per order): the orders at the points (i + offset) / n, i < n, of the
    cumulative distribution.  With offset (s + 0.5) / S for the S steps s,
    each step and the union of all steps are within one cluster per order of
    the proportional counts."""
    cdf = np.cumsum(np.asarray(counts, float) / np.sum(counts))
    u = (np.arange(n) + offset) / n
    return np.minimum(np.searchsorted(cdf, u, side="right"), len(cdf) - 1)


def cpu_steps(w, cl, one, steps, warmup, seconds_per_step, what, threads=None):
    """Times the per-cluster CPU work `one(order, index)` of the workload's
    clusters (enumeration `cl`) on all host cores: `warmup` untimed steps of
    one cluster per thread (at least one: it sizes the timed steps), then
    `steps` timed steps.  A step is a batch of clusters whose orders follow
    the workload's order counts (systematic_orders: every step, and all
    steps together, within one cluster per order of the proportional counts)
    and whose members are drawn at random, largest clusters first; its size
    is the warm-up's rate times `seconds_per_step`, at least two clusters per
    thread.  The timed steps are queued back to back on the threads, so no
    thread idles at a step boundary; a step's time runs from the previous
    step's last completion to its own.  Returns (clusters/s over the timed
    steps, mean ms per timed step, cores, sample text ending in `what`)."""
    import concurrent.futures as cf
    counts = np.array([cl.count(o) for o in range(w.max_order)], float)
    cores = threads or os.cpu_count() or 1
    rng = np.random.default_rng(7919)

    def timed_one(item):
        one(*item)
        return time.perf_counter()

    def draw(n, offset):
        items = [(int(o), int(rng.integers(cl.count(int(o)))))
                 for o in systematic_orders(n, offset, counts)]
        return sorted(items, key=lambda it: -it[0])

    def run(batches):
        t0 = time.perf_counter()
        futs = [[ex.submit(timed_one, it) for it in b] for b in batches]
        ends, last = [], t0
        for fs in futs:
            last = max([last] + [f.result() for f in fs])
            ends.append(last)
        return np.diff([t0] + ends)

    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        nw = max(1, warmup)
        warm_s = float(run([draw(cores, rng.random()) for _ in range(nw)]).sum())
        n_step = max(2 * cores, int(np.ceil(nw * cores / warm_s * seconds_per_step)))
        batches = [draw(n_step, (i + 0.5) / steps) for i in range(steps)]
        times = run(batches)
    per_order = np.bincount([o for b in batches for o, _ in b], minlength=w.max_order)
    rate = steps * n_step / float(times.sum())
    text = (f"{steps} timed steps of {n_step} clusters (per order in total {per_order.tolist()}, "
            f"in proportion to the workload's {int(counts.sum())} clusters), "
            f"{float(times.sum()):.1f} s, after {nw} untimed warm-up steps of {cores} clusters; "
            f"{cores} threads; {what}")
    return rate, 1e3 * float(np.mean(times)), cores, text


def cpu_reference_steps(w, steps, warmup, seconds_per_step, threads=None):
    """The reference's dense algorithm (oracle restatement: Pade exponentials
    of the two conditional Hamiltonians and one product per segment and time
    step) on the workload's clusters by cpu_steps, with the oracle's
    enumeration and NV states (nothing of the GPU library is loaded): the
    reference arm's steps and the GPU arm's cpu_baseline.  Returns
    (clusters/s, mean ms per timed step, cores, sample text)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.lib()
    cl = po.Enumeration(w.coords, w.cutoff, w.max_order)
    _, sv = po.nv_states(w.B)
    rows = {o: cl.clusters(o) for o in range(w.max_order)}

    def one(o, j):
        c = w.coords[[int(x) for x in rows[o][j]]]
        H = [po.dense_hamiltonian(po.cluster_hamiltonian(c, w.B, np.zeros(3), sv[s]))
             for s in (0, 1)]
        po.coherence_hilbert(H[0], H[1], w.pulse_num, w.nT, w.dt)

    return cpu_steps(w, cl, one, steps, warmup, seconds_per_step,
                     "oracle restatement of the reference's dense Pade + power propagation",
                     threads)


def bench_config(w, counts, ws):
    """The workload description both arms print (identical dictionaries)."""
    return {"workload": w.name, "clusters_per_order": [int(c) for c in counts], "nT": int(w.nT),
            "t_max_s": float(w.t_max), "pulse_num": int(w.pulse_num),
            "max_order": int(w.max_order), "cutoff_A": float(w.cutoff),
            "B_T": [float(x) for x in w.B],
            "l2": "GPU arm: flushed between timed steps (512 MiB write)",
            "parallelism": f"replicas x{ws}"}


# FP64 curves of the first clusters of each order kept for the plain Krylov
# sample's comparison
HEAD_ROWS = 256


def accuracy_check(w, params, prec, run, dev):
    """This run's curves against the FP64 path (itself within 1e-10 of the
    oracle per cluster in the tests) over the whole workload: every cluster's
    L_C(t) at every time point, and the whole-run L(t) of every order.

    The whole-run figures come with the conditioning of the CCE reduction on
    this workload: the FP64 reduction is re-run on the FP64 cluster curves
    perturbed by a relative 1e-14 (FP64 rounding scale) and 1e-11, and the
    change it makes to L(t) is reported per order.  Where sub-cluster curves
    pass near zero the reduction L~_C = L_C / prod L~_sub amplifies any
    perturbation without bound (the expansion diverges: |L(t)| > 1), and no
    finite-precision evaluation can match another there; the whole-run error
    is therefore also reported over the well-conditioned points (|L(t)| <= 1
    and a 1e-11 perturbation moving L(t) by at most 1e-9)."""
    import torch
    from oops_gb300 import cce
    out = {"reference": "FP64 path, every cluster and every time point of the workload"}
    if prec == cce.PREC_FP64:
        out["note"] = "run is FP64"
        return out, [run.L[o][:HEAD_ROWS].cpu().numpy() for o in range(w.max_order)]
    f64 = cce.DeviceRun(w.coords, w.cutoff, w.max_order, params, cce.PREC_FP64, device=dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    f64.step()
    torch.cuda.synchronize(dev)
    out["fp64_run_s"] = time.perf_counter() - t0
    per, above, pts, p9999 = [], [], 0, []
    for o in range(w.max_order):
        n = run.counts[o]
        if not n:
            per.append(0.0)
            above.append(0)
            p9999.append(0.0)
            continue
        dd = (run.L[o][:n] - f64.L[o][:n]).abs()
        per.append(float(dd.max().item()))
        above.append(int((dd > 1e-6).sum().item()))
        p9999.append(float(torch.quantile(dd.flatten()[::max(1, dd.numel() // 4000000)], 0.9999).item()))
        pts += dd.numel()
    out["max_abs_dL_cluster"] = max(per)
    out["max_abs_dL_cluster_per_order"] = per
    out["cluster_points_above_1e-6_per_order"] = above
    out["cluster_points"] = pts
    out["abs_dL_cluster_p99.99_per_order"] = p9999
    base = f64.cum.clone()
    dcum = (run.cum - base).abs()
    out["max_abs_dL_whole_run"] = float(dcum.max().item())
    out["max_abs_dL_whole_run_per_order"] = [float(x) for x in dcum.max(dim=1).values.cpu()]
    out["fp64_whole_run_min_max_per_order"] = [
        [float(a), float(b)] for a, b in zip(base.min(dim=1).values.cpu(), base.max(dim=1).values.cpu())]
    Lf = [x.clone() for x in f64.L]
    sens = {}
    for eps in (1e-14, 1e-11):
        c = f64.reduce_curves([x - eps * (1.0 - x) for x in Lf])
        sens[eps] = (c - base).abs()
    out["fp64_sensitivity_per_order"] = {
        f"{eps:g}": [float(x) for x in v.max(dim=1).values.cpu()] for eps, v in sens.items()}
    mask = (sens[1e-11] <= 1e-9) & (base.abs() <= 1.0)
    out["well_conditioned_points_per_order"] = [int(x) for x in mask.sum(dim=1).cpu()]
    out["max_abs_dL_well_conditioned_per_order"] = [
        float(x) for x in torch.where(mask, dcum, torch.zeros_like(dcum)).max(dim=1).values.cpu()]
    head = [f64.L[o][:HEAD_ROWS].cpu().numpy() for o in range(w.max_order)]
    del f64, Lf, sens
    return out, head


def plain_krylov_sample(w, sv, seconds, batched_rate, counts, rows, L_fp64=None):
    """Cluster-propagations/s of the plain FP64 Krylov path (krylov_cce: the
    one-step propagator of every distinct segment from the main_cache_
    algorithm applied to the basis states, then FP64 powers and chain
    products, one per time step as the reference's dense propagation), per
    size class.  Clusters of each size run whole, on the full time grid,
    in the workload's order, until the class's share of the budget is spent
    (at least one); the class rate is the mean over the clusters run, and
    the workload rate weights each class by its cluster count.  With
    L_fp64 (per order, the FP64 batched path's curves) the sampled curves
    are compared with it."""
    from oops_gb300.krylov_cce import cluster_coherence_krylov
    # clusters of one or two spins are left out (their time counted as zero,
    # which flatters the Krylov path): the drop-in needs m < N (zgexpv_cache.f:
    # 376-377), and with m <= 3 its step size is bounded by ~tol^(1/m)/||H||,
    # so one pulse interval of a spin pair takes ~1e6 steps at tol = 1e-12
    import torch
    # the batched complex products' library initialisation, outside the sample
    z = torch.eye(4, dtype=torch.complex128, device="cuda").expand(2, 4, 4).contiguous()
    torch.bmm(z, z)
    torch.cuda.synchronize()
    skipped = [o for o in range(w.max_order) if counts[o] > 0 and o + 1 <= 2]
    classes = [o for o in range(w.max_order) if counts[o] > 0 and o + 1 > 2]
    budget = seconds / max(1, len(classes))
    per_class, total_s, max_d = [], 0.0, 0.0
    for o in classes:
        progress(f"  Krylov class k={o + 1}")
        t_start = time.perf_counter()
        times, kry, prod, steps = [], 0.0, 0.0, 0
        for j in range(int(counts[o])):
            r = rows[o][j]
            tm = {}
            t0 = time.perf_counter()
            L = cluster_coherence_krylov(w.coords[np.asarray(r, int)], w.B, sv, w.pulse_num, w.nT, w.dt,
                                         timings=tm)
            times.append(time.perf_counter() - t0)
            kry += tm["krylov_s"]
            prod += tm["products_s"]
            steps += tm["krylov_steps"]
            if L_fp64 is not None and j < len(L_fp64[o]):
                max_d = max(max_d, float(np.abs(L - L_fp64[o][j]).max()))
            if time.perf_counter() - t_start > budget:
                break
        per_cluster = float(np.mean(times))
        total_s += counts[o] * per_cluster
        n = len(times)
        per_class.append({"k": o + 1, "clusters": int(counts[o]), "clusters_run": n,
                          "per_cluster_s": per_cluster, "krylov_s_per_cluster": kry / n,
                          "products_s_per_cluster": prod / n, "krylov_steps_per_cluster": steps / n})
    n = sum(int(counts[o]) for o in classes + skipped)
    if not classes:
        return {"value": None, "unit": UNIT,
                "note": "every cluster has one or two spins: the drop-in needs m < 2^k, and with "
                        "m <= 3 one pulse interval takes ~1e6 Krylov steps, so the plain path is "
                        "not sampled on this workload",
                "classes_counted_as_free": [{"k": o + 1, "clusters": int(counts[o])} for o in skipped]}
    rate = n / total_s
    out = {"value": rate, "unit": UNIT, "speedup_of_batched": batched_rate / rate,
           "per_class": per_class,
           "classes_counted_as_free": [{"k": o + 1, "clusters": int(counts[o])} for o in skipped],
           "sample": f"whole clusters on the full {w.nT}-point grid, the first of each size class "
                     f"until its share of a {seconds:.0f} s budget is spent, weighted by the class "
                     f"counts; FP64 throughout (m = autotuned or 30, tol = 1e-12)"}
    if L_fp64 is not None:
        out["max_abs_dL_vs_fp64_batched"] = max_d
    return out


def run_c4(args, ws, rank, local):
    """Large-cluster Krylov stress (auxiliary line, not the headline): clusters of
    14, 15 and 16 spins, 64 random normalised complex128 vectors, Krylov
    dimension m autotuned over {20, 30, 40} at tol 1e-10, outputs every 20 us.
    Reports the Kronecker matvec's throughput (CUDA events around
    oops_ham_apply on the 64-vector block) and the block propagation rate."""
    import torch
    from oops_gb300 import build as b
    b.build()
    from oops_gb300 import cce, configs
    from oops_gb300.expv import Hamiltonian, expv_block
    from oops_gb300.spin import cluster_terms
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    bf16, hbm, src = peaks()
    res = []
    for k in (14, 15, 16):
        coords, B = configs.krylov_stress_cluster(k)
        _, sv = cce.nv_states(B)
        t = cluster_terms(coords, B, np.zeros(3), sv[1])
        H = Hamiltonian(t)
        N = H.dim
        nvec = 64
        rng = np.random.default_rng(4000 + k)
        V = rng.normal(size=(N, nvec)) + 1j * rng.normal(size=(N, nvec))
        V /= np.linalg.norm(V, axis=0)
        Vd = torch.from_numpy(V).to(dev).contiguous()
        Y = torch.empty_like(Vd)
        for _ in range(3):
            H.apply(Vd, -1j, out=Y)
        torch.cuda.synchronize(dev)
        reps = 20
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            H.apply(Vd, -1j, out=Y)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        P = k * (k - 1) // 2 + k
        fused_bytes = 32.0 * N * nvec
        per_op_bytes = 48.0 * N * nvec * P
        cmacs = (1 + k + k * (k - 1) // 2) * N * nvec
        # autotune m on the first output time, then time a prefix of the grid
        tgrid = 20e-6 * np.arange(1, 101)
        best = None
        for m in (20, 30, 40):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            expv_block(H, Vd, tgrid[:1], m=m, tol=1e-10)
            torch.cuda.synchronize(dev)
            el = time.perf_counter() - t0
            if best is None or el < best[1]:
                best = (m, el)
        npts = max(1, min(100, args.c4_points))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        W, st = expv_block(H, Vd, tgrid[:npts], m=best[0], tol=1e-10)
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        nrm = float(W[-1].abs().pow(2).sum(dim=0).sqrt().sub(1).abs().max().item())
        res.append({"k": k, "N": N, "nvec": nvec, "terms": int(t.nterm), "operators": P,
                    "matvec_ms": ms, "matvec_fused_GBps": fused_bytes / (ms / 1e3) / 1e9,
                    "matvec_fused_frac_of_hbm": fused_bytes / (ms / 1e3) / 1e9 / hbm,
                    "matvec_per_operator_equiv_GBps": per_op_bytes / (ms / 1e3) / 1e9,
                    "matvec_fp64_TFLOPs": 8.0 * cmacs / (ms / 1e3) / 1e12,
                    "m_autotuned": best[0], "m_trial_s": best[1], "points": npts,
                    "integrated_s": float(tgrid[npts - 1]), "propagation_s": el,
                    "krylov_steps_col0": int(st.nstep), "matvecs_col0": int(st.nmult),
                    "anorm": st.anorm, "norm_drift_max": nrm})
        H.close()
    if rank == 0:
        cpu = cpu_sample_matvec(args.cpu_seconds) if args.cpu_seconds > 0 else None
        print(json.dumps({"metric": "Kronecker-matvec GB/s (large-cluster Krylov stress)",
                          "unit": "GB/s", "hbm_peak_GBps": hbm, "peak_source": src,
                          "fp64_peak_TFLOPs_probe": 1.19, "clusters": res,
                          "cpu_baseline": cpu}), flush=True)


def cpu_sample_matvec(seconds, k=14, threads=None):
    """The reference's CPU matvec (hamvec_func3: per term a copy, the body
    matrices applied as strided mode products, an axpy), restated in the
    oracle and pinned bit for bit to the reference's own compiled code, on
    the 14-spin stress cluster: one vector per host core, repeated for about
    `seconds`.  Reported in the GPU line's per-operator model (48 B N per
    one- or two-spin operator) and per vector."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import concurrent.futures as cf
    import pyoracle as po
    from oops_gb300 import configs
    coords, B = configs.krylov_stress_cluster(k)
    _, sv = po.nv_states(B)
    t = po.cluster_hamiltonian(coords, B, np.zeros(3), sv[1])
    N = t.dim
    cores = threads or os.cpu_count() or 1
    rng = np.random.default_rng(14)
    vecs = [rng.normal(size=N) + 1j * rng.normal(size=N) for _ in range(cores)]
    po.hamvec(t, vecs[0])  # library load and first-touch outside the sample
    done, t0 = 0, time.perf_counter()
    with cf.ThreadPoolExecutor(cores) as ex:
        while True:
            list(ex.map(lambda v: po.hamvec(t, v), vecs))
            done += cores
            el = time.perf_counter() - t0
            if el > seconds:
                break
    P = k * (k - 1) // 2 + k
    return {"value": 48.0 * N * P * done / el / 1e9, "unit": "GB/s (per-operator model)",
            "cores": cores, "kind": "port",
            "vector_matvecs_per_s": done / el,
            "sample": f"{done} single-vector matvecs of the k = {k} stress cluster (N = {N}, "
                      f"{t.nterm} terms) in {el:.1f} s on {cores} threads; oracle restatement "
                      f"of the reference's hamvec_func3 (bit-exact to it)"}


def run_serve(args, ws, rank, local):
    """Serving config (auxiliary line): the first --serve-requests requests of
    the seeded 4096-request stream, Poisson arrivals at --serve-rate per second
    in real time, continuous batching over 4 stream slots with admission by
    device-memory footprint and bath geometry resident across jobs; p50/p99
    latency and curves/s in mixed precision over the whole prefix, and the
    same for FP64 over the first --serve-fp64 requests of at most four spins
    per cluster (an FP64 six-spin job takes minutes)."""
    import torch
    from oops_gb300 import build as b
    b.build()
    from oops_gb300 import cce, serve
    torch.cuda.set_device(local)
    all_reqs = serve.make_requests(4096, rate=args.serve_rate, seed=5005)
    reqs = all_reqs[:args.serve_requests]
    res = {}
    for name, prec in (("mixed", cce.PREC_MIXED), ("fp64", cce.PREC_FP64)):
        if prec == cce.PREC_FP64:
            cut = [r for r in reqs if r.order <= 4][:args.serve_fp64]
            t_first = cut[0].arrival if cut else 0.0
            for r in cut:   # keep their spacing, starting at once
                r.arrival -= t_first
        else:
            cut = [r for r in reqs if r.arrival <= args.serve_seconds]
        if not cut:
            continue
        srv = serve.Server(slots=4, hbm_budget=200 << 30, precision=prec, device=local)
        t0 = time.perf_counter()
        out = srv.run(cut, time_scale=1.0)
        st = serve.latency_stats(out)
        st["wall_s"] = time.perf_counter() - t0
        st["requests_offered"] = len(cut)
        st["orders"] = {str(o): sum(1 for r in cut if r.order == o) for o in (2, 4, 6)}
        st["geometry_cache"] = {"hits": srv.geometry.hits, "misses": srv.geometry.misses,
                                "resident_bytes": srv.geometry.bytes}
        res[name] = st
    if rank == 0:
        print(json.dumps({"metric": "serve p50/p99 ms (coherence requests)", "unit": "ms",
                          "rate_per_s": args.serve_rate, "stream": "4096 seeded requests",
                          "prefix": args.serve_requests, "cap_s": args.serve_seconds,
                          "slots": 4, "results": res}), flush=True)


DEPHASING_HZ, DEPHASING_AXIS = 1e4, (1.0, 1.0, 1.0)   # EnsNVeBath / EnsNVLattice defaults


def dephasing_workload():
    """The CCE-4 Hahn bath with the reference application's default bath
    dephasing (1e4 Hz along (1,1,1), src/application/EnsNVeBath.cpp:133-135),
    zero polarisation: the Liouville-space path."""
    w = workload("cce4")
    w.name += "_dephasing1e4Hz_111"
    return w


def cpu_sample_liouville(w, seconds, threads=None):
    """The reference's Liouville algorithm (oracle restatement: dense 4^k
    superoperators, Pade exponentials, one power product per segment and time
    step) on the workload's clusters, per order on all host cores.  Orders of
    up to three spins run at the workload's nT for a bounded time; four-spin
    clusters cost ~1e11 flop each at nT = 401 in the oracle, so one batch
    (one cluster per core) runs at nT = 21 and at nT = 41 and its time at the
    workload's nT is extrapolated linearly (the cost is two exponentials plus
    a fixed cost per time step).  Returns (clusters/s over the whole workload,
    cores, sample text)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import concurrent.futures as cf
    import pyoracle as po
    po.lib()
    cl = po.Enumeration(w.coords, w.cutoff, w.max_order)
    _, sv = po.nv_states(w.B)
    cores = threads or os.cpu_count() or 1
    rng = np.random.default_rng(0)

    def one(idx, nT):
        c = w.coords[[int(x) for x in idx]]
        H = [po.dense_hamiltonian(po.cluster_hamiltonian(c, w.B, np.zeros(3), sv[s])) for s in (0, 1)]
        po.coherence_liouville(len(idx), H[0], H[1], w.pulse_num, nT, w.dt,
                               dephase_rate=2 * np.pi * DEPHASING_HZ, axis=DEPHASING_AXIS)
        return 1

    def batch(rows, nT):
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=cores) as ex:
            list(ex.map(lambda r: one(r, nT), rows))
        return time.perf_counter() - t0

    total_s, notes = 0.0, []
    for o in range(w.max_order):
        rows = cl.clusters(o)
        n = len(rows)
        if n == 0:
            continue
        if o + 1 <= 3:
            done, el, t0 = 0, 0.0, time.perf_counter()
            while el < seconds / w.max_order and done < n:
                pick = rows[rng.integers(n, size=cores)]
                el += batch(pick, w.nT)
                done += len(pick)
            rate = done / el
            notes.append(f"k={o + 1}: {done} clusters at nT={w.nT} in {el:.1f} s")
        else:
            pick = rows[rng.integers(n, size=cores)]
            e21, e41 = batch(pick, 21), batch(pick, 41)
            est = e21 + (e41 - e21) * (w.nT - 21) / 20.0
            rate = len(pick) / est
            notes.append(f"k={o + 1}: {len(pick)} clusters at nT=21 ({e21:.1f} s) and 41 "
                         f"({e41:.1f} s), {est:.1f} s extrapolated to nT={w.nT}")
        total_s += n / rate
    ntot = sum(cl.count(o) for o in range(w.max_order))
    text = ("; ".join(notes) + f"; {cores} threads; oracle restatement of the reference's "
            "Liouville propagation (dense Pade + one power product per segment and step)")
    return ntot / total_s, cores, text


def run_dephasing(args, ws, rank, local, dist):
    """Liouville-space ensemble CCE with bath dephasing (auxiliary line): the
    reference's default EnsembleCCE formulation.  Device-resident steps
    (every cluster through oops_cce_coherence_liouville, then the reduction)
    and the same run end to end through oops_ensemble_cce_bath."""
    import torch
    from oops_gb300 import build as b
    b.build()
    from oops_gb300 import cce
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = dephasing_workload()
    _, sv = cce.nv_states(w.B)
    params = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, w.nT, w.dt)
    bath = cce.CCEBath.make(DEPHASING_HZ, DEPHASING_AXIS)
    run = cce.DeviceRun(w.coords, w.cutoff, w.max_order, params, cce.PREC_FP64, device=dev,
                        bath=bath)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        run.step()
    torch.cuda.synchronize(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    cce.profile_enable(True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            flush.fill_(float(s))
            evs[s][0].record(stream)
            run.step()
            evs[s][1].record(stream)
        torch.cuda.synchronize(dev)
    if dist is not None:
        dist.barrier()
    ms = [a.elapsed_time(b_) for a, b_ in evs]
    launches = cce.liouville_launches() + 3 * w.max_order * args.steps
    phases = {(k, ph): cce.profile_liouville(k, ph) for k in range(1, w.max_order + 1)
              for ph in range(3)}
    cce.profile_enable(False)
    tot_ms = max_over_ranks(sum(ms), dist, dev)
    value = ws * run.n_clusters * args.steps / (tot_ms / 1e3)
    (kd, phd), (pms, pn, pfl) = max(phases.items(), key=lambda kv: kv[1][0])
    names = {0: "k_lv_gemm (exponentials: Taylor products, squarings)", 1: "k_lv_recur",
             2: "k_lv_pass (middle segments)"}
    achieved = pfl / (pms / 1e3) / 1e12 if pms > 0 else None
    roof = {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK, "unit": "TFLOP/s",
            "frac": achieved / FP64_PEAK if achieved else None, "traffic": None,
            "kernel": f"{names[phd]}, k={kd}", "peak_source": "measured FP64 FMA-chain probe",
            "phase_ms_per_step": pms / args.steps, "phase_launches_per_step": pn / args.steps,
            "phase_flop_per_step": pfl / args.steps,
            "flop_model": "8 N^3 per complex N x N product, 8 N^2 per matvec column, N = 4^k",
            "phases": {f"k{k}_p{ph}": {"ms": v[0] / args.steps, "launches": v[1] / args.steps,
                                         "TFLOPs": (v[2] / (v[0] / 1e3) / 1e12) if v[0] > 0 else None}
                       for (k, ph), v in phases.items() if v[1]},
            "timing": "CUDA events around each phase inside the timed region"}
    e2e_ms = []
    for s in range(max(2, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        cum = cce.ensemble_cce(w.coords, w.cutoff, w.max_order, params, stream=stream.cuda_stream,
                               bath=bath)[0]
        torch.cuda.synchronize(dev)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = ws * run.n_clusters / (np.mean(e2e_ms) / 1e3)
    agree = float(np.abs(run.cum.cpu().numpy().T - cum).max())
    h2d = run.h2d_bytes
    d2h = 2 * w.max_order * w.nT * 8 + w.max_order * 8
    if rank != 0:
        return
    cpu = None
    if args.cpu_seconds > 0:
        rate, cores, text = cpu_sample_liouville(w, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": text}
    line = {"metric": "cluster-propagations/s (Liouville space, bath dephasing)", "value": value,
            "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(w, run.counts, ws),
            "run": {"precision": "fp64", "dephasing_rate_hz": DEPHASING_HZ,
                    "dephasing_axis": DEPHASING_AXIS, "polarization": [0.0, 0.0, 0.0]},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": float(np.mean(e2e_ms)),
                    "max_abs_diff_vs_device_run": agree},
            "clocks": clk.summary(), "gpu_launches": launches}
    print(json.dumps(line), flush=True)


BATH_STATE_SEED = 2011


def cpu_steps_single(w, state, steps, warmup, seconds_per_step, threads=None):
    """The reference's single-sample algorithm (oracle restatement: bath
    mean field, dense Pade propagators and one power product per segment and
    step applied to the cluster's basis state) on the workload's clusters by
    cpu_steps.  Returns (clusters/s, mean ms per timed step, cores, sample
    text)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.lib()
    cl = po.Enumeration(w.coords, w.cutoff, w.max_order)
    _, sv = po.nv_states(w.B)
    rows = {o: cl.clusters(o) for o in range(w.max_order)}
    SXm = 0.5 * np.array([[0, 1], [1, 0]], complex)
    SYm = 0.5 * np.array([[0, -1j], [1j, 0]], complex)
    SZm = 0.5 * np.diag([1.0, -1.0]).astype(complex)

    def one(o, j):
        idx = [int(x) for x in rows[o][j]]
        k = len(idx)
        f = po.bath_field(w.coords, state, idx)
        Hs = []
        for s in (0, 1):
            H = po.dense_hamiltonian(po.cluster_hamiltonian(w.coords[idx], w.B, np.zeros(3), sv[s]))
            for q in range(k):
                for a, S in enumerate((SXm, SYm, SZm)):
                    H = H + f[q, a] * np.kron(np.kron(np.eye(2 ** q), S), np.eye(2 ** (k - 1 - q)))
            Hs.append(H)
        b = sum(int(state[i]) << (k - 1 - q) for q, i in enumerate(idx))
        po.coherence_state(Hs[0], Hs[1], w.pulse_num, w.nT, w.dt, b)

    return cpu_steps(w, cl, one, steps, warmup, seconds_per_step,
                     "oracle restatement of the reference's single-sample propagation", threads)


def run_single(args, ws, rank, local, dist):
    """Single-sample CCE (auxiliary line): the CCE-4 Hahn bath in the pure
    product state srand(2011); rand() % 2 draws (SingleSampleCCE), mixed
    precision.  Device-resident steps (every cluster through
    oops_cce_coherence_state, then the reduction) and the same run end to end
    through oops_single_sample_cce; accuracy against the FP64 run."""
    import torch
    from oops_gb300 import build as b
    b.build()
    from oops_gb300 import cce
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = single_workload()
    prec_name = args.precision or "mixed"
    prec = cce.PREC_MIXED if prec_name == "mixed" else cce.PREC_FP64
    state = cce.bath_state_from_seed(BATH_STATE_SEED, len(w.coords))
    _, sv = cce.nv_states(w.B)
    params = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, w.nT, w.dt)
    run = cce.DeviceRun(w.coords, w.cutoff, w.max_order, params, prec, device=dev, state=state)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        run.step()
    torch.cuda.synchronize(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for s_ in range(args.steps):
            flush.fill_(float(s_))
            evs[s_][0].record(stream)
            run.step()
            evs[s_][1].record(stream)
        torch.cuda.synchronize(dev)
    ms = [a.elapsed_time(b_) for a, b_ in evs]
    tot_ms = max_over_ranks(sum(ms), dist, dev)
    value = ws * run.n_clusters * args.steps / (tot_ms / 1e3)
    dev_cum = run.cum.cpu().numpy().T
    e2e_ms = []
    for _ in range(max(2, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        cum = cce.single_sample_cce(w.coords, state, w.cutoff, w.max_order, params, prec,
                                    stream=stream.cuda_stream)[0]
        torch.cuda.synchronize(dev)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    ref = cce.single_sample_cce(w.coords, state, w.cutoff, w.max_order, params, cce.PREC_FP64)[0]
    if rank != 0:
        return
    cpu = None
    if args.cpu_seconds > 0:
        rate, _, cores, text = cpu_steps_single(w, state, 3, 1, args.cpu_seconds / 3.0)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": text}
    line = {"metric": "cluster-propagations/s (single-sample CCE)", "value": value, "unit": UNIT,
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == cce.PREC_FP64 else "f32 (f64 eigenbasis)",
            "data": "synthetic",
            "config": bench_config(w, run.counts, ws),
            "run": {"precision": prec_name, "bath_state_seed": BATH_STATE_SEED},
            "e2e": {"value": ws * run.n_clusters / (np.mean(e2e_ms) / 1e3), "unit": UNIT,
                    "h2d_bytes_per_step": int(run.h2d_bytes + len(state)),
                    "d2h_bytes_per_step": int(2 * w.max_order * w.nT * 8 + w.max_order * 8),
                    "ms_per_step": float(np.mean(e2e_ms)),
                    "max_abs_diff_vs_device_run": float(np.abs(dev_cum - cum).max())},
            "accuracy": {"reference": "FP64 run", "max_abs_dL_whole_run": float(np.abs(cum - ref).max())},
            "cpu_baseline": cpu, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def host_libc_bath_state(seed, nbath):
    """The bath state as the reference draws it (SingleSampleCCE::
    prepare_bath_state, src/source/app/single_sample_cce.cpp:35-46): srand(seed),
    then rand() % 2 per bath spin, from the host's own C library (the
    reference arm loads nothing of the GPU library)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(ctypes.c_uint(seed))
    return np.array([libc.rand() % 2 for _ in range(nbath)], np.uint8)


def single_workload():
    w = workload("cce4")
    w.name += f"_single_sample_seed{BATH_STATE_SEED}"
    return w


def oracle_counts(w):
    """Cluster counts per order from the oracle's enumeration (the reference
    arm loads nothing of the GPU library)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    e = po.Enumeration(w.coords, w.cutoff, w.max_order)
    return [e.count(o) for o in range(w.max_order)]


def run_reference(args, ws, rank):
    if rank != 0:
        return
    if args.workload == "single":
        w = single_workload()
        state = host_libc_bath_state(BATH_STATE_SEED, len(w.coords))
        rate, ms_step, cores, text = cpu_steps_single(w, state, max(1, args.steps), args.warmup,
                                                      args.cpu_seconds / 5.0)
        print(json.dumps({
            "impl": "reference", "metric": "cluster-propagations/s (single-sample CCE)",
            "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(w, oracle_counts(w), ws),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": text},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    if args.workload == "dephasing":
        w = dephasing_workload()
        rate, cores, text = cpu_sample_liouville(w, args.cpu_seconds * max(1, args.steps) / 5.0)
        print(json.dumps({
            "impl": "reference", "metric": "cluster-propagations/s (Liouville space, bath dephasing)",
            "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(w, oracle_counts(w), ws),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": text},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    w = workload(args.workload)
    rate, ms_step, cores, text = cpu_reference_steps(w, max(1, args.steps), args.warmup,
                                                     args.cpu_seconds / 5.0)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": bench_config(w, oracle_counts(w), ws),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": text},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local, dist):
    import torch
    from oops_gb300 import build as b
    b.build()
    from oops_gb300 import cce
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = workload(args.workload, args.nt)
    prec_name = args.precision or "mixed"
    prec = cce.PREC_MIXED if prec_name == "mixed" else cce.PREC_FP64
    _, sv = cce.nv_states(w.B)
    params = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, w.nT, w.dt,
                                fp64_below=args.fp64_below, fp64_max_k=args.fp64_max_k)
    progress(f"workload {w.name}: enumerating and uploading")
    run = cce.DeviceRun(w.coords, w.cutoff, w.max_order, params, prec, device=dev,
                        limit=args.limit_clusters)
    progress(f"clusters per order {run.counts}")
    if args.limit_clusters:
        w.name += f"_limit{args.limit_clusters}"
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)  # 512 MiB > L2
    # kernel timing events are captured into the graph, so profiling is on
    # before the capture; the counters are reset before the timed region
    cce.profile_enable(True)
    use_graph = args.graph == "on" and not (prec != cce.PREC_FP64 and args.fp64_below > 0)
    for _ in range(args.warmup):
        run.step()
    if use_graph:
        run.make_graph()
        run.step_graph()
    step = run.step_graph if use_graph else run.step
    torch.cuda.synchronize(dev)
    progress("warm-up done; timed steps")
    # ---- timed region: K steps, L2 flushed between steps (flush not timed)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    cce.profile_enable(True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            flush.fill_(float(s))
            evs[s][0].record(stream)
            step()
            evs[s][1].record(stream)
        torch.cuda.synchronize(dev)
    if dist is not None:
        dist.barrier()
    ms = [a.elapsed_time(b_) for a, b_ in evs]
    ms_step = float(np.mean(ms))
    prof = {k: cce.profile_read(k) for k in range(1, w.max_order + 1)}
    prof_eig = {k: cce.profile_read_eig(k) for k in range(1, w.max_order + 1)}
    cce.profile_enable(False)
    tot_ms = max_over_ranks(sum(ms), dist, dev)
    value = ws * run.n_clusters * args.steps / (tot_ms / 1e3)
    progress(f"timed steps done: {ms_step:.1f} ms per step; size classes alone")
    iso = isolated_class_times(w, run, params, prec)
    roof, crit = roofline(w, run, prec, prof, prof_eig, iso, ms_step)
    progress("end to end through the C-ABI")
    # ---- end to end through the C-ABI with host buffers
    if args.limit_clusters:
        # profiling case: the C-ABI run would do the full workload
        e2e_ms, cum = [float("nan")], run.cum.cpu().numpy().T
    e2e_ms = [] if not args.limit_clusters else e2e_ms
    for s in range(0 if args.limit_clusters else max(2, min(args.steps, 5))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        cum = cce.ensemble_cce(w.coords, w.cutoff, w.max_order, params, prec,
                               stream=stream.cuda_stream)[0]
        torch.cuda.synchronize(dev)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = ws * run.n_clusters / (np.mean(e2e_ms) / 1e3)
    h2d = w.coords.nbytes
    d2h = 2 * w.max_order * w.nT * 8 + w.max_order * 8
    # the C-ABI run enumerates and uploads cluster lists and closures too
    h2d += run.h2d_bytes - run.coords.numel() * 8
    # results agree with the device-resident run
    dev_cum = run.cum.cpu().numpy().T
    agree = float(np.abs(dev_cum - cum).max())
    acc, head = None, None
    if not args.limit_clusters and args.accuracy == "on":
        progress("accuracy against the FP64 path")
        acc, head = accuracy_check(w, params, prec, run, dev)
    plain = None
    if args.plain_seconds > 0:
        rows = {o: run.idx[o][:run.counts[o]].cpu().numpy() for o in range(w.max_order)}
        progress("plain FP64 Krylov sample")
        plain = plain_krylov_sample(w, sv, args.plain_seconds, value / ws, run.counts, rows, head)
    if rank != 0:
        return
    cpu = None
    if args.cpu_seconds > 0:
        progress("CPU baseline sample")
        rate, _, cores, text = cpu_reference_steps(w, 3, 1, args.cpu_seconds / 3.0)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": text}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == cce.PREC_FP64 else "f32 (f64 eigenbasis)",
            "data": "synthetic",
            "config": bench_config(w, run.counts, ws),
            "run": {"precision": prec_name, "cuda_graph": use_graph,
                    "fp64_below": args.fp64_below, "fp64_max_k": args.fp64_max_k},
            "roofline": roof, "critical_path": crit, "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": float(np.mean(e2e_ms)),
                    "max_abs_diff_vs_device_run": agree},
            "accuracy": acc, "plain_fp64_krylov": plain,
            "clocks": clk.summary(), "gpu_launches": run.launches_per_step() * args.steps}
    print(json.dumps(line), flush=True)


def isolated_class_times(w, run, params, prec):
    """Each size class run alone (outside the timed region, after it): CUDA
    events around its eigensolver phase (assembly, eigensolver, overlaps,
    phase steps) and its coherence kernel with nothing else on the GPU.  In
    the timed run the classes share the GPU on concurrent streams, so their
    own events there include waiting for SMs; these isolated times are the
    kernels' durations."""
    import torch
    from oops_gb300 import cce
    out = {}
    for o in range(w.max_order):
        n = run.counts[o]
        if not n:
            continue
        k = o + 1
        cce.profile_enable(True)
        cce.cluster_coherence(run.coords, run.idx[o][:n], k, params, prec)
        torch.cuda.synchronize()
        cms, cn, cfl = cce.profile_read(k)
        ems, en = cce.profile_read_eig(k)
        out[k] = {"eig_ms": ems / max(en, 1), "coherence_ms": cms / max(cn, 1),
                  "coherence_exec_flop": cfl / max(cn, 1)}
    cce.profile_enable(False)
    return out


def roofline(w, run, prec, prof, prof_eig, iso, ms_step):
    """The roofline object of the kernel that bounds the step, and the
    per-class picture.  The dominant kernel is the single largest of the
    size classes' eigensolver phases and coherence kernels, timed alone
    (isolated_class_times); the timed run's own per-class events (concurrent
    streams, so including waits for SMs) are reported beside them.  A
    tensor-core coherence kernel is measured against the dense bf16 peak
    (algorithmic F(D) flop count); the eigensolver, a Jacobi method with FP64
    eigenvalues, against the FP64 rate of the CUDA cores, with its FP64-pipe
    utilisation from the committed ncu capture."""
    bf16, hbm, src = peaks()
    cls = []
    for k in sorted(iso):
        D = 2 ** k
        f_alg = run.counts[k - 1] * w.nT * 2 * (2 * (w.pulse_num + 1) - 1) * 8 * D ** 3
        cms, cn, _ = prof[k]
        ems, en = prof_eig[k]
        cls.append({"k": k, "eig_ms": iso[k]["eig_ms"], "coherence_ms": iso[k]["coherence_ms"],
                    "coherence_kernel": kernel_name(k, prec, w.pulse_num),
                    "coherence_alg_flop": f_alg, "coherence_exec_flop": iso[k]["coherence_exec_flop"],
                    "in_run_eig_ms": ems / max(en, 1), "in_run_coherence_ms": cms / max(cn, 1)})
    dom = max(cls, key=lambda c: max(c["eig_ms"], c["coherence_ms"]))
    eig_bound = dom["eig_ms"] > dom["coherence_ms"]
    crit = {"step_ms": ms_step, "dominant_class_k": dom["k"],
            "isolated_serial_sum_ms": sum(c["eig_ms"] + c["coherence_ms"] for c in cls),
            "classes": [{"k": c["k"], "eigensolver_ms": c["eig_ms"], "coherence_ms": c["coherence_ms"],
                         "coherence_kernel": c["coherence_kernel"],
                         "in_run_eigensolver_ms": c["in_run_eig_ms"],
                         "in_run_coherence_ms": c["in_run_coherence_ms"]} for c in cls],
            "timing": "eigensolver_ms / coherence_ms: each class alone after the timed region; "
                      "in_run_*: the timed run's own events, classes concurrent on streams"}
    # the coherence kernel of the dominant class, against the tensor peak
    kms = dom["coherence_ms"]
    achieved = dom["coherence_alg_flop"] / (kms / 1e3) / 1e12 if kms > 0 else None
    # DRAM bytes of one launch of the dominant coherence kernel: ncu
    # dram__bytes_read.sum + dram__bytes_write.sum per cluster on a small case
    # with one work item per cluster, as in the full run, times the clusters
    traffic = None
    per = COHERENCE_DRAM_BYTES_PER_CLUSTER_NCU.get(dom["k"])
    if per is not None and dom["coherence_kernel"].startswith("k_coherence_tc"):
        traffic = per * run.counts[dom["k"] - 1]
    # ncu capture of the eigensolver on a small case (profiles/
    # assemble_eig6_cce6_small.md): FP64 pipe busy fraction per size class
    fp64_pipe_ncu = EIG_FP64_PIPE_NCU.get(dom["k"])
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
            "frac": (achieved / bf16) if achieved else None, "traffic": traffic,
            "traffic_source": "ncu DRAM bytes per cluster on 1216 clusters (profiles/coherence_tc_cce6_1216.md) "
                              "x the launch's clusters" if traffic else None,
            "kernel": dom["coherence_kernel"], "peak_source": f"{src} dense bf16 (burst)",
            "kernel_ms_per_launch": kms,
            "algorithmic_flop_per_launch": dom["coherence_alg_flop"],
            "algorithmic_flop_model": "nT*2*(2*(pulse_num+1)-1)*8*D^3 per cluster",
            "executed_flop_per_launch": dom["coherence_exec_flop"],
            "executed_TFLOPs": dom["coherence_exec_flop"] / (kms / 1e3) / 1e12 if kms > 0 else None,
            "fp32_simt_peak_TFLOPs": FP32_SIMT_PEAK, "fp64_peak_TFLOPs": FP64_PEAK,
            "step_share": kms / ms_step,
            "eigensolver": {"kernel": f"k_assemble_eig<{dom['k']}> (+ overlaps, phase steps)",
                            "bound": "fp64", "ms_per_launch": dom["eig_ms"],
                            "step_share": dom["eig_ms"] / ms_step,
                            "fp64_pipe_frac_ncu": fp64_pipe_ncu,
                            "fp64_pipe_evidence": "profiles/assemble_eig6_cce6_small.md "
                                                  "(ncu sm__pipe_fp64_cycles_active)"},
            "dominant_kernel": (f"k_assemble_eig<{dom['k']}> (eigensolver, FP64 eigenvalues)"
                                if eig_bound else dom["coherence_kernel"]),
            "timing": "each size class alone after the timed region (CUDA events on its stream)"}
    return roof, crit


def main():
    args = parse()
    ws, rank, local, dist = dist_setup(args)
    try:
        if args.workload == "c4":
            run_c4(args, ws, rank, local)
        elif args.workload == "serve":
            run_serve(args, ws, rank, local)
        elif args.impl == "reference":
            run_reference(args, ws, rank)
        elif args.workload == "dephasing":
            run_dephasing(args, ws, rank, local, dist)
        elif args.workload == "single":
            run_single(args, ws, rank, local, dist)
        else:
            run_ours(args, ws, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
