"""bench.py on CPU: the N > 1 launch path with gloo (world_size 2) and the
reference arm.  The path is replicas only (clusters are independent but the
reduction needs every sub-cluster, and each box has one GPU): what there is
to check is the max-over-ranks timing reduction and that exactly one rank
prints the line.  The reference arm's line carries the contract's keys,
loads nothing of the GPU library, and its CPU estimator samples the
workload's cluster orders in proportion."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, values, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(values[rank], dist, "cpu")
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    port = _port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, port, [3.5, 7.25], out), nprocs=2, join=True,
                       start_method="spawn")
    assert dict(out) == {0: 7.25, 1: 7.25}


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5, None, "cpu") == 2.5


def test_reference_arm_under_torchrun_prints_one_line():
    port = _port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"


@pytest.mark.parametrize("workload", ["cce6", "cce4", "dephasing", "single"])
def test_reference_arm_line_has_the_contract_keys(workload):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
           "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert "workload" in d["config"]


@pytest.mark.parametrize("workload", ["cce4", "single"])
def test_reference_arm_loads_nothing_of_the_gpu_library(workload):
    """The reference arm times the oracle only: enumeration, NV states and
    bath states come from the oracle or the host C library, so the GPU
    library is never mapped into that process."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', %r, "
            "'--steps', '1', '--warmup', '0', '--cpu-seconds', '1']; sys.path.insert(0, %r); "
            "import bench; bench.main(); "
            "print('MAPPED', open('/proc/self/maps').read().count('liboops_gb300'))") % (workload, ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    mapped = [l for l in r.stdout.splitlines() if l.startswith("MAPPED")]
    assert mapped == ["MAPPED 0"]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    assert set(line["config"]) == {"workload", "clusters_per_order", "nT", "t_max_s", "pulse_num",
                                   "max_order", "cutoff_A", "B_T", "l2", "parallelism"}


@pytest.mark.parametrize("steps,n", [(1, 16), (5, 16), (20, 32), (3, 2), (7, 100)])
def test_cpu_sample_orders_follow_the_workload(steps, n):
    """The CPU estimator's steps (bench.systematic_orders): every step and
    all steps together hold each order within one cluster of its share of
    the workload (the CCE-6 counts, where six-spin clusters are most of the
    cost)."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    counts = np.array([579, 876, 1840, 4430, 11367, 30273])
    share = counts / counts.sum()
    total = np.zeros(len(counts), int)
    for s in range(steps):
        c = np.bincount(bench.systematic_orders(n, (s + 0.5) / steps, counts), minlength=len(counts))
        assert c.sum() == n
        assert np.all(np.abs(c - n * share) <= 1.0 + 1e-9), (c, n * share)
        total += c
    assert np.all(np.abs(total - steps * n * share) <= 1.0 + 1e-9), (total, steps * n * share)
