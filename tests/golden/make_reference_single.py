"""Generates tests/golden/reference_single.npz: whole single-sample CCE runs of
the reference's own SingleSampleCCE (single_sample_cce.cpp with cce.cpp,
DefectCenter.cpp, the quantum, spin and Kronecker classes and MatExp,
compiled from the reference tree by oracle/build_ref.sh into
oracle/_ref/ref_single_pin; expokit's Fortran ZGPADM is the oracle's C
restatement), so that the single-sample path can be pinned where the
reference tree is absent.  The steps are the reference's SingleSampleCCE_NV_C13
main: NVCenter (N14) at the origin (its electron at 3.57/4 (1, 1, 1)), the
bath from a file, clusters, prepare_bath_state (srand(seed); rand() % 2 per
bath spin, from this host's C library), run_each_clusters, post_treatment.
Two cases:

* "cce2_hahn": the CCE-2 workload bath (cutoff 4.5 A, two orders), Hahn echo,
  11 points of [0, 1 ms], B = (0.03, -0.01, 0.04) T, bath state seed 2024;
* "cce4_cpmg2": the CCE-4 workload bath (cutoff 6 A, four orders), CPMG-2,
  6 points of [0, 2 ms], 0.1 T tilted 3 degrees from [111] (azimuth 1.1
  rad), bath state seed 7.

Each case stores the bath, the run parameters, the NV electron position, the
bath state the reference drew and, per order, the reference's raw and reduced
cluster curves (clusters x points), then the per-order and cumulative
products.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_single.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import pyoracle as po  # noqa: E402
from make_reference_pins import write_xyz  # noqa: E402
from oops_gb300 import configs  # noqa: E402

# NVCenter::add_spin_member (DefectCenter.cpp): the electron at coord + a/4 (1, 1, 1), a = 3.57
NV_ELECTRON = 3.57 / 4.0 * np.ones(3)

CASES = {
    "cce2_hahn": dict(coords=lambda: configs.cce2_hahn().coords, cutoff=4.5, K=2, nT=11, t_max=1e-3,
                      pulse_num=1, B=np.array([0.03, -0.01, 0.04]), seed=2024),
    "cce4_cpmg2": dict(coords=lambda: configs.cce4_hahn().coords, cutoff=6.0, K=4, nT=6, t_max=2e-3,
                       pulse_num=2, B=configs.tilted_field(0.1, 3.0, 1.1), seed=7),
}


def g(x):
    return "%.17g" % float(x)


def run_case(name, c, tmp):
    coords = c["coords"]()
    xyz = os.path.join(tmp, name + ".xyz")
    write_xyz(xyz, coords)
    out = os.path.join(tmp, name + ".out")
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_single_pin")
    args = [exe, xyz, g(c["cutoff"]), str(c["K"]), str(c["nT"]), g(c["t_max"]), str(c["pulse_num"]),
            *map(g, c["B"]), str(c["seed"]), out]
    r = subprocess.run(args, check=True, capture_output=True, text=True)
    bits = [l.split()[1] for l in r.stdout.splitlines() if l.startswith("bath_state ")][0]
    state = np.array([int(ch) for ch in bits], np.uint8)
    assert state.size == len(coords)
    e = po.Enumeration(coords, c["cutoff"], c["K"])
    cnt = [e.count(o) for o in range(c["K"])]
    d = np.fromfile(out, np.float64)
    K, nT = c["K"], c["nT"]
    res = {f"{name}/coords": coords, f"{name}/center": NV_ELECTRON, f"{name}/state": state,
           f"{name}/params": np.array([c["cutoff"], K, nT, c["t_max"], c["pulse_num"], c["seed"]]),
           f"{name}/B": np.asarray(c["B"], float)}
    pos = 0
    for what in ("raw", "tilde"):
        for o in range(K):
            res[f"{name}/{what}{o}"] = d[pos:pos + cnt[o] * nT].reshape(cnt[o], nT)
            pos += cnt[o] * nT
    res[f"{name}/each"] = d[pos:pos + K * nT].reshape(K, nT)
    pos += K * nT
    res[f"{name}/cum"] = d[pos:pos + K * nT].reshape(K, nT)
    assert pos + K * nT == d.size
    return res


def main():
    os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    tmp = tempfile.mkdtemp()
    out = {}
    for name, c in CASES.items():
        out.update(run_case(name, c, tmp))
        print(name, "done")
    np.savez_compressed(os.path.join(HERE, "reference_single.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_single.npz"))


if __name__ == "__main__":
    main()
