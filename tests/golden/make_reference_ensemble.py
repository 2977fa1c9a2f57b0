"""Generates tests/golden/reference_ensemble.npz: whole ensemble-CCE runs of
the reference's own application classes (ensemble_cce.cpp, cce.cpp,
DefectCenter.cpp, the quantum operator, state and evolution classes,
KronProd/spkron, MatExp and the spin sources, compiled from the reference
tree by oracle/build_ref.sh into oracle/_ref/ref_ensemble_pin; expokit's
Fortran ZGPADM is the oracle's C restatement), so that the cluster
propagation and the reduction can be pinned where the reference tree is
absent.  The steps are the reference's EnsNVeBath main: NVCenter (N14) at the
origin (its electron at 3.57/4 (1, 1, 1)), the bath from a file, clusters,
run_each_clusters (Liouville space), post_treatment.  Two cases:

* "cce2_dephasing": the CCE-2 workload bath (cutoff 4.5 A, two orders), Hahn
  echo, 11 points of [0, 1 ms], B = (0.03, -0.01, 0.04) T, bath dephasing
  1e4 Hz along (1, 1, 1) and polarisation (0.1, -0.05, 0.2): the reference
  application's own physics;
* "cce4_cpmg2": the CCE-4 workload bath (cutoff 6 A, four orders), CPMG-2,
  6 points of [0, 2 ms], 0.1 T tilted 3 degrees from [111] (azimuth 1.1 rad),
  no dephasing and no polarisation: the configs' physics, which the
  Hilbert-space path computes (about five minutes in the reference's code).

Each case stores the bath, the run parameters, the NV electron position and,
per order, the reference's raw cluster curves L_C (clusters x points) and
reduced curves, then the per-order and cumulative products.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_ensemble.py
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
    "cce2_dephasing": dict(coords=lambda: configs.cce2_hahn().coords, cutoff=4.5, K=2, nT=11, t_max=1e-3,
                           pulse_num=1, B=np.array([0.03, -0.01, 0.04]), rate=1e4,
                           pol=np.array([0.1, -0.05, 0.2])),
    "cce4_cpmg2": dict(coords=lambda: configs.cce4_hahn().coords, cutoff=6.0, K=4, nT=6, t_max=2e-3,
                       pulse_num=2, B=configs.tilted_field(0.1, 3.0, 1.1), rate=0.0, pol=np.zeros(3)),
}


def g(x):
    return "%.17g" % float(x)


def run_case(name, c, tmp):
    coords = c["coords"]()
    xyz = os.path.join(tmp, name + ".xyz")
    write_xyz(xyz, coords)
    out = os.path.join(tmp, name + ".out")
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_ensemble_pin")
    args = [exe, xyz, g(c["cutoff"]), str(c["K"]), str(c["nT"]), g(c["t_max"]), str(c["pulse_num"]),
            *map(g, c["B"]), g(c["rate"]), *map(g, c["pol"]), out]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL)
    e = po.Enumeration(coords, c["cutoff"], c["K"])
    cnt = [e.count(o) for o in range(c["K"])]
    d = np.fromfile(out, np.float64)
    K, nT = c["K"], c["nT"]
    res = {f"{name}/coords": coords, f"{name}/center": NV_ELECTRON,
           f"{name}/params": np.array([c["cutoff"], K, nT, c["t_max"], c["pulse_num"], c["rate"]]),
           f"{name}/B": np.asarray(c["B"], float), f"{name}/pol": np.asarray(c["pol"], float)}
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
    np.savez_compressed(os.path.join(HERE, "reference_ensemble.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_ensemble.npz"))


if __name__ == "__main__":
    main()
