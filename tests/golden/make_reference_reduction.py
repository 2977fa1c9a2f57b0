"""Generates tests/golden/reference_reduction.npz: results of the reference's
own CCE reduction, src/source/app/cce.cpp (cce_coherence_reduction and
compuate_final_coherence, compiled from the reference tree by
oracle/build_ref.sh into oracle/_ref/ref_cce_pin), on cluster curves written
here, so that the reduction can be pinned where the reference tree is
absent.  Three cases, each over the reference's own enumeration of a bath:

* "cce4_random": the CCE-4 workload bath (cutoff 6 A, four orders), seeded
  curves uniform in [-1, 1] (every sign and near-zero divisors), 8 points;
* "roy_random": the reference's 548-spin RoyCoord.xyz (cutoff 5 A, four
  orders), seeded curves uniform in [-1, 1], 4 points;
* "cce4_physical": the CCE-4 workload bath with the oracle's Hilbert-space
  coherence of every cluster at 0.1 T tilted 3 degrees, CPMG-8, 6 points of
  [0, 8 ms] (curves that cross zero, as in the CCE-6 workload).

Each case stores the bath, cutoff, order, point count, the input curves per
order (clusters x points, the enumeration's order) and the reference's
reduced curves, per-order products and cumulative products.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_reduction.py
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
from oops_gb300 import bath, configs  # noqa: E402


def run_reference(coords, cutoff, K, nT, curves, tmp, name):
    xyz = os.path.join(tmp, name + ".xyz")
    write_xyz(xyz, coords)
    cin, cout = os.path.join(tmp, name + ".in"), os.path.join(tmp, name + ".out")
    with open(cin, "wb") as f:
        for L in curves:
            f.write(np.ascontiguousarray(L, np.float64).tobytes())
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_cce_pin")
    subprocess.run([exe, xyz, str(cutoff), str(K), str(nT), cin, cout], check=True,
                   stdout=subprocess.DEVNULL)
    out = np.fromfile(cout, np.float64)
    til, pos = [], 0
    for L in curves:
        n = L.shape[0]
        til.append(out[pos:pos + n * nT].reshape(n, nT))
        pos += n * nT
    each = out[pos:pos + K * nT].reshape(K, nT)
    pos += K * nT
    cum = out[pos:pos + K * nT].reshape(K, nT)
    return til, each, cum


def physical_curves(coords, cutoff, K, nT):
    B = configs.tilted_field(0.1, 3.0, 1.1)
    _, sv = po.nv_states(B)
    e = po.Enumeration(coords, cutoff, K)
    dt = 8e-3 / (nT - 1)
    curves = []
    for o in range(K):
        rows = []
        for r in e.clusters(o):
            H = [po.dense_hamiltonian(po.cluster_hamiltonian(coords[list(r)], B, np.zeros(3), sv[s]))
                 for s in (0, 1)]
            rows.append(po.coherence_hilbert(H[0], H[1], 8, nT, dt))
        curves.append(np.array(rows))
    return curves


def main():
    ref = os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    roy, _ = bath.read_xyz(os.path.join(ref, "src", "dat_example", "input", "C13Bath", "RoyCoord.xyz"))
    cce4 = configs.cce4_hahn().coords
    tmp = tempfile.mkdtemp()
    out = {}
    for name, coords, cutoff, K, nT, seed in (("cce4_random", cce4, 6.0, 4, 8, 7),
                                               ("roy_random", roy, 5.0, 4, 4, 11),
                                               ("cce4_physical", cce4, 6.0, 4, 6, None)):
        e = po.Enumeration(coords, cutoff, K)
        if seed is None:
            curves = physical_curves(coords, cutoff, K, nT)
        else:
            rng = np.random.default_rng(seed)
            curves = [rng.uniform(-1.0, 1.0, size=(e.count(o), nT)) for o in range(K)]
        til, each, cum = run_reference(coords, cutoff, K, nT, curves, tmp, name)
        out[f"{name}/coords"] = coords
        out[f"{name}/params"] = np.array([cutoff, K, nT], np.float64)
        for o in range(K):
            out[f"{name}/curves{o}"] = curves[o]
            out[f"{name}/tilde{o}"] = til[o]
        out[f"{name}/each"] = each
        out[f"{name}/cum"] = cum
        print(name, [c.shape[0] for c in curves])
    np.savez_compressed(os.path.join(HERE, "reference_reduction.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_reduction.npz"))


if __name__ == "__main__":
    main()
