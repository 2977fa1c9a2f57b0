"""Generates tests/golden/reference_expv_args.npz: the arguments the
reference's own Krylov caller hands the drop-in (MatExpVector::runInexplicit,
src/source/math/MatExp.cpp:216-360, calling main_mkl_) for NV-conditional
cluster Hamiltonians built by the reference's own classes (oracle/_ref/
ref_expv_pin, compiled by oracle/build_ref.sh), so that the drop-in boundary
can be pinned where the reference tree is absent: the product's and the
oracle's term lists are compared with them.

Clusters: the first cluster of each size 2..4 of the CCE-4 workload bath
(cutoff 6 A), in NV states 0 and 1, at 0.1 T tilted 3 degrees from [111]
(azimuth 1.1 rad); the NVCenter (N14) at the origin, so its electron sits at
3.57/4 (1, 1, 1); 5 output times up to 0.1 ms; start vector basis state 0.
(A one-spin Hamiltonian's Kronecker form starts from the empty dipolar
interaction, and the reference's SumKronProd then reports dimension 0:
MatExpVector cannot run on it, so single spins are not recorded.)

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_expv_args.py
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

NT, T_MAX = 5, 1e-4
FIELDS = ("coeff", np.float64), ("nbody", np.uint64), ("pos_offset", np.uint64), ("pos_list", np.uint64), \
    ("dim_list", np.uint64), ("mat_offset", np.uint64), ("spin_dim", np.uint64), ("mats", np.complex128), \
    ("v", np.complex128), ("tlist", np.float64)


def parse(path):
    d = open(path, "rb").read()
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(d, dt, n, pos).copy()
        pos += a.nbytes
        return a

    nspin, nterm, ndim, tnb, tdim, klim, nt, m = (int(x) for x in take(np.uint64, 8))
    tol = float(take(np.float64, 1)[0])
    sizes = {"coeff": nterm, "nbody": nterm, "pos_offset": nterm + 1, "pos_list": tnb, "dim_list": tnb,
             "mat_offset": tnb + 1, "spin_dim": nspin, "mats": tdim, "v": ndim, "tlist": nt}
    out = {k: take(dt, sizes[k]) for k, dt in FIELDS}
    assert pos == len(d)
    out["scalars"] = np.array([nspin, nterm, ndim, klim, m], np.uint64)
    out["tol"] = np.array([tol])
    return out


def main():
    os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    w = configs.cce4_hahn()
    e = po.Enumeration(w.coords, 6.0, 4)
    B = configs.tilted_field(0.1, 3.0, 1.1)
    tmp = tempfile.mkdtemp()
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_expv_pin")
    out = {"B": B, "coords": w.coords}
    for k in range(2, 5):
        idx = e.clusters(k - 1)[0]
        xyz = os.path.join(tmp, f"c{k}.xyz")
        write_xyz(xyz, w.coords[list(idx)])
        for state in (0, 1):
            path = os.path.join(tmp, f"c{k}_s{state}.bin")
            subprocess.run([exe, xyz, *("%.17g" % x for x in B), str(state), str(NT), "%.17g" % T_MAX, path],
                           check=True, stdout=subprocess.DEVNULL)
            key = f"k{k}/s{state}"
            out[f"{key}/cluster"] = np.asarray(idx, np.int64)
            for name, arr in parse(path).items():
                out[f"{key}/{name}"] = arr
            print(key, out[f"{key}/scalars"])
    np.savez_compressed(os.path.join(HERE, "reference_expv_args.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_expv_args.npz"))


if __name__ == "__main__":
    main()
