"""Generates tests/golden/hamvec_reference.npz: outputs of the reference's own
Kronecker matvec (src/expv/source/hamvec_func3.cpp, compiled from the
reference tree by oracle/build_ref.sh) on seeded term sets -- random one- and
two-body operators on spins of dimension 2 and 3, and NV-conditional cluster
Hamiltonians of the spin physics -- so that the oracle's matvec can be pinned
bit for bit where the reference tree is absent.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle as po  # noqa: E402
from helpers import random_terms  # noqa: E402


def cases():
    rng = np.random.default_rng(2024)
    for dims in [(2, 2, 2), (2, 2, 2, 2, 2, 2), (3, 2, 2), (2, 3, 2, 3), (2,) * 10]:
        yield "random_" + "x".join(map(str, dims)), random_terms(rng, list(dims))
    B = np.array([0.0, 0.0, 0.05])
    _, sv = po.nv_states(B)
    for k in (4, 8):
        coords = rng.normal(size=(k, 3)) * 3.0 + 5.0
        yield f"cluster_k{k}", po.cluster_hamiltonian(coords, B, np.zeros(3), sv[1])


def main():
    os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    if po.ref_lib() is None:
        sys.exit("reference matvec not built: the reference tree is needed to make the fixtures")
    out = {}
    rng = np.random.default_rng(99)
    for name, t in cases():
        v = rng.normal(size=t.dim) + 1j * rng.normal(size=t.dim)
        cz = -1j * t.coeff
        ref = po.ref_hamvec(t, v, cz)
        for field in ("coeff", "nbody", "pos_offset", "pos_list", "dim_list", "mat_offset", "mats",
                      "spin_dim"):
            out[f"{name}/{field}"] = getattr(t, field)
        out[f"{name}/v"] = v
        out[f"{name}/w_ref"] = ref
    np.savez_compressed(os.path.join(HERE, "hamvec_reference.npz"), **out)
    print("wrote", len({k.split('/')[0] for k in out}), "cases")


if __name__ == "__main__":
    main()
