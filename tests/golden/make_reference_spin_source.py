"""Generates tests/golden/reference_spin_source.npz: baths drawn by the
reference's own cSpinSourceUniformRandom::generate (SpinSource.cpp:112-129,
compiled from the reference tree by oracle/build_ref.sh into
oracle/_ref/ref_pin, over the armadillo stand-in's C++11 generator), with
the range EnsNVeBath's create_spin_source computes
(EnsNVeBath.cpp:193-206: 0.5e2 * length * (max_number / concentration /
num_cell)^(1/3)), so that the application layer's spin source can be pinned
where the reference tree is absent.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_spin_source.py
"""
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (length, num_cell, concentration, max_number, number, seed, isotope)
CASES = {
    "defaults": (3.57, 8, 1.0, 2000, 100, 1, "E"),
    "dense_seed7": (3.57, 8, 5.0, 400, 30, 7, "E"),
    "c13_seed12345": (3.57, 8, 0.011, 5000, 400, 12345, "13C"),
}


def main():
    os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_pin")
    out = {}
    for name, (l0, cell, conc, max_num, num, seed, iso) in CASES.items():
        rng = 0.5e2 * l0 * (max_num / conc / cell) ** (1.0 / 3.0)
        r = subprocess.run([exe, "random", "%.17g" % rng, str(max_num), str(num), iso, str(seed)],
                           check=True, capture_output=True, text=True)
        rows = [l.split() for l in r.stdout.splitlines() if l.startswith("spin ")]
        assert len(rows) == num and all(row[1] == iso for row in rows)
        out[f"{name}/coords"] = np.array([[float(x) for x in row[2:5]] for row in rows])
        out[f"{name}/params"] = np.array([l0, cell, conc, max_num, num, seed])
        out[f"{name}/isotope"] = np.array(iso)
        print(name, num, "spins")
    np.savez_compressed(os.path.join(HERE, "reference_spin_source.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_spin_source.npz"))


if __name__ == "__main__":
    main()
