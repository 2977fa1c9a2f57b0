"""Generates tests/golden/reference_export.npz: the variables the reference's
own CCE::export_mat_file (cce.cpp:191-234) writes at the end of a run, as
oracle/_ref/ref_export_pin records them (the ensemble pin with cce.cpp
compiled with HAS_MATLAB over the recording mat.h stand-in of
oracle/ref_shim), so that the result file can be pinned where the reference
tree is absent.  The run is the "cce2_dephasing" case of
make_reference_ensemble.py (CCE-2 bath, Hahn echo, 11 points of [0, 1 ms],
dephasing 1e4 Hz, polarised bath).  Stored: every variable in the order
written ("names"), with its rows x columns matrix and complex flag.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_export.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_reference_ensemble import CASES, g  # noqa: E402
from make_reference_pins import write_xyz  # noqa: E402


def read_records(path):
    """The recording stand-in's records: (name, matrix, complex flag)."""
    d = open(path, "rb").read()
    pos, out = 0, []
    while pos < len(d):
        n = int(np.frombuffer(d, np.uint32, 1, pos)[0])
        pos += 4
        name = d[pos:pos + n].decode()
        pos += n
        rows, cols = (int(x) for x in np.frombuffer(d, np.uint64, 2, pos))
        pos += 16
        cplx = int(np.frombuffer(d, np.uint32, 1, pos)[0])
        pos += 4
        a = np.frombuffer(d, np.float64, rows * cols, pos).reshape(cols, rows).T.copy()
        pos += 8 * rows * cols
        if cplx:
            a = a + 1j * np.frombuffer(d, np.float64, rows * cols, pos).reshape(cols, rows).T
            pos += 8 * rows * cols
        out.append((name, a, cplx))
    return out


def main():
    os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    c = CASES["cce2_dephasing"]
    tmp = tempfile.mkdtemp()
    xyz = os.path.join(tmp, "bath.xyz")
    write_xyz(xyz, c["coords"]())
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_export_pin")
    args = [exe, xyz, g(c["cutoff"]), str(c["K"]), str(c["nT"]), g(c["t_max"]), str(c["pulse_num"]),
            *map(g, c["B"]), g(c["rate"]), *map(g, c["pol"]), os.path.join(tmp, "curves.bin")]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL, env=dict(os.environ, OOPS_PIN_OUTPUT_DIR=tmp))
    recs = read_records(os.path.join(tmp, "pin.mat"))
    out = {"names": np.array([name for name, _, _ in recs])}
    for name, a, cplx in recs:
        out[f"var/{name}"] = a
        out[f"complex/{name}"] = np.array(cplx)
        print(name, a.shape)
    np.savez_compressed(os.path.join(HERE, "reference_export.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_export.npz"))


if __name__ == "__main__":
    main()
