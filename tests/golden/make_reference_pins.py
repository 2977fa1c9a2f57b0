"""Generates tests/golden/reference_pins.npz: outputs of the reference's own
spin, cluster and physics code (compiled from the reference tree by
oracle/build_ref.sh into oracle/_ref/ref_pin, with oracle/ref_shim/armadillo
standing in for armadillo), so that cluster enumeration, sub-cluster
closures, dipole and Zeeman coefficients and CPMG intervals can be pinned
where the reference tree is absent:

* enumeration (cSpinCollection::getConnectionMatrix, cDepthFirstPathTracing,
  cSpinCluster::getSubClusters) on the reference's own 548-spin bath file
  (src/dat_example/input/C13Bath/RoyCoord.xyz) and on the CCE-2 and CCE-4
  workload baths: every cluster's spin indices and closure; on the CCE-6
  workload bath (49k clusters, two minutes in the reference's code) the
  counts and a SHA-256 of each order's indices and closures;
* dipole() for the first 300 spin pairs of RoyCoord and of the CCE-4 bath,
  zeeman() at a fixed field, Pulse_Interval("CPMG", n) for n = 1..8.

Run from the repository root (the reference tree at OOPS_REFERENCE_ROOT,
default /root/reference):
    python tests/golden/make_reference_pins.py
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oops_gb300 import bath, configs  # noqa: E402

BZ = (0.02, -0.01, 0.07)


def run_pin(*args):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_pin")
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, check=True)
    # the reference prints progress with carriage returns; keep the last part
    return [l.split("\r")[-1] for l in r.stdout.split("\n")]


def parse_enum(lines, max_order):
    idx = {o: [] for o in range(max_order)}
    off = {o: [0] for o in range(max_order)}
    pairs = {o: [] for o in range(max_order)}
    o = -1
    for l in lines:
        if l.startswith("order "):
            o = int(l.split()[1])
        elif l.startswith("c "):
            left, right = l[2:].split("|")
            idx[o].append([int(x) for x in left.split()])
            r = [int(x) for x in right.split()]
            pairs[o].extend(r[1:])
            off[o].append(off[o][-1] + r[0])
    out = {}
    for o in range(max_order):
        out[o] = (np.array(idx[o], np.uint32).reshape(-1, o + 1), np.array(off[o], np.uint64),
                  np.array(pairs[o], np.uint32).reshape(-1, 2))
    return out


def digest(idx, off, pairs):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(idx, np.uint32).tobytes())
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(pairs, np.uint32).tobytes())
    return h.hexdigest()


def write_xyz(path, coords, iso="13C"):
    with open(path, "w") as f:
        f.write(f"{len(coords)}\n")
        for c in coords:
            f.write(f"{iso}\t%.17g\t%.17g\t%.17g\n" % tuple(c))


def main():
    ref = os.environ.setdefault("OOPS_REFERENCE_ROOT", "/root/reference")
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    roy = os.path.join(ref, "src", "dat_example", "input", "C13Bath", "RoyCoord.xyz")
    roy_coords, _ = bath.read_xyz(roy)
    out = {"roy/coords": roy_coords}
    tmp = tempfile.mkdtemp()
    baths = {"roy": (roy, roy_coords)}
    for name, fn in (("cce2", configs.cce2_hahn), ("cce4", configs.cce4_hahn), ("cce6", configs.cce6_cpmg8)):
        w = fn()
        p = os.path.join(tmp, name + ".xyz")
        write_xyz(p, w.coords)
        baths[name] = (p, w.coords)
        out[f"{name}/coords"] = w.coords
    full = [("roy", 5.0, 4), ("roy", 4.5, 3), ("cce2", 4.5, 2), ("cce4", 6.0, 4)]
    for name, cut, order in full:
        key = f"enum/{name}/c{cut}/o{order}"
        e = parse_enum(run_pin("enum", baths[name][0], cut, order), order)
        for o in range(order):
            i, f, pr = e[o]
            out[f"{key}/idx{o}"] = i
            out[f"{key}/off{o}"] = f
            out[f"{key}/pairs{o}"] = pr
        print(key, [len(e[o][0]) for o in range(order)])
    key = "digest/cce6/c7.0/o6"
    e = parse_enum(run_pin("enum", baths["cce6"][0], 7.0, 6), 6)
    out[f"{key}/counts"] = np.array([len(e[o][0]) for o in range(6)], np.int64)
    out[f"{key}/sha256"] = np.array([digest(*e[o]) for o in range(6)])
    print(key, out[f"{key}/counts"])
    for name in ("roy", "cce4"):
        lines = run_pin("phys", baths[name][0], 300, *BZ)
        dip = [l.split() for l in lines if l.startswith("dip ")]
        zee = [l.split() for l in lines if l.startswith("zee ")]
        out[f"phys/{name}/dip_ij"] = np.array([[int(a[1]), int(a[2])] for a in dip], np.int64)
        out[f"phys/{name}/dip"] = np.array([[float(x) for x in a[3:]] for a in dip])
        out[f"phys/{name}/zeeman"] = np.array([[float(x) for x in a[2:]] for a in zee])
        if name == "roy":
            cp = [l.split() for l in lines if l.startswith("cpmg ")]
            for a in cp:
                out[f"phys/cpmg{int(a[1])}"] = np.array([float(x) for x in a[2:]])
    out["phys/B"] = np.array(BZ)
    np.savez_compressed(os.path.join(HERE, "reference_pins.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_pins.npz"))


if __name__ == "__main__":
    main()
