"""Parity pins on the reference's own compiled code (tests/golden/
reference_pins.npz, made by tests/golden/make_reference_pins.py from the
reference's Spin*, SpinCollection, SpinCluster* and misc sources compiled by
oracle/build_ref.sh).  Integer work bit-exact: every cluster's spin indices
and sub-cluster closure, on the reference's own 548-spin bath file and the
workload baths, for the product's enumeration (liboops_gb300) and the
oracle's; the 49k-cluster CCE-6 enumeration through per-order SHA-256
digests.  Physics: the oracle's dipole tensors, Zeeman terms and CPMG
intervals against the reference's dipole(), zeeman(), Pulse_Interval(), bit
for bit.  Reduction (tests/golden/reference_reduction.npz, made by
tests/golden/make_reference_reduction.py from the reference's cce.cpp): the
oracle's bit for bit, the product's GPU reduction to 1e-12 relative."""
import hashlib
import os

import numpy as np
import pytest

import pyoracle as po
from oops_gb300.cce import Clusters

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = np.load(os.path.join(HERE, "golden", "reference_pins.npz"))

CASES = sorted({"/".join(k.split("/")[1:4]) for k in PINS.files if k.startswith("enum/")})


def _case(key):
    name, c, o = key.split("/")
    return name, float(c[1:]), int(o[1:])


def _product(coords, cut, order):
    c = Clusters(coords, cut, order)
    out = []
    for o in range(order):
        off, pairs = c.subclusters(o)
        out.append((c.clusters(o).astype(np.uint32), off.astype(np.uint64), pairs.astype(np.uint32)))
    return out


def _oracle(coords, cut, order):
    e = po.Enumeration(coords, cut, order)
    out = []
    for o in range(order):
        idx = e.clusters(o).astype(np.uint32)
        off, pairs = [0], []
        for j in range(e.count(o)):
            s = e.subclusters(o, j)
            pairs.extend(s)
            off.append(off[-1] + len(s))
        out.append((idx, np.array(off, np.uint64), np.array(pairs, np.uint32).reshape(-1, 2)))
    return out


@pytest.mark.parametrize("key", CASES)
@pytest.mark.parametrize("impl", ["product", "oracle"])
def test_enumeration_equals_the_reference_code(key, impl):
    name, cut, order = _case(key)
    coords = PINS[f"{name}/coords"]
    got = (_product if impl == "product" else _oracle)(coords, cut, order)
    for o in range(order):
        idx, off, pairs = got[o]
        ref_idx = PINS[f"enum/{key}/idx{o}"]
        assert np.array_equal(idx, ref_idx.reshape(idx.shape) if ref_idx.size else idx), (key, o)
        assert idx.shape[0] == ref_idx.reshape(-1, o + 1).shape[0]
        assert np.array_equal(off, PINS[f"enum/{key}/off{o}"]), (key, o)
        assert np.array_equal(pairs.reshape(-1, 2), PINS[f"enum/{key}/pairs{o}"].reshape(-1, 2)), (key, o)


def test_cce6_enumeration_digest_equals_the_reference_code():
    """The CCE-6 CPMG-8 workload bath at 7 A up to six spins: 49,365 clusters
    and their closures, equal to the reference's output through SHA-256 of
    each order's indices, closure offsets and closure pairs."""
    coords = PINS["cce6/coords"]
    got = _product(coords, 7.0, 6)
    counts = PINS["digest/cce6/c7.0/o6/counts"]
    sha = PINS["digest/cce6/c7.0/o6/sha256"]
    for o in range(6):
        idx, off, pairs = got[o]
        assert idx.shape[0] == counts[o]
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(idx, np.uint32).tobytes())
        h.update(np.ascontiguousarray(off, np.uint64).tobytes())
        h.update(np.ascontiguousarray(pairs, np.uint32).tobytes())
        assert h.hexdigest() == str(sha[o]), o


@pytest.mark.parametrize("name", ["roy", "cce4"])
def test_dipole_tensors_equal_the_reference_code(name):
    """dipole() of misc.cpp:11-36 (prefactor hbar mu0 / 4 pi g1 g2 / r^3 with
    r in Angstrom x 1e-10, armadillo's datum constants standing in as CODATA
    2014): the oracle's tensors bit for bit."""
    coords = PINS[f"{name}/coords"]
    ij = PINS[f"phys/{name}/dip_ij"]
    ref = PINS[f"phys/{name}/dip"]
    got = np.array([po.dipole(coords[i], coords[j], po.GAMMA_C13, po.GAMMA_C13) for i, j in ij])
    assert np.array_equal(got, ref)


def test_zeeman_and_cpmg_intervals_equal_the_reference_code():
    B = PINS["phys/B"]
    z = PINS["phys/roy/zeeman"]
    # zeeman(): -gamma B per axis, then the quadrupole entries (zero for 13C)
    assert np.array_equal(z[:, :3], np.tile(-po.GAMMA_C13 * B, (z.shape[0], 1)))
    assert np.all(z[:, 3:] == 0.0)
    for n in range(1, 9):
        assert np.array_equal(po.cpmg_intervals(n), PINS[f"phys/cpmg{n}"]), n


RED = np.load(os.path.join(HERE, "golden", "reference_reduction.npz"))
RED_CASES = sorted({k.split("/")[0] for k in RED.files})


def _reduction_case(name):
    cut, K, nT = RED[f"{name}/params"]
    K, nT = int(K), int(nT)
    curves = [RED[f"{name}/curves{o}"] for o in range(K)]
    tilde = [RED[f"{name}/tilde{o}"] for o in range(K)]
    return RED[f"{name}/coords"], float(cut), K, nT, curves, tilde, RED[f"{name}/each"], RED[f"{name}/cum"]


@pytest.mark.parametrize("name", RED_CASES)
def test_reduction_equals_the_reference_code(name):
    """The oracle's CCE reduction (L~_C = L_C / prod L~_sub in the closure's
    (order, position) order, then the per-order and cumulative products)
    reproduces the reference's own cce_coherence_reduction and
    compuate_final_coherence (src/source/app/cce.cpp:151-189, compiled by
    oracle/build_ref.sh) bit for bit, on random curves with every sign and on
    physical curves that cross zero."""
    coords, cut, K, nT, curves, tilde, each, cum = _reduction_case(name)
    e = po.Enumeration(coords, cut, K)
    assert [e.count(o) for o in range(K)] == [c.shape[0] for c in curves]
    til, ea, cu = e.reduce([c.T for c in curves], nT)
    for o in range(K):
        assert np.array_equal(np.asarray(til[o]).T, tilde[o])
    assert np.array_equal(np.asarray(ea).T, each)
    assert np.array_equal(np.asarray(cu).T, cum)


@pytest.mark.gpu
@pytest.mark.parametrize("name", RED_CASES)
def test_gpu_reduction_matches_the_reference_code(name):
    """The product's reduction on the GPU (oops_cce_reduce: (mantissa,
    exponent) products in FP64 over the CSR closures) against the reference's
    own reduction on the same curves, to 1e-12 relative: every operation is a
    division or a multiplication, so the results differ only by the rounding
    of a different association order."""
    torch = pytest.importorskip("torch")
    from oops_gb300 import cce, configs
    coords, cut, K, nT, curves, tilde, each, cum = _reduction_case(name)
    B = configs.tilted_field(0.1, 3.0, 1.1)
    _, sv = cce.nv_states(B)
    p = cce.CCEParams.make(B, sv[0], sv[1], 1, nT, 1e-5)
    run = cce.DeviceRun(coords, cut, K, p, cce.PREC_FP64)
    assert run.counts == [c.shape[0] for c in curves]
    got_cum = run.reduce_curves([torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in curves])
    torch.cuda.synchronize()

    def close(a, b):
        return np.all(np.abs(a - b) <= 1e-12 * np.abs(b) + 1e-300)

    for o in range(K):
        assert close(run.til[o][:curves[o].shape[0]].cpu().numpy(), tilde[o])
    assert close(run.each.cpu().numpy(), each)
    assert close(got_cum.cpu().numpy(), cum)
