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
oracle's bit for bit, the product's GPU reduction to 1e-12 relative.  Whole
ensemble-CCE runs of the reference's own application classes
(tests/golden/reference_ensemble.npz, made by
tests/golden/make_reference_ensemble.py; its Pade exponential is the
oracle's restatement of the Fortran ZGPADM): the oracle's Liouville and
Hilbert propagation and reduction, and the product's FP64, mixed and
Liouville-space paths and whole run, within the stated tolerances.  The
drop-in's arguments (tests/golden/reference_expv_args.npz, made by
tests/golden/make_reference_expv_args.py): what the reference's own
MatExpVector hands main_mkl_, against the product's and the oracle's term
lists.  Whole single-sample CCE runs of the reference's own SingleSampleCCE
(tests/golden/reference_single.npz, made by
tests/golden/make_reference_single.py): the bath state it drew against the
product's generator, bit for bit, and its cluster curves and final curves
against the oracle's single-sample propagation and reduction."""
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


ENS = np.load(os.path.join(HERE, "golden", "reference_ensemble.npz"))


def _ensemble_case(name):
    cut, K, nT, t_max, n, rate = ENS[f"{name}/params"]
    K, nT, n = int(K), int(nT), int(n)
    raw = [ENS[f"{name}/raw{o}"] for o in range(K)]
    return dict(coords=ENS[f"{name}/coords"], center=ENS[f"{name}/center"], cutoff=float(cut), K=K, nT=nT,
                dt=float(t_max) / (nT - 1), n=n, rate=float(rate), B=ENS[f"{name}/B"], pol=ENS[f"{name}/pol"],
                raw=raw, cum=ENS[f"{name}/cum"])


def _oracle_hamiltonians(c, idx, sv):
    return [po.dense_hamiltonian(po.cluster_hamiltonian(c["coords"][list(idx)], c["B"], c["center"], sv[s]))
            for s in (0, 1)]


# The reference's Liouville-space propagation (4^k-dimensional Pade
# exponentials and one product per segment and time step) against the
# Hilbert-space eigenbasis form differs by FP64 rounding of those products:
# 7.3e-11 at most over the CCE-4 case's 680 clusters
TOL_FP64_CLUSTER = 2e-10


def test_ensemble_liouville_with_dephasing_equals_the_reference_code():
    """The reference's own EnsembleCCE run (application classes compiled by
    oracle/build_ref.sh; EnsNVeBath's steps; Liouville space with bath
    dephasing 1e4 Hz and a polarised bath) against the oracle's Liouville
    propagation of every cluster and the oracle's reduction of its curves."""
    c = _ensemble_case("cce2_dephasing")
    _, sv = po.nv_states(c["B"])
    e = po.Enumeration(c["coords"], c["cutoff"], c["K"])
    axis = np.ones(3) / np.sqrt(3.0)
    curves = []
    for o in range(c["K"]):
        rows = []
        for j, idx in enumerate(e.clusters(o)):
            H = _oracle_hamiltonians(c, idx, sv)
            L = po.coherence_liouville(o + 1, H[0], H[1], c["n"], c["nT"], c["dt"],
                                       dephase_rate=2 * np.pi * c["rate"], axis=axis, pol=c["pol"])
            assert np.abs(L - c["raw"][o][j]).max() <= 1e-11
            rows.append(L)
        curves.append(np.array(rows))
    _, _, cum = e.reduce([x.T for x in curves], c["nT"])
    assert np.abs(np.asarray(cum).T - c["cum"]).max() <= 1e-9


def test_ensemble_hilbert_form_equals_the_reference_code():
    """The configs' physics (no dephasing, unpolarised bath, tilted field,
    CPMG-2) on the CCE-4 bath: the oracle's Hilbert-space coherence of every
    cluster against the reference's own Liouville-space EnsembleCCE run."""
    c = _ensemble_case("cce4_cpmg2")
    _, sv = po.nv_states(c["B"])
    e = po.Enumeration(c["coords"], c["cutoff"], c["K"])
    curves = []
    for o in range(c["K"]):
        rows = []
        for j, idx in enumerate(e.clusters(o)):
            H = _oracle_hamiltonians(c, idx, sv)
            L = po.coherence_hilbert(H[0], H[1], c["n"], c["nT"], c["dt"])
            assert np.abs(L - c["raw"][o][j]).max() <= TOL_FP64_CLUSTER
            rows.append(L)
        curves.append(np.array(rows))
    _, _, cum = e.reduce([x.T for x in curves], c["nT"])
    assert np.abs(np.asarray(cum).T - c["cum"]).max() <= 1e-9


def _product_params(c):
    from oops_gb300 import cce
    _, sv = cce.nv_states(c["B"])
    return cce.CCEParams.make(c["B"], sv[0], sv[1], c["n"], c["nT"], c["dt"], center=c["center"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, TOL_FP64_CLUSTER), (1, 1e-6)])
def test_gpu_cluster_curves_match_the_reference_code(precision, tol):
    """The product's Hilbert-space path (FP64 and mixed precision) on every
    cluster of the CCE-4 case against the reference's own EnsembleCCE run,
    and its whole FP64 run (device-resident, with the reduction) against the
    reference's final curves."""
    torch = pytest.importorskip("torch")
    from oops_gb300 import cce
    c = _ensemble_case("cce4_cpmg2")
    p = _product_params(c)
    cl = Clusters(c["coords"], c["cutoff"], c["K"])
    cd = torch.from_numpy(np.ascontiguousarray(c["coords"])).cuda()
    for o in range(c["K"]):
        idx = torch.from_numpy(cl.clusters(o).astype(np.int32)).cuda()
        L = cce.cluster_coherence(cd, idx, o + 1, p, precision).cpu().numpy()
        assert np.abs(L - c["raw"][o]).max() <= tol
    if precision == cce.PREC_FP64:
        run = cce.DeviceRun(c["coords"], c["cutoff"], c["K"], p, cce.PREC_FP64)
        cum = run.step().cpu().numpy()
        assert np.abs(cum - c["cum"]).max() <= 1e-9


@pytest.mark.gpu
def test_gpu_liouville_path_matches_the_reference_code():
    """The product's Liouville-space path with bath dephasing and polarisation
    (oops_cce_coherence_liouville) on every cluster of the CCE-2 case against
    the reference's own EnsembleCCE run."""
    torch = pytest.importorskip("torch")
    from oops_gb300 import cce
    c = _ensemble_case("cce2_dephasing")
    p = _product_params(c)
    bath = cce.CCEBath.make(dephasing_rate=c["rate"], dephasing_axis=(1.0, 1.0, 1.0), polarization=c["pol"])
    cl = Clusters(c["coords"], c["cutoff"], c["K"])
    cd = torch.from_numpy(np.ascontiguousarray(c["coords"])).cuda()
    for o in range(c["K"]):
        idx = torch.from_numpy(cl.clusters(o).astype(np.int32)).cuda()
        L = cce.cluster_coherence_liouville(cd, idx, o + 1, p, bath).cpu().numpy()
        assert np.abs(L - c["raw"][o]).max() <= 1e-10


ARGS = np.load(os.path.join(HERE, "golden", "reference_expv_args.npz"))
ARG_KEYS = sorted({"/".join(k.split("/")[:2]) for k in ARGS.files if k.startswith("k")})
NV_ELECTRON = 3.57 / 4.0 * np.ones(3)


def _captured_terms(key):
    from oops_gb300.expv import KronTerms
    return KronTerms(*(ARGS[f"{key}/{f}"] for f in ("coeff", "nbody", "pos_offset", "pos_list", "dim_list",
                                                    "mat_offset", "mats", "spin_dim")))


@pytest.mark.parametrize("key", ARG_KEYS)
@pytest.mark.parametrize("impl", ["product", "oracle"])
def test_term_lists_equal_what_the_reference_caller_passes(key, impl):
    """The arguments the reference's own MatExpVector (MatExp.cpp:216-360)
    hands main_mkl_ for an NV-conditional cluster Hamiltonian built by the
    reference's own classes: the product's term lists (oops_gb300.spin) and
    the oracle's equal them -- term order, bodies, positions, dimensions and
    operator matrices bit for bit, coefficients to 1e-13 relative (the
    hyperfine mean-field terms depend on the NV eigenstate, which the two
    sides compute with different eigensolvers; the others are bit-exact).
    The GPU tests of main_cache_ (tests/test_gpu_expv.py) run on the product's
    term lists, so they hold for the reference caller's arguments too."""
    from oops_gb300 import spin
    ref = _captured_terms(key)
    cluster = ARGS[f"{key}/cluster"]
    state = int(key.split("/")[1][1:])
    _, sv = po.nv_states(ARGS["B"])
    coords = ARGS["coords"][cluster]
    t = (spin.cluster_terms if impl == "product" else po.cluster_hamiltonian)(coords, ARGS["B"], NV_ELECTRON,
                                                                             sv[state])
    for f in ("nbody", "pos_offset", "pos_list", "dim_list", "mat_offset", "spin_dim"):
        assert np.array_equal(np.asarray(getattr(t, f), np.uint64), getattr(ref, f)), f
    assert np.array_equal(np.asarray(t.mats, np.complex128), ref.mats)
    c = np.asarray(t.coeff)
    assert c.shape == ref.coeff.shape
    assert np.all(np.abs(c - ref.coeff) <= 1e-13 * np.abs(ref.coeff))


SINGLE = np.load(os.path.join(HERE, "golden", "reference_single.npz"))
SINGLE_CASES = sorted({k.split("/")[0] for k in SINGLE.files})


def _single_case(name):
    cut, K, nT, t_max, n, seed = SINGLE[f"{name}/params"]
    K, nT = int(K), int(nT)
    return dict(coords=SINGLE[f"{name}/coords"], center=SINGLE[f"{name}/center"], state=SINGLE[f"{name}/state"],
                cutoff=float(cut), K=K, nT=nT, dt=float(t_max) / (nT - 1), n=int(n), seed=int(seed),
                B=SINGLE[f"{name}/B"], raw=[SINGLE[f"{name}/raw{o}"] for o in range(K)],
                each=SINGLE[f"{name}/each"], cum=SINGLE[f"{name}/cum"])


@pytest.mark.parametrize("name", SINGLE_CASES)
def test_bath_state_equals_the_reference_draw(name):
    """The product's bath state (oops_bath_state_from_seed, glibc's srand/rand
    restated) equals the state the reference's own prepare_bath_state drew
    (single_sample_cce.cpp:35-46, compiled and run on this host)."""
    from oops_gb300 import cce
    c = _single_case(name)
    assert np.array_equal(cce.bath_state_from_seed(c["seed"], len(c["coords"])), c["state"])


@pytest.mark.parametrize("name", SINGLE_CASES)
def test_single_sample_equals_the_reference_code(name):
    """Whole single-sample CCE runs of the reference's own SingleSampleCCE
    (tests/golden/reference_single.npz): the oracle's cluster Hamiltonians
    with the mean dipolar field of the bath outside the cluster
    (pyoracle.bath_field), its propagation of the cluster's basis state
    (orc_coherence_state) and its reduction.  Measured: 1.9e-12 per cluster
    and 1.4e-12 over the whole run at most (FP64 rounding of the reference's
    Pade exponentials and power products)."""
    from helpers import SX, SY, SZ
    c = _single_case(name)
    _, sv = po.nv_states(c["B"])
    e = po.Enumeration(c["coords"], c["cutoff"], c["K"])
    curves = []
    for o in range(c["K"]):
        rows = []
        for j, idx in enumerate(e.clusters(o)):
            k = len(idx)
            f = po.bath_field(c["coords"], c["state"], idx)
            H = _oracle_hamiltonians(c, idx, sv)
            for s in (0, 1):
                for q in range(k):
                    for a, S in enumerate((SX, SY, SZ)):
                        H[s] = H[s] + f[q, a] * np.kron(np.kron(np.eye(2 ** q), S), np.eye(2 ** (k - 1 - q)))
            b = sum(int(c["state"][i]) << (k - 1 - q) for q, i in enumerate(idx))
            L = po.coherence_state(H[0], H[1], c["n"], c["nT"], c["dt"], b)
            assert np.abs(L - c["raw"][o][j]).max() <= 1e-11
            rows.append(L)
        curves.append(np.array(rows))
    _, each, cum = e.reduce([x.T for x in curves], c["nT"])
    assert np.abs(np.asarray(each).T - c["each"]).max() <= 1e-10
    assert np.abs(np.asarray(cum).T - c["cum"]).max() <= 1e-10
