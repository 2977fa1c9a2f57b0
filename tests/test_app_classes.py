"""The reference application's classes in the C++ layer (include/oops_host.hpp):
tests/cpp/ensnvebath_demo.cpp is EnsNVeBath's main (src/application/
EnsNVeBath.cpp:40-62) over liboops_gb300 -- options map, NVCenter,
cSpinSourceUniformRandom, cSpinCollection::getConnectionMatrix,
cDepthFirstPathTracing, EnsembleCCE(my_rank, worker_num, para) and its five
steps; tests/cpp/ensnvnbath_demo.cpp is EnsNVnBath's (src/application/
EnsNVnBath.cpp:13-60), the nuclear-spin bath read by cSpinSourceFromFile
from its default input under $CCE_PROJ_PATH/dat/input/.

CPU: the bath the spin source draws is armadillo's C++11 randu (std::
mt19937_64 seeded with `seed`, std::uniform_real_distribution) restated in
Python bit for bit, and equals the reference's own spin source compiled from
its sources (tests/golden/reference_spin_source.npz, made by
tests/golden/make_reference_spin_source.py) bit for bit; the clusters grown
from the connection matrix equal the oracle's enumeration.  GPU: the whole run equals the oracle's pipeline
(enumeration, per-cluster propagation, reduction) on the same bath.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import pyoracle as po
from oops_gb300 import build as ob

GAMMA = {"13C": 6.728284e7, "E": -1.760859708e11}
GAMMA_NVE = -1.760859708e11


class MT19937_64:
    """std::mt19937_64 (the standard's parameters)."""

    def __init__(self, seed):
        self.mt = [0] * 312
        self.mt[0] = seed & 0xFFFFFFFFFFFFFFFF
        for i in range(1, 312):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) \
                & 0xFFFFFFFFFFFFFFFF
        self.i = 312

    def __call__(self):
        if self.i >= 312:
            up, lo = 0xFFFFFFFF80000000, 0x7FFFFFFF
            for k in range(312):
                y = (self.mt[k] & up) | (self.mt[(k + 1) % 312] & lo)
                v = self.mt[(k + 156) % 312] ^ (y >> 1)
                if y & 1:
                    v ^= 0xB5026F5AA96619E9
                self.mt[k] = v
            self.i = 0
        y = self.mt[self.i]
        self.i += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y


def uniform_random_bath(range_, max_num, num, seed):
    """cSpinSourceUniformRandom::generate (SpinSource.cpp:112-129) with the
    C++11 randu: canonical doubles x / 2^64 rounded to nearest."""
    g = MT19937_64(seed)
    u = []
    for _ in range(3 * max_num):
        x = float(g()) / 2.0 ** 64
        u.append(x if x < 1.0 else np.nextafter(1.0, 0.0))
    m = np.array(u).reshape(max_num, 3)  # column i of the 3 x max_num matrix
    c = 2.0 * range_ * m - range_
    d = np.sqrt((c * c).sum(axis=1))
    order = np.argsort(d, kind="stable")
    return c[order[:num]]


def _demo(args, bath_only=False):
    exe = ob.build_ensnvebath_demo()
    cmd = [exe] + (["--bath-only"] if bath_only else []) + list(args)
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    return r


OPTS = ["--number", "30", "--max_number", "400", "--concentration", "5", "--cutoff", "350",
        "--cce", "3", "--seed", "7"]


def test_spin_source_and_clusters_match_the_reference_algorithms():
    r = _demo(OPTS, bath_only=True)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.splitlines()[-1])
    coords = np.array(d["coords"])
    range_ = 0.5e2 * 3.57 * (400 / 5.0 / 8) ** (1.0 / 3.0)
    ref = uniform_random_bath(range_, 400, 30, 7)
    assert np.array_equal(coords, ref)
    assert d["isotope"] == "E"
    diff = coords[:, None, :] - coords[None, :, :]
    dist = np.sqrt((diff ** 2).sum(axis=2))
    assert d["connections"] == int(((dist <= 350.0).sum()) - len(coords))
    e = po.Enumeration(coords, 350.0, 3)
    for o in range(3):
        got = np.array(d["clusters"][o], dtype=np.uint64).reshape(-1, o + 1)
        assert np.array_equal(got, e.clusters(o)), o


SOURCE = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_spin_source.npz"))


@pytest.mark.parametrize("name", sorted({k.split("/")[0] for k in SOURCE.files}))
def test_spin_source_equals_the_reference_code(name):
    """The bath the demo's cSpinSourceUniformRandom draws, with the range
    EnsNVeBath's create_spin_source computes from the options, equals the
    reference's own cSpinSourceUniformRandom::generate (compiled from its
    sources over the armadillo stand-in's C++11 generator;
    tests/golden/reference_spin_source.npz) bit for bit."""
    l0, cell, conc, mx, num, seed = SOURCE[f"{name}/params"]
    iso = str(SOURCE[f"{name}/isotope"])
    r = _demo(["--length", "%.17g" % l0, "--num_cell", str(int(cell)), "--concentration", "%.17g" % conc,
               "--max_number", str(int(mx)), "--number", str(int(num)), "--seed", str(int(seed)),
               "--isotope", iso, "--cutoff", "1", "--cce", "1"], bath_only=True)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.splitlines()[-1])
    assert d["isotope"] == iso
    assert np.array_equal(np.array(d["coords"]), SOURCE[f"{name}/coords"])


def test_ensnvnbath_reads_its_bath_and_grows_the_reference_clusters(tmp_path):
    """EnsNVnBath's main (tests/cpp/ensnvnbath_demo.cpp) with its default
    input, C13Bath/RoyCoord.xyz under $CCE_PROJ_PATH/dat/input/ (the
    reference's own 548-spin bath, from tests/golden/reference_pins.npz):
    the bath it reads, the options' default output name, and the clusters
    it grows, equal to the reference's own enumeration of that bath at
    cutoff 5 A up to four spins, bit for bit."""
    from oops_gb300 import build as ob
    pins = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pins.npz"))
    coords = pins["roy/coords"]
    d_in = tmp_path / "dat" / "input" / "C13Bath"
    d_in.mkdir(parents=True)
    with open(d_in / "RoyCoord.xyz", "w") as f:
        f.write(f"{len(coords)}\n")
        for c in coords:
            f.write("13C\t%.17g\t%.17g\t%.17g\n" % tuple(c))
    exe = ob.build_ensnvnbath_demo()
    r = subprocess.run([exe, "--bath-only", "--cutoff", "5.0", "--cce", "4"], capture_output=True, text=True,
                       timeout=600, env=dict(os.environ, CCE_PROJ_PATH=str(tmp_path)))
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.splitlines()[-1])
    assert np.array_equal(np.array(d["coords"]), coords)
    assert d["isotope"] == "13C"
    assert d["output"] == "EnsNVnBath--cutoff5.0--cce4"
    for o in range(4):
        got = np.array(d["clusters"][o], dtype=np.uint64).reshape(-1, o + 1)
        ref = pins[f"enum/roy/c5.0/o4/idx{o}"].astype(np.uint64).reshape(-1, o + 1)
        assert np.array_equal(got, ref), o


def test_unknown_option_is_an_error_not_a_crash():
    r = _demo(["--no_such_option", "1"], bath_only=True)
    assert r.returncode == 2 and "unknown option" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("rate", [0.0, 1e4])
def test_ensnvebath_main_matches_the_oracle_pipeline(rate):
    """Steps 1-5 of EnsNVeBath, Hilbert space (no dephasing) and the
    application's default bath dephasing (Liouville space)."""
    # a short grid: electron-spin pairs 300 A apart decohere within ~1e-4 s,
    # after which the cluster expansion of this bath no longer converges
    nT, t1, Bs = 11, 1e-5, "0.002 0.001 0.003"
    args = OPTS + ["--nTime", str(nT), "--finish", str(t1), "--magnetic_field", Bs,
                   "--dephasing_rate", str(rate)]
    r = _demo(args)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.splitlines()[-1])
    coords = np.array(d["coords"])
    B = np.array([float(x) for x in Bs.split()])
    center = np.full(3, 3.57 / 4.0)
    _, sv = po.nv_states(B)
    e = po.Enumeration(coords, 350.0, 3)
    dt = t1 / (nT - 1)
    Lraw = []
    for o in range(3):
        Lo = []
        for row in e.clusters(o):
            c = coords[[int(x) for x in row]]
            H = [po.dense_hamiltonian(po.cluster_hamiltonian(c, B, center, sv[s], g=GAMMA["E"],
                                                             gc=GAMMA_NVE)) for s in (0, 1)]
            if rate:
                Lo.append(po.coherence_liouville(o + 1, H[0], H[1], 1, nT, dt,
                                                 dephase_rate=2 * np.pi * rate, axis=(1.0, 1.0, 1.0)))
            else:
                Lo.append(po.coherence_hilbert(H[0], H[1], 1, nT, dt))
        Lraw.append(np.stack(Lo, axis=1) if Lo else np.zeros((nT, 0)))
    _, _, cum = e.reduce(Lraw, nT)
    got = np.array(d["final"]).T
    assert got.shape == cum.shape
    assert np.abs(cum).max() <= 2.0  # no divergence of the expansion on this grid
    assert np.abs(got - cum).max() <= 1e-8
