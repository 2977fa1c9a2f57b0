"""The C++ host layer (include/oops_host.hpp): KronProd / SumKronProd /
MatExpVector and EnsembleCCE driven from C++ (tests/cpp/host_demo.cpp, built
by build()) exactly as the reference's C++ drives its own classes
(src/source/math/MatExp.cpp:86-160, src/source/app/cce.cpp:42-80).

CPU: the demo program links against liboops_gb300.so and runs without a
device.
GPU: its results equal the Python path's (same library calls) and the
oracle's within the parity tolerances.
"""
import subprocess

import numpy as np
import pytest

import pyoracle as po
from oops_gb300 import build as ob


def _demo():
    return ob.build_host_demo()


def test_host_demo_links_and_runs_without_a_device():
    r = subprocess.run([_demo(), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage" in r.stdout


def test_host_demo_rejects_bad_usage(tmp_path):
    r = subprocess.run([_demo(), "expv", str(tmp_path / "missing.txt"), str(tmp_path / "o.txt")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1


def _cx(z):
    return f"{float(z.real)!r} {float(z.imag)!r}"


def _write_expv_input(path, t, v, tl, m, tol):
    from oops_gb300.expv import KronTerms
    coeff, nbody, poff, plist, dlist, moff, mats, sdim = KronTerms.coerce(t).arrays()
    lines = [str(len(sdim)), " ".join(str(int(x)) for x in sdim), str(len(coeff))]
    for j in range(len(coeff)):
        lines.append(f"{float(coeff[j])!r} {int(nbody[j])}")
        for b in range(int(poff[j]), int(poff[j + 1])):
            d = int(dlist[b])
            blk = mats[int(moff[b]):int(moff[b + 1])]
            lines.append(f"{int(plist[b])} {d} " + " ".join(_cx(z) for z in blk))
    lines.append(" ".join(_cx(z) for z in v))
    lines.append(str(len(tl)))
    lines.append(" ".join(repr(float(x)) for x in tl))
    lines.append(f"{int(m)} {float(tol)!r}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@pytest.mark.gpu
def test_cpp_matexpvector_matches_oracle_and_python_path(tmp_path):
    import oops_gb300 as og
    rng = np.random.default_rng(11)
    coords = rng.normal(size=(7, 3)) * 3.0 + 4.0
    B = np.array([0.0, 0.0, 0.05])
    _, sv = po.nv_states(B)
    t = po.cluster_hamiltonian(coords, B, np.zeros(3), sv[1])
    v = rng.normal(size=t.dim) + 1j * rng.normal(size=t.dim)
    v /= np.linalg.norm(v)
    tl = np.array([0.0, 2e-5, 7e-5, 1.5e-4])
    inp, out = tmp_path / "expv.txt", tmp_path / "expv.out"
    _write_expv_input(inp, t, v, tl, 30, 1e-12)
    r = subprocess.run([_demo(), "expv", str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.loadtxt(out).reshape(-1, 2)
    got = (raw[:, 0] + 1j * raw[:, 1]).reshape(len(tl), t.dim).T   # N x nt, column-major
    py = og.main_cache(t, v, tl, m=30, tol=1e-12)
    assert np.abs(got - py).max() <= 1e-14
    ref, _ = po.expv(t, v, tl, m=30, tol=1e-12)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-10


@pytest.mark.gpu
def test_cpp_ensemble_cce_matches_python_path_and_oracle(tmp_path):
    from oops_gb300 import cce, configs
    w = configs.cce2_hahn()
    nT, t1 = 41, 2e-3
    inp, out = tmp_path / "cce.txt", tmp_path / "cce.out"
    with open(inp, "w") as f:
        f.write(" ".join(repr(float(x)) for x in w.B) + f" {float(w.cutoff)!r} {int(w.max_order)} {int(w.pulse_num)} "
                f"{t1!r} {nT} {cce.PREC_FP64} {len(w.coords)}\n")
        for c in w.coords:
            f.write(" ".join(repr(float(x)) for x in c) + "\n")
    mat = tmp_path / "cce.mat"
    r = subprocess.run([_demo(), "cce", str(inp), str(out), str(mat)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    vals = np.loadtxt(out)
    K = w.max_order
    counts = vals[:K].astype(int)
    cum = vals[K:K + K * nT].reshape(K, nT).T        # nT x K, column-major
    each = vals[K + K * nT:].reshape(K, nT).T
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, nT, t1 / (nT - 1))
    py_cum, py_each, py_counts = cce.ensemble_cce(w.coords, w.cutoff, K, p, cce.PREC_FP64)
    assert list(counts) == list(py_counts)
    assert np.abs(cum - py_cum).max() <= 1e-12
    assert np.abs(each - py_each).max() <= 1e-12
    # the oracle pipeline (CPU restatement of enumeration, propagation, reduction)
    e = po.Enumeration(w.coords, w.cutoff, K)
    Lraw = []
    for o in range(K):
        rows = e.clusters(o)
        assert counts[o] == len(rows)
        Lo = []
        for r in rows:
            H = [po.dense_hamiltonian(po.cluster_hamiltonian(w.coords[list(r)], w.B, np.zeros(3), sv[s]))
                 for s in (0, 1)]
            Lo.append(po.coherence_hilbert(H[0], H[1], w.pulse_num, nT, t1 / (nT - 1)))
        Lraw.append(np.stack(Lo, axis=1))
    _, each_o, cum_o = e.reduce(Lraw, nT)
    assert np.abs(cum - cum_o).max() <= 1e-8
    assert np.abs(each - each_o).max() <= 1e-8
    # export_mat_file: the reference's result variables, bit-identical to the text output
    import scipy.io as sio
    m = sio.loadmat(str(mat))
    assert np.array_equal(m["final_result"], cum)
    assert np.array_equal(m["final_result_each_order"], each)
    assert m["time_list"].shape == (nT, 1) and m["time_list"][-1, 0] == pytest.approx(t1)
    for o in range(K):
        assert m[f"CCE{o}"].shape == (nT, counts[o])


@pytest.mark.gpu
def test_cpp_ensemble_cce_with_dephasing_matches_python_path(tmp_path):
    """EnsembleCCE with the reference's bath dephasing and polarisation
    parameters (ensemble_cce.cpp:16-18) runs the Liouville path and equals the
    Python front end's oops_ensemble_cce_bath run."""
    from oops_gb300 import cce, configs
    w = configs.cce2_hahn()
    nT, t1, K = 21, 2e-3, 3
    rate, axis, pol = 1e4, (1.0, 1.0, 1.0), (0.05, 0.0, 0.1)
    inp, out = tmp_path / "cce.txt", tmp_path / "cce.out"
    with open(inp, "w") as f:
        f.write(" ".join(repr(float(x)) for x in w.B) + f" {float(w.cutoff)!r} {K} {int(w.pulse_num)} "
                f"{t1!r} {nT} {cce.PREC_FP64} {len(w.coords)}\n")
        for c in w.coords:
            f.write(" ".join(repr(float(x)) for x in c) + "\n")
        f.write(f"{rate!r} " + " ".join(repr(float(x)) for x in axis + pol) + "\n")
    r = subprocess.run([_demo(), "cce", str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vals = np.loadtxt(out)
    cum = vals[K:K + K * nT].reshape(K, nT).T
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, nT, t1 / (nT - 1))
    py_cum = cce.ensemble_cce(w.coords, w.cutoff, K, p, bath=cce.CCEBath.make(rate, axis, pol))[0]
    assert np.abs(cum - py_cum).max() <= 1e-12
