"""GPU parity of the Liouville-space cluster coherence (bath dephasing and
polarisation, oops_cce_coherence_liouville / oops_ensemble_cce_bath) against
the CPU oracle's restatement of the reference's Liouville propagation
(orc_coherence_liouville: dense 4^k superoperators, Pade exponentials, one
power product per time step, QuantumEvolutionAlgorithm.cpp:60-83), itself
pinned against an independent kron construction in test_oracle.py.
Tolerances: 1e-10 absolute on every L_C(t_i) (FP64 path); whole-run L(t)
1e-8 absolute."""
import numpy as np
import pytest

import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import cce, configs  # noqa: E402
from oops_gb300._lib import OopsError  # noqa: E402

B0 = 0.05 * configs.NV_AXIS
RATE_HZ = 1e4                      # EnsNVeBath default dephasing rate
AXIS = (1.0, 1.0, 1.0)             # EnsNVeBath default dephasing axis
POL = (0.1, -0.05, 0.2)


def _pick(k, count, seed):
    w = configs.cce4_hahn(seed)
    cl = cce.Clusters(w.coords, 6.0, k)
    rows = cl.clusters(k - 1)
    rng = np.random.default_rng(seed)
    return w.coords, rows[rng.choice(len(rows), size=min(count, len(rows)), replace=False)]


def _oracle(coords, idx, B, sv, n, nT, dt, rate_hz, axis, pol):
    H = [po.dense_hamiltonian(po.cluster_hamiltonian(coords[list(idx)], B, np.zeros(3), sv[s]))
         for s in (0, 1)]
    return po.coherence_liouville(len(idx), H[0], H[1], n, nT, dt,
                                  dephase_rate=2 * np.pi * rate_hz, axis=axis, pol=pol)


def _run(coords, pick, k, p, bath):
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    return cce.cluster_coherence_liouville(cd, cl, k, p, bath).cpu().numpy()


@pytest.mark.parametrize("k,n,count", [(1, 1, 6), (2, 1, 6), (2, 2, 4), (2, 3, 4), (3, 1, 4),
                                       (3, 2, 3), (3, 3, 2), (4, 1, 2), (4, 2, 1)])
def test_liouville_matches_oracle_with_dephasing_and_polarisation(k, n, count):
    coords, pick = _pick(k, count, seed=300 + 10 * k + n)
    _, sv = cce.nv_states(B0)
    nT, dt = (9, 2e-4) if k == 4 else (17, 2e-4)
    p = cce.CCEParams.make(B0, sv[0], sv[1], n, nT, dt)
    bath = cce.CCEBath.make(RATE_HZ, AXIS, POL)
    L = _run(coords, pick, k, p, bath)
    for c in range(len(pick)):
        ref = _oracle(coords, pick[c], B0, sv, n, nT, dt, RATE_HZ, AXIS, POL)
        assert np.abs(L[c] - ref).max() <= 1e-10, (c, np.abs(L[c] - ref).max())


@pytest.mark.parametrize("k,n", [(2, 8), (3, 4)])
def test_liouville_many_time_points_binary_powers(k, n):
    """nT = 77 exercises seven binary digits of the middle-segment powers
    (tilted field, dephasing off the field axis, no polarisation)."""
    coords, pick = _pick(k, 2, seed=500 + k)
    B = configs.tilted_field(0.1, 3.0, 0.7)
    _, sv = cce.nv_states(B)
    nT, dt = 77, 1e-4
    p = cce.CCEParams.make(B, sv[0], sv[1], n, nT, dt)
    bath = cce.CCEBath.make(2.5e3, (0.0, 0.3, 1.0), (0.0, 0.0, 0.0))
    L = _run(coords, pick, k, p, bath)
    for c in range(len(pick)):
        ref = _oracle(coords, pick[c], B, sv, n, nT, dt, 2.5e3, (0.0, 0.3, 1.0), (0, 0, 0))
        assert np.abs(L[c] - ref).max() <= 1e-10, (c, np.abs(L[c] - ref).max())
        assert L[c, 0] == pytest.approx(1.0, abs=1e-14)


@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("n", [1, 2])
def test_liouville_without_bath_terms_equals_hilbert_path(k, n):
    """At zero dephasing and polarisation the Liouville observable equals the
    Hilbert-space trace form (the same identity the oracle is pinned on)."""
    coords, pick = _pick(k, 8, seed=700 + k)
    _, sv = cce.nv_states(B0)
    nT, dt = 101, 4e-5
    p = cce.CCEParams.make(B0, sv[0], sv[1], n, nT, dt)
    Ll = _run(coords, pick, k, p, cce.CCEBath.make(0.0, AXIS, (0.0, 0.0, 0.0)))
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    Lh = cce.cluster_coherence(cd, cl, k, p, cce.PREC_FP64).cpu().numpy()
    assert np.abs(Ll - Lh).max() <= 1e-10


def test_liouville_dephasing_changes_curve_and_rejects_large_clusters():
    coords, pick = _pick(3, 4, seed=901)
    _, sv = cce.nv_states(B0)
    p = cce.CCEParams.make(B0, sv[0], sv[1], 1, 41, 1e-4)
    L0 = _run(coords, pick, 3, p, cce.CCEBath.make(0.0))
    L1 = _run(coords, pick, 3, p, cce.CCEBath.make(RATE_HZ))
    assert np.all(L1[:, 0] == pytest.approx(1.0, abs=1e-14))
    assert np.abs(L1).max() <= 1 + 1e-12
    assert np.abs(L1 - L0).max() > 1e-6
    # clusters of more than six spins are rejected (4^7 x 4^7 superoperators)
    with pytest.raises(OopsError):
        _run(coords, np.zeros((1, 7), np.uint32) + np.arange(7, dtype=np.uint32), 7, p,
             cce.CCEBath.make(RATE_HZ))


def test_five_spin_liouville_matches_kron_construction():
    """k = 5 (N = 1024) with dephasing and polarisation against the reference's
    Liouville form built literally from numpy kron products and scipy's
    expm (the construction the oracle is pinned on in test_oracle.py)."""
    sla = pytest.importorskip("scipy.linalg")
    from test_oracle import _liouville_numpy
    coords, pick = _pick(5, 1, seed=950)
    _, sv = cce.nv_states(B0)
    nT, dt = 3, 2e-4
    p = cce.CCEParams.make(B0, sv[0], sv[1], 1, nT, dt)
    L = _run(coords, pick, 5, p, cce.CCEBath.make(RATE_HZ, AXIS, POL))
    H = [po.dense_hamiltonian(po.cluster_hamiltonian(coords[list(pick[0])], B0, np.zeros(3), sv[s]))
         for s in (0, 1)]
    ref = _liouville_numpy(5, H[0], H[1], 1, dt * np.arange(nT), 2 * np.pi * RATE_HZ, AXIS, POL)
    # with polarisation L(0) = D Tr(rho0^2) (68.2 here): the parity bound is
    # relative to the curve's scale
    assert np.abs(L[0] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max()), np.abs(L[0] - ref).max()


@pytest.mark.parametrize("k,nT", [(5, 9), (6, 3)])
def test_large_liouville_clusters_without_bath_terms_equal_hilbert_path(k, nT):
    """Five- and six-spin clusters (N = 1024, 4096): at zero dephasing and
    polarisation the Liouville observable equals the FP64 Hilbert-space path."""
    w = configs.cce6_cpmg8()
    cl = cce.Clusters(w.coords, w.cutoff, k)
    pick = cl.clusters(k - 1)[:1]
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 2, nT, 5e-5)
    Ll = _run(w.coords, pick, k, p, cce.CCEBath.make(0.0, AXIS, (0.0, 0.0, 0.0)))
    cd = torch.from_numpy(w.coords).cuda()
    cl_d = torch.from_numpy(pick.astype(np.int32)).cuda()
    Lh = cce.cluster_coherence(cd, cl_d, k, p, cce.PREC_FP64).cpu().numpy()
    assert np.abs(Ll - Lh).max() <= 1e-10, np.abs(Ll - Lh).max()


def test_ensemble_cce_bath_matches_oracle_pipeline():
    w = configs.cce2_hahn()
    nT, dt = 21, 1e-4
    order = 3
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, nT, dt)
    bath = cce.CCEBath.make(RATE_HZ, AXIS, POL)
    cum, each, counts, per = cce.ensemble_cce(w.coords, w.cutoff, order, p, want_clusters=True,
                                              bath=bath)
    e = po.Enumeration(w.coords, w.cutoff, order)
    Lraw = []
    for o in range(order):
        rows = e.clusters(o)
        assert counts[o] == len(rows)
        Lo = [_oracle(w.coords, r, w.B, sv, 1, nT, dt, RATE_HZ, AXIS, POL) for r in rows]
        Lo = np.stack(Lo, axis=1)
        assert np.abs(per[o] - Lo.T).max() <= 1e-10
        Lraw.append(Lo)
    _, each_o, cum_o = e.reduce(Lraw, nT)
    assert np.abs(cum - cum_o).max() <= 1e-8
    assert np.abs(each - each_o).max() <= 1e-8
