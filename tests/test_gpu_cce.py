"""GPU parity of the batched cluster-coherence path and the ensemble-CCE run
against the CPU oracle (dense Pade + power propagation, the reference's own
algorithm restated in Hilbert space, itself pinned against the Liouville form
in test_oracle.py).  Tolerances: FP64 mode 1e-10 absolute on every L_C(t_i);
mixed mode 1e-6 absolute; whole-run L(t) 1e-8 absolute (FP64)."""
import numpy as np
import pytest

import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import cce, configs  # noqa: E402

B0 = 0.05 * configs.NV_AXIS


def _oracle_L(coords, idx, B, sv, n, nT, dt):
    H = [po.dense_hamiltonian(po.cluster_hamiltonian(coords[list(idx)], B, np.zeros(3), sv[s]))
         for s in (0, 1)]
    return po.coherence_hilbert(H[0], H[1], n, nT, dt)


def _clusters_of(k, count, seed):
    w = configs.cce6_cpmg8(seed) if k > 2 else configs.cce4_hahn(seed)
    cl = cce.Clusters(w.coords, 7.0, k)
    rows = cl.clusters(k - 1)
    rng = np.random.default_rng(seed)
    pick = rows[rng.choice(len(rows), size=min(count, len(rows)), replace=False)]
    return w.coords, pick


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("n", [1, 2, 8])
def test_cluster_coherence_fp64_and_mixed(k, n):
    coords, pick = _clusters_of(k, 3 if k >= 5 else 6, seed=100 + k)
    B = configs.tilted_field(0.1, 3.0, 0.7) if n == 8 else B0
    _, sv = cce.nv_states(B)
    nT, dt = (13, 4e-4) if k == 6 else (25, 2e-4)
    p = cce.CCEParams.make(B, sv[0], sv[1], n, nT, dt)
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    L64 = cce.cluster_coherence(cd, cl, k, p, cce.PREC_FP64).cpu().numpy()
    Lmp = cce.cluster_coherence(cd, cl, k, p, cce.PREC_MIXED).cpu().numpy()
    for c in range(len(pick)):
        ref = _oracle_L(coords, pick[c], B, sv, n, nT, dt)
        assert np.abs(L64[c] - ref).max() <= 1e-10, (c, np.abs(L64[c] - ref).max())
        assert np.abs(Lmp[c] - ref).max() <= 1e-6, (c, np.abs(Lmp[c] - ref).max())
        assert L64[c, 0] == 1.0


def test_ensemble_cce_matches_oracle_pipeline():
    w = configs.cce4_hahn()
    nT, dt = 21, 2e-4
    order = 3
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, nT, dt)
    cum, each, counts, per = cce.ensemble_cce(w.coords, w.cutoff, order, p, cce.PREC_FP64,
                                              want_clusters=True)
    e = po.Enumeration(w.coords, w.cutoff, order)
    Lraw = []
    for o in range(order):
        rows = e.clusters(o)
        assert counts[o] == len(rows)
        Lo = np.stack([_oracle_L(w.coords, r, w.B, sv, 1, nT, dt) for r in rows], axis=1)
        np.testing.assert_allclose(per[o].T, Lo, atol=1e-10, rtol=0)
        Lraw.append(Lo)
    til, each_o, cum_o = e.reduce(Lraw, nT)
    np.testing.assert_allclose(cum, cum_o, atol=1e-8, rtol=0)
    np.testing.assert_allclose(each, each_o, atol=1e-8, rtol=0)


def test_ensemble_cce_mixed_precision_close():
    w = configs.cce4_hahn()
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, 41, 1e-4)
    a = cce.ensemble_cce(w.coords, w.cutoff, 4, p, cce.PREC_FP64)[0]
    b = cce.ensemble_cce(w.coords, w.cutoff, 4, p, cce.PREC_MIXED)[0]
    assert np.abs(a - b).max() <= 1e-6


def test_argument_errors():
    p = cce.CCEParams.make(B0, [0, 0, 0], [0, 0, 1], 1, 5, 1e-4)
    cd = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    cl = torch.zeros((1, 7), dtype=torch.int32, device="cuda")
    from oops_gb300 import OopsError
    with pytest.raises(OopsError):
        cce.cluster_coherence(cd, cl, 7, p)


@pytest.mark.parametrize("k,n,nT", [(3, 1, 6), (3, 2, 6), (4, 8, 41)])
def test_plain_krylov_cluster_path_matches_dense(k, n, nT):
    """The plain FP64 Krylov path (the drop-in's one-step propagators of every
    segment applied to the basis states, then FP64 powers and chains) gives
    the same L_C(t) as the dense batched path, also after 40 powers."""
    from oops_gb300.krylov_cce import cluster_coherence_krylov
    coords, pick = _clusters_of(k, 2, seed=7)
    _, sv = cce.nv_states(B0)
    dt = 2e-4
    p = cce.CCEParams.make(B0, sv[0], sv[1], n, nT, dt)
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    Ld = cce.cluster_coherence(cd, cl, k, p, cce.PREC_FP64).cpu().numpy()
    for c in range(len(pick)):
        tm = {}
        Lk = cluster_coherence_krylov(coords[pick[c].astype(int)], B0, sv, n, nT, dt, m=30,
                                      tol=1e-12, timings=tm)
        assert tm["krylov_steps"] > 0
        assert np.abs(Lk - Ld[c]).max() <= 1e-9


@pytest.mark.parametrize("n", [1, 2, 4, 6, 8, 16])
@pytest.mark.parametrize("k,nT", [(6, 31), (5, 31), (5, 40)])
def test_tensor_core_paths(k, nT, n):
    """Five- and six-spin clusters in mixed mode run on tcgen05 (FP16 hi/lo,
    FP32 accumulate; five-spin clusters two time points per product, so time
    slices of odd and even length), Hahn and CPMG-2 to CPMG-16 (chains of up
    to 17 segments).  The mixed-precision error of a cluster
    scales with sqrt(1 - L_C): clusters that stay within 1 % of full coherence
    must be within 1e-6 of the FP64 path, strongly decohering ones within
    1e-5."""
    coords, pick = _clusters_of(k, 24, seed=300 + n)
    B = configs.tilted_field(0.1, 3.0, 1.1)
    _, sv = cce.nv_states(B)
    p = cce.CCEParams.make(B, sv[0], sv[1], n, nT, 8e-3 / (nT - 1))
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    L64 = cce.cluster_coherence(cd, cl, k, p, cce.PREC_FP64).cpu().numpy()
    Ltc = cce.cluster_coherence(cd, cl, k, p, cce.PREC_MIXED).cpu().numpy()
    Lsimt = cce.cluster_coherence(cd, cl, k, p, cce.PREC_MIXED_SIMT).cpu().numpy()
    assert np.all(Ltc[:, 0] == 1.0)
    weak = L64.min(axis=1) >= 0.99
    for L in (Ltc, Lsimt):
        err = np.abs(L - L64).max(axis=1)
        assert np.all(err[weak] <= 1e-6), err[weak].max()
        assert np.all(err <= 1e-5), err.max()


@pytest.mark.parametrize("precision", [cce.PREC_FP64, cce.PREC_MIXED])
def test_graph_replay_matches_direct_run(precision):
    """oops_cce_graph_*: the captured run replayed twice gives the direct
    device-resident run's curves (every size class, the reduction)."""
    w = configs.cce4_hahn()
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, 61, w.t_max / 60)
    run = cce.DeviceRun(w.coords, w.cutoff, 4, p, precision)
    ref = run.step().clone()
    ref_L = [x.clone() for x in run.L]
    run.make_graph()
    for _ in range(2):
        for x in run.L:
            x.fill_(float("nan"))
        run.cum.fill_(float("nan"))
        got = run.step_graph()
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        assert (got - ref).abs().max().item() <= 1e-12
        for a, b in zip(run.L, ref_L):
            assert (a - b).abs().max().item() <= 1e-12
    run.close_graph()


@pytest.mark.parametrize("k", [4, 6])
def test_fp64_correction_options(k):
    """oops_cce_params.fp64_max_k >= k runs the whole class in FP64 (the FP64
    path's result); fp64_below above every L_C recomputes every cluster in
    FP64 from the same FP64 eigenbasis (the FP64 path's result up to the
    eigensolver's rounding)."""
    w = configs.cce6_cpmg8() if k == 6 else configs.cce4_hahn()
    cl = cce.Clusters(w.coords, w.cutoff, k)
    rows = cl.clusters(k - 1)[:24]
    _, sv = cce.nv_states(w.B)
    coords = torch.from_numpy(w.coords).cuda()
    idx = torch.from_numpy(rows.astype(np.int32)).cuda()
    nT, dt = 41, w.t_max / 40
    mk = lambda **kw: cce.CCEParams.make(w.B, sv[0], sv[1], w.pulse_num, nT, dt, **kw)
    ref = cce.cluster_coherence(coords, idx, k, mk(), cce.PREC_FP64).cpu().numpy()
    whole = cce.cluster_coherence(coords, idx, k, mk(fp64_max_k=k), cce.PREC_MIXED).cpu().numpy()
    assert np.abs(whole - ref).max() <= 1e-12
    corr = cce.cluster_coherence(coords, idx, k, mk(fp64_below=2.0), cce.PREC_MIXED).cpu().numpy()
    assert np.abs(corr - ref).max() <= 1e-10
    mixed = cce.cluster_coherence(coords, idx, k, mk(), cce.PREC_MIXED).cpu().numpy()
    assert np.abs(mixed - ref).max() <= 1e-5
