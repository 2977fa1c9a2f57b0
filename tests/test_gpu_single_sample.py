"""GPU parity of single-sample CCE (oops_cce_coherence_state /
oops_single_sample_cce; SingleSampleCCE, src/source/app/single_sample_cce.cpp)
against the CPU oracle: cluster Hamiltonians with the mean dipolar field of
the bath spins outside the cluster (pyoracle.bath_field), and the
reference's state propagation restated in orc_coherence_state (pinned
against scipy in test_oracle.py, and with the bath field and the reduction
against whole runs of the reference's own SingleSampleCCE in
test_reference_pins.py).  Tolerances: FP64 1e-10, mixed precision
1e-6 absolute on every L_C(t_i); whole-run L(t) 1e-8 (FP64)."""
import numpy as np
import pytest

import pyoracle as po
from helpers import SX, SY, SZ

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import cce, configs  # noqa: E402

B0 = 0.05 * configs.NV_AXIS


def _dense_h(coords, idx, B, sv, field):
    k = len(idx)
    H = po.dense_hamiltonian(po.cluster_hamiltonian(coords[list(idx)], B, np.zeros(3), sv))
    for s in range(k):
        for a, S in enumerate((SX, SY, SZ)):
            H = H + field[s, a] * np.kron(np.kron(np.eye(2 ** s), S), np.eye(2 ** (k - 1 - s)))
    return H


def _oracle(coords, state, idx, B, sv, n, nT, dt):
    f = po.bath_field(coords, state, idx)
    H0, H1 = (_dense_h(coords, idx, B, sv[s], f) for s in (0, 1))
    b = 0
    for s, j in enumerate(idx):
        b |= int(state[j]) << (len(idx) - 1 - s)
    return po.coherence_state(H0, H1, n, nT, dt, b)


def _pick(k, count, seed):
    w = configs.cce6_cpmg8(seed) if k > 2 else configs.cce4_hahn(seed)
    cl = cce.Clusters(w.coords, 7.0, k)
    rows = cl.clusters(k - 1)
    rng = np.random.default_rng(seed)
    return w.coords, rows[rng.choice(len(rows), size=min(count, len(rows)), replace=False)]


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("n", [1, 2, 8])
def test_single_sample_coherence_fp64_and_mixed(k, n):
    coords, pick = _pick(k, 3 if k >= 5 else 5, seed=1200 + k)
    state = cce.bath_state_from_seed(17 + k, len(coords))
    B = configs.tilted_field(0.1, 3.0, 0.7) if n == 8 else B0
    _, sv = cce.nv_states(B)
    nT, dt = (13, 4e-4) if k == 6 else (21, 2e-4)
    p = cce.CCEParams.make(B, sv[0], sv[1], n, nT, dt)
    cd = torch.from_numpy(coords).cuda()
    sd = torch.from_numpy(state).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    L64 = cce.cluster_coherence_state(cd, sd, cl, k, p, cce.PREC_FP64).cpu().numpy()
    Lmp = cce.cluster_coherence_state(cd, sd, cl, k, p, cce.PREC_MIXED).cpu().numpy()
    for c in range(len(pick)):
        ref = _oracle(coords, state, pick[c], B, sv, n, nT, dt)
        assert np.abs(L64[c] - ref).max() <= 1e-10, (c, np.abs(L64[c] - ref).max())
        assert np.abs(Lmp[c] - ref).max() <= 1e-6, (c, np.abs(Lmp[c] - ref).max())


def test_single_sample_differs_from_ensemble_and_depends_on_the_state():
    coords, pick = _pick(3, 4, seed=1301)
    _, sv = cce.nv_states(B0)
    p = cce.CCEParams.make(B0, sv[0], sv[1], 1, 41, 1e-4)
    cd = torch.from_numpy(coords).cuda()
    cl = torch.from_numpy(pick.astype(np.int32)).cuda()
    La = cce.cluster_coherence_state(cd, torch.from_numpy(cce.bath_state_from_seed(1, len(coords))).cuda(),
                                     cl, 3, p).cpu().numpy()
    Lb = cce.cluster_coherence_state(cd, torch.from_numpy(cce.bath_state_from_seed(2, len(coords))).cuda(),
                                     cl, 3, p).cpu().numpy()
    Le = cce.cluster_coherence(cd, cl, 3, p, cce.PREC_FP64).cpu().numpy()
    assert np.abs(La[:, 0] - 1.0).max() <= 1e-13
    assert np.abs(La).max() <= 1 + 1e-12
    assert np.abs(La - Lb).max() > 1e-8
    assert np.abs(La - Le).max() > 1e-8


def test_single_sample_cce_run_matches_oracle_pipeline():
    w = configs.cce2_hahn()
    nT, dt, order = 21, 1e-4, 3
    state = cce.bath_state_from_seed(2024, len(w.coords))
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, nT, dt)
    cum, each, counts, per = cce.single_sample_cce(w.coords, state, w.cutoff, order, p,
                                                   want_clusters=True)
    e = po.Enumeration(w.coords, w.cutoff, order)
    Lraw = []
    for o in range(order):
        rows = e.clusters(o)
        assert counts[o] == len(rows)
        Lo = np.stack([_oracle(w.coords, state, r, w.B, sv, 1, nT, dt) for r in rows], axis=1)
        assert np.abs(per[o] - Lo.T).max() <= 1e-10
        Lraw.append(Lo)
    _, each_o, cum_o = e.reduce(Lraw, nT)
    assert np.abs(cum - cum_o).max() <= 1e-8
    assert np.abs(each - each_o).max() <= 1e-8


def test_single_sample_device_run_equals_host_run():
    w = configs.cce4_hahn()
    state = cce.bath_state_from_seed(99, len(w.coords))
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, 41, 1e-4)
    for prec in (cce.PREC_FP64, cce.PREC_MIXED):
        run = cce.DeviceRun(w.coords, w.cutoff, 3, p, prec, state=state)
        dev = run.step().cpu().numpy().T
        host = cce.single_sample_cce(w.coords, state, w.cutoff, 3, p, prec)[0]
        assert np.array_equal(dev, host)
