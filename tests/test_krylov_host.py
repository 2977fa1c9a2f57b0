"""Host logic of the plain FP64 Krylov cluster path (oops_gb300/krylov_cce.py)
on the CPU: given exact one-step propagators of its distinct segments, the
segment plan, the powers and the chains give the oracle's dense Hilbert-space
coherence (orc_coherence_hilbert, the reference's piecewise propagation,
QuantumEvolutionAlgorithm.cpp:60-83, ensemble_cce.cpp:33-55).  The GPU test
(tests/test_gpu_cce.py) then only has to show the drop-in's propagators."""
import numpy as np
import pytest
import scipy.linalg as sla
import torch

import pyoracle as po
from oops_gb300 import configs
from oops_gb300.krylov_cce import chain_coherence, cpmg_fractions, segment_plan


def test_segment_plan_covers_each_branch():
    """Branch 0 starts on H_0 and branch 1 on H_1, alternating at every
    pulse; the segment fractions are the oracle's CPMG intervals and sum
    to one."""
    for n in (1, 2, 3, 8, 16):
        f = cpmg_fractions(n)
        assert np.allclose(f, po.cpmg_intervals(n), rtol=0, atol=1e-15)
        assert abs(f.sum() - 1.0) < 1e-14
        plan, need = segment_plan(n)
        for br in (0, 1):
            assert len(plan[br]) == n + 1
            assert [a for a, _ in plan[br]] == [(j + br) & 1 for j in range(n + 1)]
            assert set(plan[br]) <= set(need)
        # Hahn: two distinct segments; CPMG-n (n > 1): half and full intervals on both Hamiltonians
        assert len(need) == (2 if n == 1 else 4)


@pytest.mark.parametrize("k,n,nT", [(1, 1, 7), (2, 1, 9), (3, 2, 11), (3, 8, 6), (4, 16, 5)])
def test_chain_coherence_matches_oracle(k, n, nT):
    """One-step propagators exp(-i H_a f dt) from scipy's expm of the oracle's
    dense Hamiltonians: the chains match orc_coherence_hilbert to 1e-10 (the
    FP64 parity tolerance; the two exponentials -- scipy's and the oracle's
    Pade restatement -- differ by rounding that the squarings amplify with
    ||H f dt||, a few hundred here, and the powers accumulate: 3e-12 at
    most on these cases)."""
    w = configs.cce4_hahn()
    B = configs.tilted_field(0.1, 3.0, 1.1)
    _, sv = po.nv_states(B)
    idx = po.Enumeration(w.coords, 6.0, k).clusters(k - 1)[3]
    coords = w.coords[list(idx)]
    H = [po.dense_hamiltonian(po.cluster_hamiltonian(coords, B, np.zeros(3), sv[s])) for s in (0, 1)]
    dt = 1.6e-3 / (nT - 1)
    _, need = segment_plan(n)
    G = torch.from_numpy(np.stack([sla.expm(-1j * H[a] * f * dt) for a, f in need]))
    L = chain_coherence(G, n, nT)
    Lo = po.coherence_hilbert(H[0], H[1], n, nT, dt)
    assert L[0] == pytest.approx(1.0, abs=1e-14)
    assert np.abs(L - Lo).max() <= 1e-10
