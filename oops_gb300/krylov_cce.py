"""Cluster coherence through the plain FP64 Krylov drop-in (the baseline the
batched dense path is measured against).

L_C(t_i) = (1/D) Re Tr[B1(t_i)^+ B0(t_i)], with B0 = U0(s0 t) U1(s1 t) ...
U_{a_n}(s_n t) and B1 the same with 0 <-> 1 (the riffle of the reference's
PiecewiseFullMatrixVectorEvolution, QuantumEvolutionAlgorithm.cpp:60-83,
ensemble_cce.cpp:33-55).  The reference builds every segment propagator of
one time step with a dense Pade exponential and advances it one product per
time step (E_j^i = E_j E_j^{i-1}, QuantumEvolutionAlgorithm.cpp:73-80).  Here
the one-step propagator of every distinct segment -- H_0 or H_1 over a half
or a full pulse interval of one time step, exp(-i H_a s dt) -- comes from the
Krylov expv (oops_expv_block, the main_cache_ algorithm, FP64) applied to the
2^k basis states, and the powers and chains are FP64 products (batched
complex128 GEMMs, one per time step as in the reference).  A Hahn echo needs
two one-step propagators per cluster, CPMG-n four.  The Krylov step count of
one interval depends on the Krylov dimension the drop-in allows (m < 2^k):
3-19 steps at k >= 4, several hundred at k = 3 (m <= 7), about 10^6 at
k = 2 (m <= 3), so clusters of one and two spins are out of its reach.
"""
from __future__ import annotations

import time

import numpy as np

from .expv import Hamiltonian, expv_block
from .spin import cluster_terms


def cpmg_fractions(n):
    prev, out = 0.0, []
    for i in range(n):
        t = (2.0 * i + 1.0) / (2.0 * n)
        out.append(t - prev)
        prev = t
    out.append(1.0 - prev)
    return np.array(out)


def segment_plan(pulse_num):
    """Per branch the (Hamiltonian index, fraction key) of every segment, the
    first segment leftmost in the product; and the distinct keys."""
    frac = cpmg_fractions(pulse_num)
    keys = [round(float(f), 15) for f in frac]
    nseg = pulse_num + 1
    plan = {br: [((j + br) & 1, keys[j]) for j in range(nseg)] for br in (0, 1)}
    need = sorted({x for br in (0, 1) for x in plan[br]})
    return plan, need


def chain_coherence(G, pulse_num, nT):
    """L_C(t_i), i < nT, from the one-step propagators G[j] (complex128, any
    torch device) of the distinct segments, in segment_plan's `need` order:
    P[i] = G^i by one batched product per time step, then each branch's chain
    of segment powers and L = (1/D) Re Tr[B1^+ B0]."""
    import torch
    plan, need = segment_plan(pulse_num)
    slot = {key: i for i, key in enumerate(need)}
    D = G.shape[-1]
    P = torch.empty((nT, len(need), D, D), dtype=G.dtype, device=G.device)
    P[0] = torch.eye(D, dtype=G.dtype, device=G.device)
    for i in range(1, nT):
        torch.bmm(G, P[i - 1], out=P[i])
    Bm = {}
    for br in (0, 1):
        X = P[:, slot[plan[br][0]]]
        for key in plan[br][1:]:
            X = torch.bmm(X, P[:, slot[key]])
        Bm[br] = X
    L = (torch.conj(Bm[1]) * Bm[0]).real.sum(dim=(1, 2)) / D
    return L.cpu().numpy()


def cluster_coherence_krylov(coords, B, sv, pulse_num, nT, dt, m=None, tol=1e-12, k_lanczos=10,
                             deadline=None, timings=None):
    """L_C(t_i), t_i = i dt for i < nT, of one cluster by the Krylov drop-in.
    deadline: optional time.perf_counter() value checked between the Krylov
    calls.  timings: optional dict receiving the seconds spent in the Krylov
    calls ("krylov_s"), in the powers and chain products ("products_s") and
    the drop-in's step count summed over the calls ("krylov_steps").  m:
    Krylov dimension; None takes the autotuner's cached choice for this size
    (oops_gb300.tune.krylov_m), else 30; it is capped at 2^k - 1."""
    import torch
    coords = np.asarray(coords, float).reshape(-1, 3)
    k = coords.shape[0]
    D = 1 << k
    if m is None:
        from .tune import krylov_m
        mm = krylov_m(D, D)
    else:
        mm = max(1, min(m, D - 1))
    H = [Hamiltonian(cluster_terms(coords, B, np.zeros(3), sv[s])) for s in (0, 1)]
    _, need = segment_plan(pulse_num)
    eye = torch.eye(D, dtype=torch.complex128, device="cuda").contiguous()
    t0 = time.perf_counter()
    steps = 0
    G = torch.empty((len(need), D, D), dtype=torch.complex128, device="cuda")
    try:
        for j, (a, f) in enumerate(need):
            if deadline is not None and time.perf_counter() > deadline:
                raise TimeoutError("plain Krylov sample exceeded its time budget")
            # column b of W[0] = exp(-i H_a f dt) e_b: the one-step propagator
            W, st = expv_block(H[a], eye, np.full((1, D), f * dt), m=mm, tol=tol, k=k_lanczos)
            G[j] = W[0]
            steps += int(st.nstep)
    finally:
        for h in H:
            h.close()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    out = chain_coherence(G, pulse_num, nT)
    t2 = time.perf_counter()
    if timings is not None:
        timings["krylov_s"] = t1 - t0
        timings["products_s"] = t2 - t1
        timings["krylov_steps"] = steps
    return out
