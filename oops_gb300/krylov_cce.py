"""Cluster coherence through the plain FP64 Krylov drop-in (the baseline the
batched dense path is measured against).

L_C(t_i) = (1/D) Re Tr[B1(t_i)^+ B0(t_i)], with B0 = U0(s0 t) U1(s1 t) ...
U_{a_n}(s_n t) and B1 the same with 0 <-> 1 (the riffle of the reference's
PiecewiseFullMatrixVectorEvolution, QuantumEvolutionAlgorithm.cpp:60-83,
ensemble_cce.cpp:33-55).  The reference builds every segment propagator with
a dense Pade exponential and powers of it (U_j^i, one product per time step);
here every distinct segment propagator U_a(s t_i) -- H_0 or H_1 over a half
or a full pulse interval -- comes from the Krylov expv (oops_expv_block, the
main_cache_ algorithm, FP64) applied to the 2^k basis states along ONE
trajectory that outputs at every s t_i, and the chains are FP64 products of
those propagators (batched complex128 GEMMs).  A Hahn echo needs two
trajectories per cluster, CPMG-n four.  The Krylov part's cost grows with
||H|| t_max (its step size is bounded by the Krylov dimension), which is
why it is far slower than the eigenbasis form for clusters of up to 64
states.
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


def cluster_coherence_krylov(coords, B, sv, pulse_num, nT, dt, m=None, tol=1e-12, k_lanczos=10,
                             t_scale=1.0, deadline=None, timings=None):
    """L_C(t_i), i < nT, t_i = i dt t_scale, of one cluster by the Krylov
    drop-in.  t_scale < 1 propagates over a prefix of the grid (bounded
    sampling: the trajectory cost is proportional to the time covered).
    deadline: optional time.perf_counter() value checked between trajectories.
    timings: optional dict receiving the seconds spent in trajectories and in
    the chain products.  m: Krylov dimension; None takes the autotuner's
    cached choice for this size (oops_gb300.tune.krylov_m), else 30."""
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
    plan, need = segment_plan(pulse_num)
    t = dt * t_scale * np.arange(nT)
    eye = torch.eye(D, dtype=torch.complex128, device="cuda").contiguous()
    U = {}
    t0 = time.perf_counter()
    for a, f in need:
        if deadline is not None and time.perf_counter() > deadline:
            raise TimeoutError("plain Krylov sample exceeded its time budget")
        W, _ = expv_block(H[a], eye, np.repeat((f * t)[:, None], D, axis=1), m=mm, tol=tol,
                          k=k_lanczos)
        U[(a, f)] = W  # (nT, D, D): W[i] = U_a(f t_i)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    Bm = {}
    for br in (0, 1):
        P = U[plan[br][0]]
        for key in plan[br][1:]:
            P = torch.bmm(P, U[key])
        Bm[br] = P
    L = (torch.conj(Bm[1]) * Bm[0]).real.sum(dim=(1, 2)) / D
    out = L.cpu().numpy()
    t2 = time.perf_counter()
    for h in H:
        h.close()
    if timings is not None:
        timings["trajectories_s"] = t1 - t0
        timings["products_s"] = t2 - t1
    return out
