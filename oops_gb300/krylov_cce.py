"""Cluster coherence through the plain FP64 Krylov drop-in (the baseline the
batched dense path is measured against).

L_C(t_i) = (1/D) sum_c Re < B1(t_i) e_c, B0(t_i) e_c >, with
B0 = U0(s0 t) U1(s1 t) ... U_{a_n}(s_n t) and B1 the same with 0 <-> 1, every
factor applied to vectors with the Krylov expv (oops_expv_block, the
main_cache_ algorithm): the innermost segment for all time points in one
call, then every (time point, basis state) column with its own time.  This is
how the reference's MatExpVector (src/source/math/MatExp.cpp:139-160) would
propagate a cluster's 2^k basis states through the pulse sequence; it is far
slower than the dense path for small clusters, which is why the dense path
exists.
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


def cluster_coherence_krylov(coords, B, sv, pulse_num, nT, dt, m=30, tol=1e-12, k_lanczos=10,
                             deadline=None):
    """deadline: optional time.perf_counter() value after which the next block
    call raises TimeoutError (bounded sampling)."""
    import torch
    coords = np.asarray(coords, float).reshape(-1, 3)
    k = coords.shape[0]
    D = 1 << k
    mm = max(1, min(m, D - 1))
    H = [Hamiltonian(cluster_terms(coords, B, np.zeros(3), sv[s])) for s in (0, 1)]
    frac = cpmg_fractions(pulse_num)
    nseg = pulse_num + 1
    t = dt * np.arange(nT)
    out = {}
    for br in (0, 1):
        # innermost (last) segment for every time point: D columns, nT times
        a = (nseg - 1 + br) & 1
        V = torch.eye(D, dtype=torch.complex128, device="cuda").contiguous()
        W, _ = expv_block(H[a], V, np.repeat((frac[-1] * t)[:, None], D, axis=1), m=mm, tol=tol,
                          k=k_lanczos)
        cols = W.permute(1, 0, 2).reshape(D, nT * D).contiguous()  # column (i, c)
        times_i = np.repeat(t, D)
        for j in range(nseg - 2, -1, -1):
            a = (j + br) & 1
            nxt = torch.empty_like(cols)
            for c0 in range(0, nT * D, 256):
                if deadline is not None and time.perf_counter() > deadline:
                    raise TimeoutError("plain Krylov sample exceeded its time budget")
                c1 = min(nT * D, c0 + 256)
                blk = cols[:, c0:c1].contiguous()
                Wj, _ = expv_block(H[a], blk, (frac[j] * times_i[c0:c1])[None, :], m=mm, tol=tol,
                                   k=k_lanczos)
                nxt[:, c0:c1] = Wj[0]
            cols = nxt
        out[br] = cols.reshape(D, nT, D)
    # L_i = (1/D) sum_c Re <B1 e_c, B0 e_c>
    L = (torch.conj(out[1]) * out[0]).real.sum(dim=(0, 2)) / D
    return L.cpu().numpy()
