"""Spin Hamiltonians as Kronecker term lists (host side).

Builds the SumKronProd the reference's EnsembleCCE::create_spin_hamiltonian
produces (src/source/app/ensemble_cce.cpp:57-71): SpinDipolarInteraction
(every pair i<j, components xx..zz), SpinZeemanInteraction (-gamma B_a per
spin; the quadrupole terms vanish for 13C) and DipolarField (the NV's
mean field D.<S> on every spin), each term emitted only when its coefficient
is non-zero (cSpinInteraction::make, src/source/spin/SpinInteraction/
SpinInteraction.cpp:29-65).  Physics helpers restate misc.cpp:11-57.
"""
from __future__ import annotations

import numpy as np

from .expv import KronTerms

HBAR = 1.054571800e-34
MU0 = 1.2566370614e-06
GAMMA_C13 = 6.728284e7
GAMMA_NVE = -1.760859708e11

SX = 0.5 * np.array([[0, 1], [1, 0]], np.complex128)
SY = 0.5 * np.array([[0, -1j], [1j, 0]], np.complex128)
SZ = 0.5 * np.array([[1, 0], [0, -1]], np.complex128)
SPIN_HALF = (SX, SY, SZ)


def dipole(c1, c2, g1, g2):
    """misc.cpp:11-36: 3x3 tensor hbar mu0/4pi g1 g2 / r^3 (1 - 3 n n), r in A."""
    r = np.asarray(c1, float) - np.asarray(c2, float)
    d = np.sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])
    if d <= 1e-10:
        return np.zeros((3, 3))
    n = r / d
    d0 = d * 1e-10
    pre = HBAR * MU0 / (4.0 * np.pi) * (g1 * g2) / (d0 * d0 * d0)
    return pre * (np.eye(3) - 3.0 * np.outer(n, n))


def cluster_terms(coords, B, center, sv, g=GAMMA_C13, gc=GAMMA_NVE) -> KronTerms:
    """Term list of one NV-conditional cluster Hamiltonian (spin 0 most
    significant), in the reference's term order."""
    coords = np.asarray(coords, float).reshape(-1, 3)
    k = coords.shape[0]
    terms = []
    for i in range(k):
        for j in range(i + 1, k):
            D = dipole(coords[i], coords[j], g, g)
            for a in range(3):
                for b in range(3):
                    if D[a, b] != 0.0:
                        terms.append((D[a, b], [(i, SPIN_HALF[a]), (j, SPIN_HALF[b])]))
    for i in range(k):
        for a in range(3):
            c = -g * B[a]
            if c != 0.0:
                terms.append((c, [(i, SPIN_HALF[a])]))
    for i in range(k):
        D = dipole(coords[i], center, g, gc)
        f = D.T @ np.asarray(sv, float)
        for a in range(3):
            if f[a] != 0.0:
                terms.append((f[a], [(i, SPIN_HALF[a])]))
    return from_list([2] * k, terms)


def from_list(spin_dim, terms) -> KronTerms:
    coeff, nbody, pos, dims, mats, moff = [], [], [], [], [], [0]
    for c, bodies in terms:
        coeff.append(float(c))
        nbody.append(len(bodies))
        for p, M in bodies:
            M = np.asarray(M, np.complex128)
            pos.append(int(p))
            dims.append(M.shape[0])
            mats.append(M.reshape(-1, order="F"))
            moff.append(moff[-1] + M.size)
    poff = np.concatenate([[0], np.cumsum(nbody)]).astype(np.uint64)
    return KronTerms(np.asarray(coeff, np.float64), np.asarray(nbody, np.uint64), poff,
                     np.asarray(pos, np.uint64), np.asarray(dims, np.uint64),
                     np.asarray(moff, np.uint64),
                     np.concatenate(mats) if mats else np.zeros(0, np.complex128),
                     np.asarray(spin_dim, np.uint64))
