"""Shared test utilities: random term lists and small numpy restatements."""
import numpy as np

from pyoracle import KronTerms

SX = 0.5 * np.array([[0, 1], [1, 0]], np.complex128)
SY = 0.5 * np.array([[0, -1j], [1j, 0]], np.complex128)
SZ = 0.5 * np.array([[1, 0], [0, -1]], np.complex128)
S1X = np.array([[0, 1, 0], [1, 0, 1], [0, 1, 0]], np.complex128) / np.sqrt(2)
S1Y = np.array([[0, -1j, 0], [1j, 0, -1j], [0, 1j, 0]], np.complex128) / np.sqrt(2)
S1Z = np.diag([1.0, 0.0, -1.0]).astype(np.complex128)


def ops_for(d):
    return (SX, SY, SZ) if d == 2 else (S1X, S1Y, S1Z)


def random_terms(rng, spin_dim, n_single=None, n_pair=None, scale=1.0, hermitian=True):
    """A random Hamiltonian in the reference's term format: one- and two-body
    spin-operator products with real coefficients (as SpinInteraction emits)."""
    k = len(spin_dim)
    terms = []
    n_single = k * 3 if n_single is None else n_single
    n_pair = (k * (k - 1) // 2) * 3 if n_pair is None else n_pair
    for _ in range(n_single):
        i = int(rng.integers(k))
        a = int(rng.integers(3))
        terms.append((scale * rng.normal(), [(i, ops_for(spin_dim[i])[a])]))
    if k > 1:
        for _ in range(n_pair):
            i, j = sorted(rng.choice(k, 2, replace=False).tolist())
            a, b = int(rng.integers(3)), int(rng.integers(3))
            terms.append((scale * rng.normal(), [(i, ops_for(spin_dim[i])[a]),
                                                 (j, ops_for(spin_dim[j])[b])]))
    return KronTerms.from_list(spin_dim, terms)


def dense_from_terms(t: KronTerms):
    """numpy Kronecker construction of sum_t c_t (x) bodies (spin 0 most
    significant), independent of the oracle's matvec."""
    dims = [int(d) for d in t.spin_dim]
    D = int(np.prod(dims))
    H = np.zeros((D, D), np.complex128)
    for ti in range(t.nterm):
        facs = [np.eye(d, dtype=np.complex128) for d in dims]
        a, b = int(t.pos_offset[ti]), int(t.pos_offset[ti + 1])
        for q in range(a, b):
            d = int(t.dim_list[q])
            mo = int(t.mat_offset[q])
            facs[int(t.pos_list[q])] = t.mats[mo:mo + d * d].reshape(d, d, order="F")
        M = facs[0]
        for f in facs[1:]:
            M = np.kron(M, f)
        H += t.coeff[ti] * M
    return H
