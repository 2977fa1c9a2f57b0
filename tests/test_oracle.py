"""Pins for the CPU oracle (oracle/oracle.c) before it is trusted as checker.

The reference ships no golden vectors or tests, so the pins here are: the
reference's own Kronecker matvec compiled from its source (oracle/_ref),
scipy's expm / expm_multiply, a big-integer restatement of the LAPACK
generator, numpy restatements of the spin physics, and a brute-force
enumerator.  The pins on the reference's own enumeration, physics,
reduction, spin source, whole ensemble and single-sample runs, result file
and Krylov arguments are in test_reference_pins.py, test_app_classes.py and
test_matfile.py.
"""
import itertools
import os

import numpy as np
import pytest
import scipy.linalg as sla

import pyoracle as po
from helpers import SX, SY, SZ, dense_from_terms, random_terms


# ---------------------------------------------------------------- DLARAN
def _dlaran_fortran_steps(iseed):
    """The integer steps of DLARAN.f:62-85, in Python integers."""
    M1, M2, M3, M4, IPW2 = 494, 322, 2508, 2549, 4096
    it4 = iseed[3] * M4
    it3 = it4 // IPW2
    it4 -= IPW2 * it3
    it3 += iseed[2] * M4 + iseed[3] * M3
    it2 = it3 // IPW2
    it3 -= IPW2 * it2
    it2 += iseed[1] * M4 + iseed[2] * M3 + iseed[3] * M2
    it1 = it2 // IPW2
    it2 -= IPW2 * it1
    it1 += iseed[0] * M4 + iseed[1] * M3 + iseed[2] * M2 + iseed[3] * M1
    it1 %= IPW2
    r = 1.0 / IPW2
    val = r * (it1 + r * (it2 + r * (it3 + r * it4)))
    return [it1, it2, it3, it4], val


def test_dlaran_matches_fortran_integer_steps():
    seq, final = po.dlaran_sequence(5000)
    s = [0, 0, 0, 5]
    for k in range(5000):
        s, val = _dlaran_fortran_steps(s)
        assert val == seq[k]
    assert tuple(s) == final
    assert np.all((seq > 0) & (seq < 1))


# ---------------------------------------------------------------- matvec
@pytest.mark.parametrize("dims", [(2,), (2, 2), (2, 2, 2, 2, 2), (3, 2, 2), (2, 3, 2, 3)])
def test_hamvec_matches_dense_kron(dims):
    rng = np.random.default_rng(1 + len(dims))
    t = random_terms(rng, list(dims))
    H = dense_from_terms(t)
    v = rng.normal(size=H.shape[0]) + 1j * rng.normal(size=H.shape[0])
    w = po.hamvec(t, v)
    np.testing.assert_allclose(w, H @ v, rtol=0, atol=1e-12 * np.abs(H @ v).max())


@pytest.mark.parametrize("dims", [(2, 2, 2, 2, 2, 2), (3, 2, 2), (2, 3, 2, 3)])
def test_hamvec_bit_exact_vs_reference_source(dims):
    """oracle/_ref is the reference's own hamvec_func3.cpp compiled here."""
    if po.ref_lib() is None:
        pytest.skip("reference matvec not built (reference tree absent)")
    rng = np.random.default_rng(7)
    t = random_terms(rng, list(dims))
    D = t.dim
    v = rng.normal(size=D) + 1j * rng.normal(size=D)
    cz = -1j * t.coeff
    ours = po.hamvec(t, v, cz)
    ref = po.ref_hamvec(t, v, cz)
    assert np.array_equal(ours.view(np.float64), ref.view(np.float64))


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hamvec_reference.npz")


def _golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    return g, names


@pytest.mark.parametrize("name", _golden_cases()[1])
def test_hamvec_bit_exact_vs_reference_golden(name):
    """Golden outputs of the reference's own hamvec_func3.cpp (made by
    tests/golden/make_golden.py from the reference tree): the oracle's
    matvec reproduces them bit for bit without the reference present."""
    g, _ = _golden_cases()
    t = po.KronTerms(*(g[f"{name}/{f}"] for f in ("coeff", "nbody", "pos_offset", "pos_list",
                                                   "dim_list", "mat_offset", "mats", "spin_dim")))
    v = g[f"{name}/v"]
    ours = po.hamvec(t, v, -1j * t.coeff)
    assert np.array_equal(ours.view(np.float64), g[f"{name}/w_ref"].view(np.float64))


# ---------------------------------------------------------------- Pade
@pytest.mark.parametrize("m,scale", [(1, 0.3), (4, 0.01), (8, 1.0), (16, 20.0), (52, 3.0)])
def test_padm_matches_scipy_expm(m, scale):
    rng = np.random.default_rng(m)
    A = scale * (rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))) / np.sqrt(m)
    E, ns = po.padm(A, 1.0)
    ref = sla.expm(A)
    assert np.linalg.norm(E - ref) <= 1e-12 * max(1.0, np.linalg.norm(ref)) * max(1, 2 ** ns)


def test_padm_time_scale_and_unitarity():
    rng = np.random.default_rng(3)
    Hh = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    Hh = Hh + Hh.conj().T
    E, _ = po.padm(-1j * Hh, 0.7)
    np.testing.assert_allclose(E @ E.conj().T, np.eye(6), atol=1e-12)
    np.testing.assert_allclose(E, sla.expm(-0.7j * Hh), atol=1e-12)


def test_padm_null_matrix_is_an_error():
    with pytest.raises(RuntimeError):
        po.padm(np.zeros((3, 3)), 1.0)


# ---------------------------------------------------------------- Krylov
@pytest.mark.parametrize("dims,m", [((2,) * 6, 30), ((2,) * 7, 20), ((3, 2, 2, 2), 10),
                                    ((2,) * 5, 8)])
def test_expv_matches_dense_exponential(dims, m):
    rng = np.random.default_rng(len(dims) * 10 + m)
    t = random_terms(rng, list(dims), scale=2e4)
    H = dense_from_terms(t)
    D = H.shape[0]
    v = rng.normal(size=D) + 1j * rng.normal(size=D)
    v /= np.linalg.norm(v)
    tl = np.array([1e-5, 3e-5, 3e-5, 2e-4, 5e-4])
    W, st = po.expv(t, v, tl, m=m, tol=1e-12)
    assert st.iflag == 0 and st.nstep > 0
    for i, tt in enumerate(tl):
        ref = sla.expm(-1j * H * tt) @ v
        assert np.linalg.norm(W[:, i] - ref) <= 1e-10 * np.linalg.norm(ref)


def _liouvillian_terms(k, seed, rate_hz=1e4):
    """A dephasing Liouvillian in the reference's per-spin Liouville form
    (KronProd with 4-dimensional sites: SHARP(H_0) - FLAT(H_1) + i g
    (sigma^T (x) sigma - 1) per spin; KronProd.cpp:84-107,
    SpinInteractionComponent.cpp:285-304): the non-Hermitian operator the
    reference's MatExpTest.cpp cross-checks its Krylov paths on."""
    rng = np.random.default_rng(seed)
    coords = rng.normal(size=(k, 3)) * 4.0 + 5.0
    B = np.array([0.0, 0.0, 0.05])
    _, sv = po.nv_states(B)
    I2 = np.eye(2)
    sharp = lambda S: np.kron(S.T, I2)   # rho S
    flat = lambda S: np.kron(I2, S)      # S rho
    terms = []
    for s_idx, sign, f in ((0, 1.0, sharp), (1, -1.0, flat)):
        t = po.cluster_hamiltonian(coords, B, np.zeros(3), sv[s_idx])
        for ti in range(t.nterm):
            bodies = []
            for q in range(int(t.pos_offset[ti]), int(t.pos_offset[ti + 1])):
                mo = int(t.mat_offset[q])
                S = t.mats[mo:mo + 4].reshape(2, 2, order="F")
                bodies.append((int(t.pos_list[q]), f(S)))
            terms.append((sign * float(t.coeff[ti]), bodies))
    nx, ny, nz = np.ones(3) / np.sqrt(3.0)
    sig = np.array([[nz, nx - 1j * ny], [nx + 1j * ny, -nz]])
    deph = 1j * (np.kron(sig.T, sig) - np.eye(4))
    for s_idx in range(k):
        terms.append((2 * np.pi * rate_hz, [(s_idx, deph)]))
    return po.KronTerms.from_list([4] * k, terms)


@pytest.mark.parametrize("k", [2, 3])
def test_expv_on_dephasing_liouvillian_matches_dense_exponential(k):
    """The Krylov driver (Arnoldi, not Lanczos) on a non-Hermitian operator with
    4-dimensional sites, against scipy's dense exponential."""
    t = _liouvillian_terms(k, 500 + k)
    L = dense_from_terms(t)
    assert np.abs(L - L.conj().T).max() > 1e3          # non-Hermitian
    rng = np.random.default_rng(k)
    v = rng.normal(size=L.shape[0]) + 1j * rng.normal(size=L.shape[0])
    v /= np.linalg.norm(v)
    tl = np.array([1e-6, 5e-6, 2e-5])   # g t up to ~1.3: the state decays, not vanishes
    W, st = po.expv(t, v, tl, m=min(30, L.shape[0] - 2), tol=1e-12)
    assert st.iflag == 0
    for i, tt in enumerate(tl):
        ref = sla.expm(-1j * L * tt) @ v
        assert np.linalg.norm(W[:, i] - ref) <= 1e-10   # |v| = 1
        assert np.linalg.norm(W[:, i]) < 1.0            # dephasing decays


def test_expv_happy_breakdown_on_eigenvector():
    rng = np.random.default_rng(11)
    t = random_terms(rng, [2] * 5, scale=1e3)
    H = dense_from_terms(t)
    w_, V = np.linalg.eigh(H)
    v = V[:, 3].astype(np.complex128)
    W, st = po.expv(t, v, np.array([1e-3, 2e-3]), m=10, tol=1e-12)
    assert st.ibrkflag == 1 and st.mbrkdwn == 1
    for i, tt in enumerate([1e-3, 2e-3]):
        np.testing.assert_allclose(W[:, i], np.exp(-1j * w_[3] * tt) * v, atol=1e-10)


def test_expv_bad_sizes():
    rng = np.random.default_rng(1)
    t = random_terms(rng, [2, 2])
    with pytest.raises(RuntimeError):
        po.expv(t, np.ones(4, complex), [1.0], m=4)


def test_expv_block_equals_columns():
    rng = np.random.default_rng(5)
    t = random_terms(rng, [2] * 6, scale=1e4)
    D = t.dim
    V = rng.normal(size=(D, 3)) + 1j * rng.normal(size=(D, 3))
    T = np.array([[1e-4, 2e-4], [5e-5, 3e-4], [0.0, 1e-4]]).T
    W = po.expv_block(t, V, T, m=20)
    H = dense_from_terms(t)
    for c in range(3):
        for i in range(2):
            ref = sla.expm(-1j * H * T[i, c]) @ V[:, c]
            assert np.linalg.norm(W[:, i, c] - ref) <= 1e-10 * np.linalg.norm(ref)


# ---------------------------------------------------------------- physics
HBAR, MU0 = 1.054571800e-34, 1.2566370614e-06


def test_dipole_tensor_formula():
    c1, c2 = np.array([1.0, 2.0, -0.5]), np.array([-1.2, 0.3, 2.2])
    d = po.dipole(c1, c2, po.GAMMA_C13, po.GAMMA_C13).reshape(3, 3)
    r = c1 - c2
    rn = np.linalg.norm(r)
    n = r / rn
    pre = HBAR * MU0 / (4 * np.pi) * po.GAMMA_C13 ** 2 / (rn * 1e-10) ** 3
    np.testing.assert_allclose(d, pre * (np.eye(3) - 3 * np.outer(n, n)), rtol=1e-14, atol=0)
    assert np.all(po.dipole(c1, c1, 1.0, 1.0) == 0)


def _nv_numpy(B):
    s1x = np.array([[0, 1, 0], [1, 0, 1], [0, 1, 0]]) / np.sqrt(2)
    s1y = np.array([[0, -1j, 0], [1j, 0, -1j], [0, 1j, 0]]) / np.sqrt(2)
    s1z = np.diag([1.0, 0, -1])
    s111 = (s1x + s1y + s1z) / np.sqrt(3)
    H = 2.87e3 * 2 * np.pi * 1e6 * s111 @ s111 + po.GAMMA_NVE * (B[0] * s1x + B[1] * s1y + B[2] * s1z)
    w, V = np.linalg.eigh(H)
    sv = np.array([[np.real(V[:, i].conj() @ op @ V[:, i]) for op in (s1x, s1y, s1z)]
                   for i in range(3)])
    return w, sv


@pytest.mark.parametrize("B", [[0.05 / np.sqrt(3)] * 3, [0.02, -0.01, 0.07], [0.3, 0.1, 0.2]])
def test_nv_states_match_eigh(B):
    ev, sv = po.nv_states(B)
    w, svn = _nv_numpy(np.asarray(B))
    np.testing.assert_allclose(ev, w, rtol=0, atol=1e-13 * np.abs(w).max())
    np.testing.assert_allclose(sv, svn, atol=1e-9)


def _cluster_h_numpy(coords, B, center, sv):
    k = len(coords)
    ops = (SX, SY, SZ)

    def emb(i, M):
        out = np.eye(1)
        for q in range(k):
            out = np.kron(out, M if q == i else np.eye(2))
        return out

    H = np.zeros((2 ** k, 2 ** k), complex)
    for i in range(k):
        for j in range(i + 1, k):
            Dm = po.dipole(coords[i], coords[j], po.GAMMA_C13, po.GAMMA_C13).reshape(3, 3)
            for a in range(3):
                for b in range(3):
                    H += Dm[a, b] * emb(i, ops[a]) @ emb(j, ops[b])
    for i in range(k):
        for a in range(3):
            H += -po.GAMMA_C13 * B[a] * emb(i, ops[a])
        Dc = po.dipole(coords[i], center, po.GAMMA_C13, po.GAMMA_NVE).reshape(3, 3)
        f = Dc @ sv
        for a in range(3):
            H += f[a] * emb(i, ops[a])
    return H


def test_cluster_hamiltonian_term_list():
    rng = np.random.default_rng(2)
    coords = rng.normal(size=(4, 3)) * 3.0
    B = np.array([0.01, 0.02, 0.05])
    ev, sv = po.nv_states(B)
    center = np.zeros(3)
    t = po.cluster_hamiltonian(coords, B, center, sv[1])
    k = 4
    # term count: 9 per pair, 3 Zeeman + 3 field per spin (none zero here)
    assert t.nterm == 9 * k * (k - 1) // 2 + 6 * k
    assert list(t.nbody[:9]) == [2] * 9 and list(t.pos_list[:2]) == [0, 1]
    H = po.dense_hamiltonian(t)
    np.testing.assert_allclose(H, _cluster_h_numpy(coords, B, center, sv[1]),
                               atol=1e-9 * np.abs(H).max())
    np.testing.assert_allclose(H, dense_from_terms(t), atol=1e-9 * np.abs(H).max())


def test_zero_coefficients_are_skipped():
    coords = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0]])
    t = po.cluster_hamiltonian(coords, [0.0, 0.0, 0.1], [0.0, 0.0, -5.0], [0.0, 0.0, 0.0])
    # pair along z: only xx, yy, zz nonzero; Zeeman only z; field all zero
    assert t.nterm == 3 + 2
    assert np.all(t.coeff != 0)


def test_cpmg_intervals():
    np.testing.assert_allclose(po.cpmg_intervals(1), [0.5, 0.5])
    np.testing.assert_allclose(po.cpmg_intervals(8), [1 / 16] + [1 / 8] * 7 + [1 / 16])


# ---------------------------------------------------------------- coherence
def _bath(k, seed):
    rng = np.random.default_rng(seed)
    coords = rng.normal(size=(k, 3)) * 4.0 + np.array([5.0, 5.0, 5.0])
    B = np.array([0.0, 0.0, 0.05])
    _, sv = po.nv_states(B)
    H0 = po.dense_hamiltonian(po.cluster_hamiltonian(coords, B, np.zeros(3), sv[0]))
    H1 = po.dense_hamiltonian(po.cluster_hamiltonian(coords, B, np.zeros(3), sv[1]))
    return H0, H1


def _coherence_direct(H0, H1, n, times):
    frac = po.cpmg_intervals(n)
    D = H0.shape[0]
    out = []
    for t in times:
        B0 = np.eye(D, dtype=complex)
        B1 = np.eye(D, dtype=complex)
        for j, f in enumerate(frac):
            Ha, Hb = (H0, H1) if j % 2 == 0 else (H1, H0)
            B0 = B0 @ sla.expm(-1j * Ha * f * t)
            B1 = B1 @ sla.expm(-1j * Hb * f * t)
        out.append(np.real(np.trace(B1.conj().T @ B0)) / D)
    return np.array(out)


@pytest.mark.parametrize("k,n", [(1, 1), (2, 1), (3, 2), (3, 4)])
def test_coherence_hilbert_equals_liouville_and_direct(k, n):
    H0, H1 = _bath(k, 10 + k)
    nT, dt = 21, 2e-5
    Lh = po.coherence_hilbert(H0, H1, n, nT, dt)
    Ll = po.coherence_liouville(k, H0, H1, n, nT, dt)
    Ld = _coherence_direct(H0, H1, n, dt * np.arange(nT))
    assert Lh[0] == 1.0
    np.testing.assert_allclose(Ll, Ld, atol=1e-10)
    np.testing.assert_allclose(Lh, Ld, atol=1e-10)
    assert np.all(np.abs(Lh) <= 1 + 1e-12)


def test_single_spin_hahn_echo_closed_form():
    """One 13C with a pure-z hyperfine field: the echo refocuses exactly."""
    H0 = 0.5 * np.diag([1.0, -1.0]) * 2e4
    H1 = 0.5 * np.diag([1.0, -1.0]) * 7e4
    L = po.coherence_hilbert(H0.astype(complex), H1.astype(complex), 1, 11, 1e-5)
    np.testing.assert_allclose(L, 1.0, atol=1e-13)


def test_liouville_dephasing_decays():
    H0, H1 = _bath(2, 3)
    L0 = po.coherence_liouville(2, H0, H1, 1, 11, 5e-5)
    L1 = po.coherence_liouville(2, H0, H1, 1, 11, 5e-5, dephase_rate=2 * np.pi * 1e3,
                                axis=(0, 0, 1))
    assert np.all(np.abs(L1[1:]) < np.abs(L0[1:]) + 1e-12)


def _liouville_numpy(k, H0, H1, n, times, rate, axis, pol):
    """The reference's Liouville form built literally with numpy kron products
    (column-major vec: vec(A X B) = (B^T (x) A) vec X):
    SHARP(H_a) - FLAT(H_b) (ensemble_cce.cpp:86-92), i g (sigma^T (x) sigma - 1)
    per spin (SpinInteractionComponent.cpp:285-304), rho0 = I/D + sum p.S
    (SpinState.cpp:9-60), L = Re <D rho0, prod_j expm(-i L_j f_j t) rho0>."""
    D = 2 ** k
    I = np.eye(D)
    nx, ny, nz = np.asarray(axis, float) / np.linalg.norm(axis)
    sig = np.array([[nz, nx - 1j * ny], [nx + 1j * ny, -nz]])
    ops = [SX, SY, SZ]

    def on_spin(m, s):
        return np.kron(np.kron(np.eye(2 ** s), m), np.eye(2 ** (k - 1 - s)))
    deph = sum(np.kron(on_spin(sig, s).T, on_spin(sig, s)) - np.eye(D * D) for s in range(k))
    LA = np.kron(H0.T, I) - np.kron(I, H1) + 1j * rate * deph
    LB = np.kron(H1.T, I) - np.kron(I, H0) + 1j * rate * deph
    rho0 = I / D + sum(pol[a] * on_spin(ops[a], s) for s in range(k) for a in range(3))
    v0 = rho0.reshape(-1, order="F")
    frac = po.cpmg_intervals(n)
    out = []
    for t in times:
        v = v0.astype(complex)
        for j, f in enumerate(frac):
            v = sla.expm(-1j * (LA if j % 2 == 0 else LB) * f * t) @ v
        out.append(np.real(np.vdot(D * v0, v)))
    return np.array(out)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_liouville_branch_propagators_are_rho_dagger_mirrors(k):
    """The identity the GPU Liouville path uses to skip branch B's exponential:
    with J rho = rho^+, J L_A J = L_B for the reference's Liouvillians with
    dephasing, so exp(-i L_B tau) = P conj(exp(-i L_A tau)) P, P the transpose
    permutation of column-major vec(rho)."""
    H0, H1 = _bath(k, 80 + k)
    D = 2 ** k
    I = np.eye(D)
    nx, ny, nz = np.array([1.0, 1.0, 1.0]) / np.sqrt(3.0)
    sig = np.array([[nz, nx - 1j * ny], [nx + 1j * ny, -nz]])

    def on_spin(m, s):
        return np.kron(np.kron(np.eye(2 ** s), m), np.eye(2 ** (k - 1 - s)))
    deph = sum(np.kron(on_spin(sig, s).T, on_spin(sig, s)) - np.eye(D * D) for s in range(k))
    g, tau = 2 * np.pi * 1e4, 5e-6
    LA = np.kron(H0.T, I) - np.kron(I, H1) + 1j * g * deph
    LB = np.kron(H1.T, I) - np.kron(I, H0) + 1j * g * deph
    GA, GB = sla.expm(-1j * tau * LA), sla.expm(-1j * tau * LB)
    P = np.array([(e // D) + D * (e % D) for e in range(D * D)])
    np.testing.assert_allclose(GB, np.conj(GA[np.ix_(P, P)]), atol=1e-13)


@pytest.mark.parametrize("k,n", [(1, 1), (2, 1), (2, 2), (2, 3)])
def test_liouville_dephasing_and_polarisation_match_numpy_kron(k, n):
    """Pins orc_coherence_liouville's dephasing superoperator and initial state
    against an independent kron construction of the reference's operators."""
    H0, H1 = _bath(k, 40 + k)
    nT, dt = 9, 4e-5
    rate, axis, pol = 2 * np.pi * 3e3, (1.0, 1.0, 1.0), (0.1, -0.05, 0.2)
    Lo = po.coherence_liouville(k, H0, H1, n, nT, dt, dephase_rate=rate, axis=axis, pol=pol)
    Ln = _liouville_numpy(k, H0, H1, n, dt * np.arange(nT), rate, axis, pol)
    np.testing.assert_allclose(Lo, Ln, atol=1e-11)
    assert abs(Lo[0] - Ln[0]) < 1e-14


@pytest.mark.parametrize("k,n", [(1, 1), (2, 1), (3, 2), (3, 3)])
def test_coherence_state_matches_direct_propagation(k, n):
    """orc_coherence_state against scipy: the basis state propagated segment by
    segment through riffle(H0, H1) and riffle(H1, H0)."""
    H0, H1 = _bath(k, 60 + k)
    nT, dt = 11, 3e-5
    frac = po.cpmg_intervals(n)
    D = 2 ** k
    for b in (0, D - 1, D // 2):
        Lo = po.coherence_state(H0, H1, n, nT, dt, b)
        ref = []
        for t in dt * np.arange(nT):
            v = [np.eye(D)[:, b].astype(complex), np.eye(D)[:, b].astype(complex)]
            for a in (0, 1):
                for j, f in enumerate(frac):
                    H = (H0, H1)[(j + a) % 2]
                    v[a] = sla.expm(-1j * H * f * t) @ v[a]
            ref.append(np.real(np.vdot(v[0], v[1])))
        np.testing.assert_allclose(Lo, ref, atol=1e-11)


def test_bath_state_from_seed_matches_the_c_library():
    """oops_bath_state_from_seed restates glibc's srand/rand; on a glibc host
    the library's own rand() % 2 sequence must be identical."""
    import ctypes
    import ctypes.util
    from oops_gb300 import cce
    name = ctypes.util.find_library("c")
    libc = ctypes.CDLL(name) if name else None
    if libc is None or not hasattr(libc, "gnu_get_libc_version"):
        pytest.skip("not a glibc host")
    for seed in (0, 1, 7, 12345, 2 ** 31 - 1):
        libc.srand(ctypes.c_uint(seed))
        want = np.array([libc.rand() % 2 for _ in range(700)], np.uint8)
        got = cce.bath_state_from_seed(seed, 700)
        assert np.array_equal(got, want), seed


# ---------------------------------------------------------------- enumeration
def _brute_force(coords, cutoff, max_order):
    n = len(coords)
    d = np.linalg.norm(coords[:, None, :] - coords[None, :, :], axis=-1)
    adj = (d <= cutoff) & ~np.eye(n, dtype=bool)
    sets = [sorted((i,) for i in range(n))]
    parents = [{}]
    for o in range(1, max_order):
        found = {}
        for pi, p in enumerate(sets[o - 1]):
            cand = set()
            for a in p:
                cand |= set(np.nonzero(adj[a])[0].tolist())
            for j in sorted(cand - set(p)):
                c = tuple(sorted(p + (j,)))
                found.setdefault(c, set()).add(pi)
        sets.append(sorted(found))
        parents.append(found)
    return sets, parents


@pytest.mark.parametrize("seed,n,cut,order", [(0, 40, 3.0, 4), (1, 25, 4.0, 5), (2, 60, 2.5, 3)])
def test_enumeration_matches_brute_force(seed, n, cut, order):
    rng = np.random.default_rng(seed)
    coords = rng.uniform(-6, 6, size=(n, 3))
    e = po.Enumeration(coords, cut, order)
    sets, parents = _brute_force(coords, cut, order)
    for o in range(order):
        cl = e.clusters(o)
        assert [tuple(int(x) for x in r) for r in cl] == sets[o]
        if o > 0:
            for i, c in enumerate(sets[o]):
                assert list(e.parents(o, i)) == sorted(parents[o][c])


def test_subcluster_closure_and_reduction():
    rng = np.random.default_rng(4)
    coords = rng.uniform(-4, 4, size=(20, 3))
    order = 3
    e = po.Enumeration(coords, 3.5, order)
    sets = [[tuple(int(x) for x in r) for r in e.clusters(o)] for o in range(order)]
    pos = [{c: i for i, c in enumerate(s)} for s in sets]
    for o in range(order):
        for i, c in enumerate(sets[o]):
            # closure = every connected proper sub-cluster reachable by growth
            got = set(e.subclusters(o, i))
            want = set()
            for r in range(1, o + 1):
                for sub in itertools.combinations(c, r):
                    if sub in pos[r - 1]:
                        want.add((r - 1, pos[r - 1][sub]))
            assert got <= want
            assert all(len(sets[a][b]) < len(c) for a, b in got)
    nT = 5
    Lraw = [1.0 - 0.01 * rng.random((nT, e.count(o))) for o in range(order)]
    til, each, cum = e.reduce(Lraw, nT)
    # numpy restatement of cce.cpp:151-189
    til_np = []
    for o in range(order):
        T = Lraw[o].copy()
        for j in range(e.count(o)):
            for (a, b) in sorted(e.subclusters(o, j)):
                T[:, j] = T[:, j] / til_np[a][:, b]
        til_np.append(T)
    for o in range(order):
        assert np.array_equal(til[o], til_np[o])
    np.testing.assert_allclose(cum[:, -1], np.prod([np.prod(t, axis=1) for t in til_np], axis=0),
                               rtol=1e-12)
