"""GPU parity of the Krylov drop-in and the device matvec against the CPU
oracle (which is itself pinned in test_oracle.py)."""
import numpy as np
import pytest

import pyoracle as po
from helpers import dense_from_terms, random_terms

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oops_gb300 as og  # noqa: E402


def _cluster_terms(k, seed, state=1, B=(0.0, 0.0, 0.05)):
    rng = np.random.default_rng(seed)
    coords = rng.normal(size=(k, 3)) * 3.0 + np.array([4.0, 3.0, 5.0])
    _, sv = po.nv_states(np.asarray(B))
    return po.cluster_hamiltonian(coords, B, np.zeros(3), sv[state])


@pytest.mark.parametrize("dims", [(2,) * 6, (2,) * 10, (3, 2, 2), (2, 3, 2, 3)])
@pytest.mark.parametrize("nvec", [1, 4])
def test_matvec_matches_oracle(dims, nvec):
    rng = np.random.default_rng(len(dims) + nvec)
    t = random_terms(rng, list(dims))
    D = t.dim
    X = rng.normal(size=(D, nvec)) + 1j * rng.normal(size=(D, nvec))
    H = og.Hamiltonian(t)
    Y = H.apply(torch.from_numpy(X).cuda().contiguous(), alpha=-1j).cpu().numpy()
    for b in range(nvec):
        ref = po.hamvec(t, X[:, b], -1j * t.coeff)
        np.testing.assert_allclose(Y[:, b], ref, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("k,m", [(6, 30), (9, 30), (11, 20)])
def test_main_cache_matches_oracle(k, m):
    t = _cluster_terms(k, seed=k)
    rng = np.random.default_rng(k)
    v = rng.normal(size=t.dim) + 1j * rng.normal(size=t.dim)
    v /= np.linalg.norm(v)
    tl = np.array([0.0, 2e-6, 1e-5, 1e-5, 4e-5])
    got = og.main_cache(t, v, tl, m=m, tol=1e-12)
    ref, _ = po.expv(t, v, tl, m=m, tol=1e-12)
    for i in range(tl.size):
        assert np.linalg.norm(got[:, i] - ref[:, i]) <= 1e-10 * np.linalg.norm(ref[:, i])


def test_main_mkl_symbol_is_the_same_gpu_path():
    t = _cluster_terms(7, seed=3)
    v = np.zeros(t.dim, complex)
    v[5] = 1.0
    tl = np.array([1e-5, 3e-5])
    a = og.main_cache(t, v, tl)
    b = og.main_cache(t, v, tl, use_mkl_symbol=True)
    np.testing.assert_allclose(a, b, atol=1e-14)


def test_generic_dims_expv():
    rng = np.random.default_rng(9)
    t = random_terms(rng, [3, 2, 2, 3], scale=1e4)
    v = rng.normal(size=t.dim) + 1j * rng.normal(size=t.dim)
    tl = np.array([1e-5, 1e-4])
    got = og.main_cache(t, v, tl, m=20)
    ref, _ = po.expv(t, v, tl, m=20)
    assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)


def test_happy_breakdown_on_eigenvector():
    rng = np.random.default_rng(11)
    t = random_terms(rng, [2] * 5, scale=1e3)
    H = dense_from_terms(t)
    w, V = np.linalg.eigh(H)
    v = V[:, 3].astype(np.complex128)
    got = og.main_cache(t, v, [1e-3, 2e-3], m=10)
    for i, tt in enumerate([1e-3, 2e-3]):
        np.testing.assert_allclose(got[:, i], np.exp(-1j * w[3] * tt) * v, atol=1e-10)


def test_block_expv_per_column_times():
    t = _cluster_terms(8, seed=5)
    rng = np.random.default_rng(5)
    D = t.dim
    nvec = 5
    V = rng.normal(size=(D, nvec)) + 1j * rng.normal(size=(D, nvec))
    T = np.sort(rng.uniform(0, 3e-5, size=(3, nvec)), axis=0)
    H = og.Hamiltonian(t)
    W, st = og.expv_block(H, torch.from_numpy(V).cuda().contiguous(), T, m=25, tol=1e-12)
    W = W.cpu().numpy()
    ref = po.expv_block(t, V, T, m=25, tol=1e-12)
    for b in range(nvec):
        for i in range(3):
            r = ref[:, i, b]
            assert np.linalg.norm(W[i, :, b] - r) <= 1e-10 * np.linalg.norm(r)
    assert st.nstep >= 1 and st.anorm > 0


def test_errors_are_reported_not_fatal():
    t = _cluster_terms(3, seed=1)
    v = np.ones(t.dim, complex)
    with pytest.raises(og.OopsError) as e:
        og.main_cache(t, v, [1e-5], m=t.dim)       # m >= n: 'bad sizes'
    assert e.value.code == -3
    three = po.KronTerms.from_list([2, 2, 2], [(1.0, [(0, np.eye(2)), (1, np.eye(2)), (2, np.eye(2))])])
    with pytest.raises(og.OopsError) as e:
        og.main_cache(three, np.ones(8, complex), [1e-5], m=4)
    assert e.value.code == -4
    # the library stays usable after errors
    got = og.main_cache(t, v / np.linalg.norm(v), [1e-6], m=4)
    assert np.isfinite(got).all()
