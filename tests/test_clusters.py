"""Product cluster enumeration (host C++ in liboops_gb300.so) against the
oracle restatement and the reference's own bath fixture.  Integer work:
bit-exact."""
import os

import numpy as np
import pytest

import pyoracle as po
from oops_gb300 import bath, configs
from oops_gb300.cce import Clusters, nv_states

REF_ROOT = os.environ.get("OOPS_REFERENCE_ROOT", "")
ROY = os.path.join(REF_ROOT, "src", "dat_example", "input", "C13Bath", "RoyCoord.xyz") if REF_ROOT else ""


def _same(coords, cutoff, order):
    c = Clusters(coords, cutoff, order)
    e = po.Enumeration(coords, cutoff, order)
    for o in range(order):
        a = c.clusters(o).astype(np.uint64)
        b = e.clusters(o)
        assert a.shape == b.shape and np.array_equal(a, b), f"order {o}"
        off, pairs = c.subclusters(o)
        for j in range(c.count(o)):
            got = [tuple(int(x) for x in p) for p in pairs[off[j]:off[j + 1]]]
            assert got == e.subclusters(o, j)
    return c


@pytest.mark.parametrize("seed,n,cut,order", [(0, 40, 3.0, 4), (1, 25, 4.0, 5), (3, 120, 2.2, 6)])
def test_enumeration_bit_exact_random(seed, n, cut, order):
    rng = np.random.default_rng(seed)
    _same(rng.uniform(-7, 7, size=(n, 3)), cut, order)


def test_enumeration_bit_exact_diamond_cce4():
    w = configs.cce4_hahn()
    c = _same(w.coords, w.cutoff, w.max_order)
    assert c.count(0) == len(w.coords)


@pytest.mark.skipif(not ROY or not os.path.exists(ROY), reason="OOPS_REFERENCE_ROOT not set")
def test_enumeration_on_reference_fixture():
    """RoyCoord.xyz: the 548-site 13C bath the reference ships
    (src/dat_example/input/C13Bath/RoyCoord.xyz), read in place from the tree
    OOPS_REFERENCE_ROOT names (tests/test_reference_pins.py holds the same
    bath and the reference code's own enumeration of it as a fixture)."""
    coords, iso = bath.read_xyz(ROY)
    assert len(coords) == 548 and set(iso) == {"13C"}
    c = _same(coords, 5.0, 3)
    assert [c.count(o) for o in range(3)][0] == 548


def test_edge_cases():
    # no connections: higher orders are empty (the reference's armadillo code
    # would abort on an empty growth matrix)
    far = np.array([[0, 0, 0], [100, 0, 0], [0, 100, 0]], float)
    c = Clusters(far, 1.0, 3)
    assert [c.count(o) for o in range(3)] == [3, 0, 0]
    # empty bath
    c = Clusters(np.zeros((0, 3)), 1.0, 2)
    assert c.count(0) == 0
    # cutoff is inclusive (dist <= cutoff)
    two = np.array([[0, 0, 0], [2.0, 0, 0]])
    assert Clusters(two, 2.0, 2).count(1) == 1
    assert Clusters(two, 2.0 - 1e-12, 2).count(1) == 0


@pytest.mark.parametrize("B", [[0, 0, 0.05], [0.02, -0.01, 0.07], [0.3, 0.1, 0.2]])
def test_nv_states_match_oracle(B):
    ev, sv = nv_states(B)
    ev0, sv0 = po.nv_states(B)
    np.testing.assert_allclose(ev, ev0, rtol=0, atol=1e-12 * np.abs(ev0).max())
    np.testing.assert_allclose(sv, sv0, atol=1e-10)


def test_diamond_bath_generator():
    s = bath.diamond_sites(10.0)
    # nearest-neighbour distance a*sqrt(3)/4 appears, no site at the origin or N
    d = np.linalg.norm(s, axis=1)
    assert d.min() > 1.0
    b1 = bath.diamond_bath(20.0, 0.011, 5)
    b2 = bath.diamond_bath(20.0, 0.011, 5)
    assert np.array_equal(b1, b2)
    assert 30 < len(b1) < 120
