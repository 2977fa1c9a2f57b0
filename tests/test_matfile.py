"""The MAT-file result writer (oops_cce_export_mat), the counterpart of
CCE::export_mat_file (src/source/app/cce.cpp:191-234), read back with
scipy.io.loadmat: variable names, shapes, values (bit-exact) and the global
flag that matPutVariableAsGlobal sets; and against the variables the
reference's own export_mat_file writes (tests/golden/reference_export.npz)."""
import numpy as np
import pytest

sio = pytest.importorskip("scipy.io")

from oops_gb300 import cce  # noqa: E402


def _data(counts, nT, seed=3):
    rng = np.random.default_rng(seed)
    K = len(counts)
    L = [rng.normal(size=(n, nT)) for n in counts]
    T = [rng.normal(size=(n, nT)) for n in counts]
    return rng.normal(size=(nT, K)), rng.normal(size=(nT, K)), L, T, np.linspace(0, 2e-3, nT)


def test_export_mat_round_trip(tmp_path):
    counts, nT = [5, 3, 0, 2], 7
    cum, each, L, T, t = _data(counts, nT)
    path = tmp_path / "res.mat"
    cce.export_mat(path, t, cum, each, L, T)
    m = sio.loadmat(str(path))
    names = {f"CCE{o}" for o in range(4)} | {f"CCE{o}_tilder" for o in range(4)} | \
        {"final_result_each_order", "final_result", "time_list"}
    assert names <= set(m)
    assert set(m["__globals__"]) == names
    for o, n in enumerate(counts):
        assert m[f"CCE{o}"].shape == (nT, n)            # nTime x nClst, column = cluster
        assert np.array_equal(m[f"CCE{o}"], L[o].T)
        assert np.array_equal(m[f"CCE{o}_tilder"], T[o].T)
    assert np.array_equal(m["final_result"], cum)
    assert np.array_equal(m["final_result_each_order"], each)
    assert np.array_equal(m["time_list"], t.reshape(nT, 1))
    assert m["__header__"].startswith(b"MATLAB 5.0 MAT-file")


def test_export_mat_without_cluster_curves(tmp_path):
    counts, nT = [2, 1], 4
    cum, each, _, _, t = _data(counts, nT, seed=4)
    path = tmp_path / "final.mat"
    cce.export_mat(path, t, cum, each)
    m = sio.loadmat(str(path))
    assert not any(k.startswith("CCE") for k in m)
    assert np.array_equal(m["final_result"], cum)


def test_export_mat_rejects_bad_shapes(tmp_path):
    with pytest.raises(ValueError):
        cce.export_mat(tmp_path / "x.mat", np.zeros(3), np.zeros((4, 2)), np.zeros((4, 2)))


def test_result_file_equals_what_the_reference_exports(tmp_path):
    """The variables the reference's own CCE::export_mat_file writes after a
    run (tests/golden/reference_export.npz: cce.cpp compiled with a
    recording stand-in of MATLAB's mat.h, made by
    tests/golden/make_reference_export.py), fed through oops_cce_export_mat:
    the same variables in the same order, each global, real, with the same
    shape and the same values bit for bit."""
    import os
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_export.npz"))
    names = [str(n) for n in ref["names"]]
    K = sum(1 for n in names if n.startswith("CCE") and not n.endswith("_tilder"))
    var = {n: ref[f"var/{n}"] for n in names}
    assert not any(int(ref[f"complex/{n}"]) for n in names)
    path = tmp_path / "result.mat"
    cce.export_mat(path, var["time_list"].ravel(), var["final_result"], var["final_result_each_order"],
                   [var[f"CCE{o}"].T for o in range(K)], [var[f"CCE{o}_tilder"].T for o in range(K)])
    assert [w[0] for w in sio.whosmat(str(path))] == names
    m = sio.loadmat(str(path))
    assert set(m["__globals__"]) == set(names)
    for n in names:
        assert m[n].dtype == np.float64 and m[n].shape == var[n].shape, n
        assert np.array_equal(m[n], var[n]), n
