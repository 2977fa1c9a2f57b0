"""The host-buffer whole run (oops_ensemble_cce) replays a per-thread run plan
(device buffers + CUDA graph keyed on the run's shape and parameters).  Every
call must recompute from its own inputs: a second bath with the same cluster
structure, a changed parameter, and a released plan all give exactly the
device-resident run's results for those inputs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oops_gb300 import cce, configs  # noqa: E402


def _device(coords, w, p, prec, order):
    run = cce.DeviceRun(coords, w.cutoff, order, p, prec)
    return run.step().cpu().numpy().T, run.counts


@pytest.mark.parametrize("prec", [cce.PREC_FP64, cce.PREC_MIXED])
def test_plan_recomputes_every_call(prec):
    w = configs.cce4_hahn()
    order, nT = 3, 41
    _, sv = cce.nv_states(w.B)
    p = cce.CCEParams.make(w.B, sv[0], sv[1], 1, nT, 1e-4)
    # same cluster structure, different geometry: a uniform 0.1 % dilation
    # keeps every pair on its side of the cutoff for this bath
    coords2 = w.coords * 1.001
    ref1, c1 = _device(w.coords, w, p, prec, order)
    ref2, c2 = _device(coords2, w, p, prec, order)
    assert c1 == c2, "dilation changed the cluster structure"
    assert np.abs(ref1 - ref2).max() > 1e-9          # the curves do change
    cce.release_plans()
    a1 = cce.ensemble_cce(w.coords, w.cutoff, order, p, prec)[0]     # builds the plan
    a2 = cce.ensemble_cce(coords2, w.cutoff, order, p, prec)[0]      # replays it
    a1b = cce.ensemble_cce(w.coords, w.cutoff, order, p, prec)[0]    # replays again
    assert np.array_equal(a1, ref1) and np.array_equal(a1b, ref1)
    assert np.array_equal(a2, ref2)
    p2 = cce.CCEParams.make(w.B, sv[0], sv[1], 1, nT, 1.2e-4)          # new key: rebuild
    ref3, _ = _device(w.coords, w, p2, prec, order)
    assert np.array_equal(cce.ensemble_cce(w.coords, w.cutoff, order, p2, prec)[0], ref3)
    cce.release_plans()
    assert np.array_equal(cce.ensemble_cce(coords2, w.cutoff, order, p, prec)[0], ref2)
