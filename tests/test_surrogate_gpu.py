"""The learned warm start end to end on a small scale (48^3 boxes): FP64 training
data from the solver, a U-Net trained on the GPU by the library's kernels, and
held-out geometries started from its prediction.  The trained network must beat
the same start procedure without it (rest, then the one-off averaging), and the
warm-started field must end as close to the plain solve as that start does."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from hemelb_gb300 import surrogate as S  # noqa: E402


def test_trained_warm_start_reaches_steady_state_sooner():
    box = 48
    train = [S.Sample.draw(i, base_seed=5, box=box) for i in range(192)]
    test = [S.Sample.draw(10_000 + i, base_seed=5, box=box) for i in range(12)]
    grids, recs = S.generate(train, box, average=True, workers=8)
    assert all(r["steps"] > 0 for r in recs)
    net = S.UNet(seed=0)
    # a fixed number of epochs, so that the outcome does not depend on the GPU's speed
    hist = S.train(net, grids, len(train), batch=4, epochs=250)
    assert hist[-1] < 0.1 * hist[0]
    ev = S.evaluate(net, test, box)
    summ = S.summarise(ev)
    for arm in ("rest", "rest_avg", "warm"):
        assert summ[arm]["converged"] == len(test), arm
    # what the network gains over the same start without it
    assert summ["warm"]["total_steps"] < summ["rest_avg"]["total_steps"]
    assert summ["prediction_u_rel_l2"]["median"] < 0.5
    # and the final fields agree with the plain solve as well as the rest start's do
    warm_err = np.array([e["warm_u_rel_l2"] for e in ev])
    rest_err = np.array([e["rest_avg_u_rel_l2"] for e in ev])
    assert np.median(warm_err) <= 2.0 * np.median(rest_err) + 1e-6
