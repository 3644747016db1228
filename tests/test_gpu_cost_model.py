"""The hybrid partitioner's cost model against measurement.  The reference
calibrates its evaluator per qubit count offline (evaluator-preprocess/
process.cpp:24-176, src/evaluator.cpp:60-229); here the model's per-group
device time (hq_circuit_predict) is checked against CUDA-event timings of the
same groups (hq_circuit_profile) on three circuit families: the groups must
come out in the same order of cost and within a stated factor of their
measured times."""
import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = {
    "grid26": (26, lambda: W.grid_random(2, 2, 13, 20)),
    "qft24": (24, lambda: W.qft(24)),
    "ryrz26": (26, lambda: W.ry_rz_cz(W.SplitMix64(8), 26, 30)),
}


def spearman(a, b):
    ra = np.argsort(np.argsort(a))
    rb = np.argsort(np.argsort(b))
    if np.std(ra) == 0 or np.std(rb) == 0:
        return 1.0
    return float(np.corrcoef(ra, rb)[0, 1])


@pytest.mark.parametrize("name", list(CASES))
def test_predicted_group_times_track_measured(hq, name):
    n, make = CASES[name]
    c = hq.Circuit(n)
    c.addGates(W.to_gates(make()))
    c.compile("oshm")
    s = hq.State(n)
    c.run_on(s)
    meas = np.median([c.profile(s) for _ in range(3)], axis=0)
    pred = c.predict()
    s.free()
    assert pred.shape == meas.shape and np.all(pred > 0) and np.all(meas > 0)
    ratio = pred / meas
    # every group within a factor 1.6 of its measured time, the circuit's total
    # within 25 %, and (with enough groups to rank) the same order of cost
    msg = f"{name}: predicted {np.round(pred).tolist()} measured {np.round(meas).tolist()} us"
    assert np.all((ratio > 1 / 1.6) & (ratio < 1.6)), msg
    assert abs(pred.sum() / meas.sum() - 1) < 0.25, msg
    if len(meas) >= 5 and np.ptp(meas) > 0.2 * np.mean(meas):
        assert spearman(pred, meas) >= 0.6, msg
