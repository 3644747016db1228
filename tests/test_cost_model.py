"""The cost model's parameters (host) and the autotuner that measures them
(GPU).  They replace the reference's per-GPU parameter files and their
calibrator (src/evaluator.cpp:98-107, evaluator-preprocess/process.cpp)."""
import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W


def test_params_round_trip_and_validation():
    p0 = hq.cost_params()
    assert all(v > 0 for v in p0.values())
    try:
        hq.set_cost_params({"oshm_gate": 1e-13})
        assert hq.cost_params()["oshm_gate"] == 1e-13
        with pytest.raises(hq.HQError):
            hq.set_cost_params({"pass_floor": -1.0})
        assert hq.cost_params()["pass_floor"] == p0["pass_floor"]  # rejected: unchanged
    finally:
        hq.set_cost_params(p0)


def test_params_drive_the_hybrid_choice():
    """A cheap TransMM makes the hybrid partitioner pick it; an expensive one
    makes it pick OShareMem (host-only planning)."""
    import ctypes as C
    from test_partition import plan
    p0 = hq.cost_params()
    desc = W.qft(16)
    try:
        hq.set_cost_params({"mm_bf16x3": 1e-15, "mm_tf32": 1e-15, "mm_fp32": 1e-15, "launch": 0.0})
        g1 = plan(16, desc, hq.BACKEND_HYBRID, reference=False)
        hq.set_cost_params({"mm_bf16x3": 1e-6, "mm_tf32": 1e-6, "mm_fp32": 1e-6})
        g2 = plan(16, desc, hq.BACKEND_HYBRID, reference=False)
    finally:
        hq.set_cost_params(p0)
    assert any(g["backend"] == hq.BACKEND_TRANSMM for g in g1)
    assert all(g["backend"] == hq.BACKEND_OSHM for g in g2)


@pytest.mark.gpu
def test_autotune_measures_plausible_constants(hq):
    p0 = hq.cost_params()
    try:
        p = hq.autotune(24)
        assert p == hq.cost_params()  # installed
        # HBM floor: 16 B per amplitude at 1..10 TB/s
        assert 1.6e-12 < p["pass_floor"] < 1.6e-11, p
        # oshm_gate is per arithmetic unit and the probe's RX gates cost two
        # units, so an interleaved T gate costs less than one RX
        assert 0 < p["oshm_gate"] < 1e-11, p
        assert 0 <= p["oshm_diag"] < 2 * p["oshm_gate"], p
        assert 0 < p["mm_tf32"] and 0 < p["mm_bf16x3"] < p["mm_fp32"], p
        assert 0 < p["launch"] < 1e-3, p
    finally:
        hq.set_cost_params(p0)


def test_tile_width_is_chosen_per_circuit():
    """tile_qubits = 0 partitions at 11, 12 and 13 tile qubits and keeps the
    partition the cost model predicts fastest; an explicit width is kept."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    g = W.to_gates(W.grid_random(2, 5, 6, 20))
    auto = hq.plan_groups(30, g)
    assert {x["width"] for x in auto} == {13} and len(auto) == 11
    for t in (11, 12):
        fixed = hq.plan_groups(30, g, tile_qubits=t)
        assert {x["width"] for x in fixed} == {t} and len(fixed) > len(auto)
    small = hq.plan_groups(9, W.to_gates(W.grid_random(3, 3, 3, 6)))
    assert {x["width"] for x in small} == {9}


def test_hybrid_keeps_the_best_whole_schedule():
    """The hybrid's per-group choice is set against the OShareMem-only and
    TransMM-only schedules and the predicted-fastest kept: deep dense 7-qubit
    blocks fuse into TransMM groups throughout, the grid circuit stays
    OShareMem."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W

    def kinds(n, g, backend):
        return [x["backend"] for x in hq.plan_groups(n, g, backend=backend)]

    blocked = W.to_gates(W.blocked_u3_cnot(11, 28, 7, 10, 2))
    assert set(kinds(28, blocked, hq.BACKEND_HYBRID)) == {hq.BACKEND_TRANSMM}
    grid = W.to_gates(W.grid_random(2, 5, 6, 20))
    assert set(kinds(30, grid, hq.BACKEND_HYBRID)) == {hq.BACKEND_OSHM}
