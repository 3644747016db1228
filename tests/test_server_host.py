"""Serving admission checks on the host (no GPU): qubit range, gate indices,
state bytes (2^n x 8 B) against the HBM budget."""
import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W


def test_accepts_in_range():
    hq.server_check(12, W.to_gates(W.ry_rz_cz(W.SplitMix64(1), 12, 3)))
    hq.server_check(32, [], hbm_budget=150 * 10**9)


@pytest.mark.parametrize("n", [0, 9, 35, 40])
def test_rejects_qubit_count(n):
    with pytest.raises(hq.HQError):
        hq.server_check(n, [])


def test_rejects_over_budget():
    with pytest.raises(hq.HQError) as e:
        hq.server_check(20, [], hbm_budget=1 << 20)
    assert e.value.code == -3  # HQ_ERR_NOMEM
    hq.server_check(34, [], hbm_budget=150 * 10**9)  # 137 GB state fits 150 GB
    with pytest.raises(hq.HQError):
        hq.server_check(34, [], hbm_budget=100 * 10**9)


def test_budget_boundary():
    n = 20
    hq.server_check(n, [], hbm_budget=8 << n)
    with pytest.raises(hq.HQError):
        hq.server_check(n, [], hbm_budget=(8 << n) - 1)


def test_rejects_bad_gates():
    with pytest.raises(hq.HQError):
        hq.server_check(12, [hq.Gate.CNOT(3, 12)])
    with pytest.raises(hq.HQError):
        hq.server_check(12, [hq.Gate.CNOT(3, 3)])


def test_oracle_sampler_is_inverse_cdf():
    import numpy as np
    import oracle as O
    a = np.zeros(16, dtype=np.complex64)
    a[3] = 0.6
    a[9] = 0.8j
    s = O.sample(a, 4000, 7)
    assert set(np.unique(s).tolist()) <= {3, 9}
    assert abs(np.mean(s == 9) - 0.64) < 0.03
