"""Pins the CPU oracle (oracle/oracle.c) to the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference's CPU code
(gate factories, GateGroup::initCPUMatrix) built by oracle/Makefile `ref`
(script: tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from hyquas_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_matrices_match_reference_factories():
    recs = json.loads((GOLDEN / "matrices.json").read_text())
    assert len(recs) == 66
    for r in recs:
        got = O.gate_matrix(r["type"], r["params"])
        np.testing.assert_allclose(got, r["mat"], rtol=0, atol=1e-15, err_msg=str(r))


@pytest.mark.parametrize("n", [4, 5, 6, 7, 8])
def test_gate_by_gate_matches_reference_fused_unitary(n):
    z = np.load(GOLDEN / f"unitary_n{n}.npz")
    desc = [tuple(x[:4]) + (tuple(x[4]),) for x in json.loads(str(z["desc"]))]
    out0 = O.run_f64(n, desc)
    np.testing.assert_allclose(out0, z["out_zero"], rtol=0, atol=1e-12)
    out1 = O.apply_f64(n, z["psi"], desc)
    np.testing.assert_allclose(out1, z["out_psi"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("n", [6, 8])
def test_group_unitary_matches_gate_by_gate(n):
    z = np.load(GOLDEN / f"unitary_n{n}.npz")
    desc = [tuple(x[:4]) + (tuple(x[4]),) for x in json.loads(str(z["desc"]))]
    U = O.group_unitary(list(range(n)), desc)
    np.testing.assert_allclose(U @ z["psi"], z["out_psi"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(U.conj().T @ U, np.eye(1 << n), atol=1e-12)


def test_f32_baseline_tracks_f64():
    desc = W.plain_u3_cnot(1, 14, 6)
    a64 = O.run_f64(14, desc)
    a32 = O.apply_f32(14, O.zero_state(14, np.complex64), desc)
    cmp = O.compare(a64, a32)
    assert cmp["max_abs_err"] < 1e-5
    assert cmp["one_minus_fidelity"] < 1e-9


def test_swap_is_three_cnots_and_relabels():
    n = 5
    psi = W.random_state(3, n).astype(np.complex128)
    out = O.apply_f64(n, psi, [(W.SWAP, 1, 3, -1, ())])
    idx = np.arange(1 << n)
    b1, b3 = (idx >> 1) & 1, (idx >> 3) & 1
    perm = idx ^ ((b1 ^ b3) << 1) ^ ((b1 ^ b3) << 3)
    np.testing.assert_allclose(out, psi[perm], atol=1e-15)


def test_oracle_rejects_bad_qubits():
    with pytest.raises(ValueError):
        O.apply_f64(3, O.zero_state(3), [(W.H, 5, -1, -1, ())])
    with pytest.raises(ValueError):
        O.apply_f64(3, O.zero_state(3), [(W.CNOT, 1, 1, -1, ())])


def test_prob_zero_matches_numpy():
    n = 10
    psi = W.random_state(5, n)
    for q in (0, 4, 9):
        p = O.lib.oracle_prob_zero_f32(n, psi.ctypes.data, q, 2)
        mask = ((np.arange(1 << n) >> q) & 1) == 0
        assert abs(p - np.sum(np.abs(psi[mask].astype(np.complex128)) ** 2)) < 1e-12


@pytest.mark.parametrize("n,width", [(12, 5), (18, 14), (19, 9)])
def test_blocked_application_is_bit_identical(n, width):
    """The cache-blocked FP64 application runs the same operations on every
    amplitude as the flat gate-by-gate one: identical bits, every gate type,
    controls inside and outside a block's qubits."""
    rng = W.SplitMix64(300 + n)
    desc = []
    for _ in range(250):
        t = rng.below(22)
        qs = rng.shuffle(list(range(n)))[:3]
        params = tuple(rng.uniform() * W.TWO_PI for _ in range(3))
        if t == W.CCX:
            desc.append((t, qs[2], qs[0], qs[1], ()))
        elif t <= W.CRZ:
            desc.append((t, qs[1], qs[0], -1, params[:1]))
        else:
            desc.append((t, qs[0], -1, -1, params))
    psi = W.random_state(9, n).astype(np.complex128)
    flat = O.apply_f64(n, psi, desc, blocked=False)
    arr, k = O.gate_structs(desc)
    blk = psi.copy()
    assert O.lib.oracle_apply_f64_blocked(n, blk.ctypes.data, arr, k, 4, width) == 0
    assert np.array_equal(flat, blk)


def test_compare_one_pass_matches_numpy():
    rng = np.random.default_rng(3)
    ref = (rng.normal(size=4096) + 1j * rng.normal(size=4096)).astype(np.complex128)
    got = (ref + 1e-4 * rng.normal(size=4096)).astype(np.complex64)
    fast = O.compare(ref, got)
    slow = O.compare(ref, got.astype(np.complex128))
    assert abs(fast["max_abs_err"] - slow["max_abs_err"]) < 1e-12
    assert abs(fast["one_minus_fidelity"] - slow["one_minus_fidelity"]) < 1e-9


def test_sampler_restatement_follows_the_cdf():
    """The oracle sampler (the sampler's FP64 summation order) lands every
    shot on an index whose CDF interval holds u * total."""
    n = 13
    a = W.random_state(4, n)
    a[::7] = 0
    shots = O.sample(a, 500, 77)
    p = np.abs(a.astype(np.complex128)) ** 2
    cdf = np.cumsum(p)
    u = O._mix64_uniforms(77, 500) * cdf[-1]
    lo = np.concatenate([[0.0], cdf[:-1]])[shots.astype(np.int64)]
    hi = cdf[shots.astype(np.int64)]
    assert np.all(p[shots.astype(np.int64)] > 0)
    assert np.all((u >= lo - 1e-12) & (u < hi + 1e-12))
