"""Serving (request loop with admission and continuous batching) and the
sampler, against the FP64 oracle.  A request's result must be the same when it
runs alone and when it runs in a mix of concurrent requests."""
import time

import numpy as np
import pytest

import hyquas_gb300 as hqmod
from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5
FID = 1e-6


def check(O, ref, got, tol=TOL):
    c = O.compare(ref, got)
    assert c["max_abs_err"] <= tol, c
    assert c["one_minus_fidelity"] <= FID, c
    return c


def drain(sv, ids, timeout=120.0):
    """Wait for every id; returns {id: amplitudes}, releasing each result."""
    out = {}
    t_end = time.time() + timeout
    pending = set(ids)
    while pending and time.time() < t_end:
        for rid in sv.poll():
            if rid in pending:
                assert sv.wait(rid, 0) == "done"
                out[rid] = sv.state(rid).store()
                sv.release(rid)
                pending.discard(rid)
        time.sleep(0.001)
    assert not pending, f"requests did not finish: {sorted(pending)[:5]}"
    return out


def test_served_results_match_oracle(hq, oracle):
    stream = W.served_stream(seed=7, count=16, rate=1000.0, nmin=10, nmax=16, dmin=4, dmax=12)
    sv = hq.Server()
    ids = [sv.submit(n, W.to_gates(desc)) for _, n, desc in stream]
    got = drain(sv, ids)
    for rid, (_, n, desc) in zip(ids, stream):
        check(oracle, oracle.run_f64(n, desc), got[rid])
        s, a, d = sv.times(rid)
        assert 0 <= s <= a <= d
    st = sv.stats()
    assert st["finished"] == len(ids) and st["steps"] >= 1 and st["resident_bytes"] == 0
    sv.close()


def test_same_alone_and_in_mix(hq, oracle):
    rng = W.SplitMix64(71)
    probe = (18, W.ry_rz_cz(rng, 18, 30))
    others = [(n, W.ry_rz_cz(rng, n, 20 + rng.below(20))) for n in
              [22, 20, 15, 21, 13, 22, 16, 14, 20, 17, 12, 18]]
    sv = hq.Server(step_budget_us=100.0)  # many short steps, shared by the requests
    arrays = [hq.gate_array(W.to_gates(d)) for _, d in others]
    parr = hq.gate_array(W.to_gates(probe[1]))
    alone_id = sv.submit(probe[0], parr)
    alone = drain(sv, [alone_id])[alone_id]
    ids = [sv.submit(n, a) for (n, _), a in zip(others[:6], arrays[:6])]
    mix_id = sv.submit(probe[0], parr)
    ids += [sv.submit(n, a) for (n, _), a in zip(others[6:], arrays[6:])]
    res = drain(sv, ids + [mix_id])
    assert np.array_equal(alone, res[mix_id])  # same program, same arithmetic
    check(oracle, oracle.run_f64(*probe), res[mix_id])
    for rid, (n, d) in zip(ids, others):
        check(oracle, oracle.run_f64(n, d), res[rid])
    # the probe shared batched launches with other requests
    f, l = sv.steps(mix_id)
    shared = sum(1 for rid in ids if sv.steps(rid)[0] <= l and sv.steps(rid)[1] >= f)
    assert shared >= 1
    assert sv.steps(alone_id)[0] >= 0
    sv.close()


def test_admission_respects_budget(hq, oracle):
    n = 16
    budget = 2 * (8 << n)  # two resident states at a time
    sv = hq.Server(hbm_budget=budget)
    rng = W.SplitMix64(81)
    circs = [W.ry_rz_cz(rng, n, 6) for _ in range(6)]
    ids = [sv.submit(n, W.to_gates(c)) for c in circs]
    time.sleep(0.5)
    # results are held until released: at most two can have been admitted
    st = sv.stats()
    assert st["peak_resident_bytes"] <= budget
    done_now = [rid for rid in ids if sv.wait(rid, 0) == "done"]
    assert len(done_now) <= 2
    got = drain(sv, ids)
    for rid, c in zip(ids, circs):
        check(oracle, oracle.run_f64(n, c), got[rid])
    assert sv.stats()["peak_resident_bytes"] <= budget
    sv.close()


def test_served_rejects_bad_requests(hq):
    sv = hq.Server(hbm_budget=1 << 20)
    with pytest.raises(hq.HQError):
        sv.submit(18, [])  # 2 MiB state > 1 MiB budget
    with pytest.raises(hq.HQError):
        sv.submit(12, [hq.Gate.H(12)])
    with pytest.raises(hq.HQError):
        sv.submit(8, [])
    rid = sv.submit(12, [])  # gate-less: |0...0>
    assert sv.wait(rid, 30) == "done"
    a = sv.state(rid).store()
    assert a[0] == 1 and np.count_nonzero(a) == 1
    sv.release(rid)
    with pytest.raises(hq.HQError):
        sv.release(rid)
    sv.close()


@pytest.mark.parametrize("n", [10, 14, 19])
def test_sampler_matches_oracle(hq, oracle, n):
    desc = W.ry_rz_cz(W.SplitMix64(90 + n), n, 6)
    s = hq.State(n)
    s.apply_gates(W.to_gates(desc))
    amps = s.store()
    got = s.sample(3000, seed=1234 + n)
    ref = oracle.sample(amps, 3000, 1234 + n)
    # the oracle adds the FP64 probabilities in the sampler's order: every index agrees
    assert np.array_equal(got, ref), np.nonzero(got != ref)[0][:10]
    # outcome frequencies follow |amp|^2
    p = np.abs(amps.astype(np.complex128)) ** 2
    assert np.all(p[got.astype(np.int64)] > 0)


def test_sampler_honours_layout(hq, oracle):
    n = 12
    desc = W.ry_rz_cz(W.SplitMix64(5), n, 4) + [(W.SWAP, 0, 11, -1, ()), (W.SWAP, 2, 5, -1, ())]
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm", specialize=0)
    s = hq.State(n)
    c.run_on(s)
    assert s.layout() != list(range(n))
    got = s.sample(2000, seed=9)
    ref = oracle.sample(oracle.run_f64(n, desc).astype(np.complex64), 2000, 9)
    assert np.mean(got == ref) >= 0.99


def test_plan_cache_reuses_plans(hq, oracle):
    """A circuit submitted again is not planned again, and gives the same result."""
    rng = W.SplitMix64(123)
    desc = W.ry_rz_cz(rng, 16, 12)
    arr = hq.gate_array(W.to_gates(desc))
    sv = hq.Server()
    first = sv.submit(16, arr)
    a = drain(sv, [first])[first]
    assert sv.plan_cache()["entries"] >= 1
    second = sv.submit(16, arr)
    b = drain(sv, [second])[second]
    assert sv.plan_cache()["hits"] >= 1
    assert np.array_equal(a, b)
    check(oracle, oracle.run_f64(16, desc), b)
    sv.close()


def test_generated_kernel_lane(hq, oracle):
    """Requests at or above jit_min_qubits run generated group kernels between
    the batched launches; their results match the oracle and the small
    requests served beside them."""
    rng = W.SplitMix64(131)
    circuits = [(n, W.ry_rz_cz(rng, n, 8 + rng.below(8))) for n in [12, 16, 15, 17, 13, 16]]
    sv = hq.Server(jit_min_qubits=15)
    arrays = [hq.gate_array(W.to_gates(d)) for _, d in circuits]
    ids = [sv.submit(n, a) for (n, _), a in zip(circuits, arrays)]
    got = drain(sv, ids, timeout=300.0)
    for rid, (n, d) in zip(ids, circuits):
        check(oracle, oracle.run_f64(n, d), got[rid])
    sv.close()
