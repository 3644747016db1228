"""Batched execution (one persistent launch over many circuits) against the
FP64 oracle and against each circuit run alone.  Same error bar as the single
circuit paths: max |d amp| <= 1e-5, 1 - fidelity <= 1e-6."""
import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5
FID = 1e-6


def check(O, ref, got, tol=TOL):
    c = O.compare(ref, got)
    assert c["max_abs_err"] <= tol, c
    assert c["one_minus_fidelity"] <= FID, c
    return c


def make_batch(hq, circuits, zero=True, tile_qubits=0):
    b = hq.Batch()
    states, circs = [], []
    for n, desc in circuits:
        c = hq.Circuit(n)
        c.addGates(W.to_gates(desc))
        s = hq.State(n, zero=zero)
        b.add(c, s)
        states.append(s)
        circs.append(c)
    b.compile(tile_qubits=tile_qubits)
    return b, states, circs


def small_mix(seed=11, count=12, nmin=10, nmax=15, dmin=4, dmax=10):
    return W.batched(seed, count, nmin, nmax, dmin, dmax)


def test_batch_matches_oracle_zero_init(hq, oracle):
    circuits = small_mix()
    b, states, _ = make_batch(hq, circuits)
    info = b.info()
    assert info["circuits"] == len(circuits)
    assert info["items"] > 0 and info["groups"] >= len(circuits)
    assert all(10 <= k <= 13 for k in info["tile_qubits"])
    b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        check(oracle, oracle.run_f64(n, desc), s.store())


@pytest.mark.parametrize("tile", [10, 11, 12, 13])
def test_batch_fixed_tile_widths(hq, oracle, tile):
    circuits = small_mix(seed=20 + tile, count=6, nmin=13, nmax=16)
    b, states, _ = make_batch(hq, circuits, tile_qubits=tile)
    assert all(k == tile for k in b.info()["tile_qubits"])
    b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        check(oracle, oracle.run_f64(n, desc), s.store())


def test_batch_loaded_states(hq, oracle):
    """zero_init=False: each circuit acts on the amplitudes already in its state."""
    circuits = small_mix(seed=31, count=8)
    b, states, _ = make_batch(hq, circuits, zero=False)
    inits = []
    for i, ((n, _), s) in enumerate(zip(circuits, states)):
        psi = W.random_state(100 + i, n)
        s.load(psi)
        inits.append(psi)
    b.run(zero_init=False)
    for (n, desc), s, psi in zip(circuits, states, inits):
        check(oracle, oracle.run_f64(n, desc, init=psi), s.store())


def test_batch_same_as_alone(hq, oracle):
    """Each circuit's result in the batch equals its result run alone."""
    circuits = small_mix(seed=41, count=16, nmin=10, nmax=18, dmin=6, dmax=16)
    b, states, _ = make_batch(hq, circuits)
    b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        c = hq.Circuit(n)
        c.addGates(W.to_gates(desc))
        c.compile("oshm", specialize=0)
        alone = hq.State(n)
        c.run_on(alone)
        ref = alone.store()
        got = s.store()
        assert np.max(np.abs(ref.astype(np.complex128) - got)) <= 1e-6


def test_batch_graph_replay_and_rerun(hq, oracle):
    circuits = small_mix(seed=51, count=10)
    b, states, _ = make_batch(hq, circuits)
    b.capture_graph(zero_init=True)
    for _ in range(3):  # replays start from |0> each time
        b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        check(oracle, oracle.run_f64(n, desc), s.store())


def test_batch_swaps_small_and_empty(hq, oracle):
    """SWAPs fold into the layout; circuits under 10 qubits run gate by gate;
    a gate-less circuit leaves |0...0>."""
    rng = W.SplitMix64(61)
    big = W.ry_rz_cz(rng, 12, 5)
    big = big[:20] + [(W.SWAP, 0, 11, -1, ())] + big[20:] + [(W.SWAP, 3, 7, -1, ())]
    small = W.ry_rz_cz(rng, 7, 4)
    circuits = [(12, big), (7, small), (11, [])]
    b, states, _ = make_batch(hq, circuits)
    b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        check(oracle, oracle.run_f64(n, desc), s.store())


def test_batch_rejects_mismatch(hq):
    b = hq.Batch()
    c = hq.Circuit(12)
    s = hq.State(11)
    with pytest.raises(hq.HQError):
        b.add(c, s)
    with pytest.raises(hq.HQError):
        b.run()  # not compiled


def test_batch_512_circuits_full(hq, oracle):
    """The 512-circuit workload (n 10-22, depth 8-40): every state normalised,
    a sample of circuits bit-for-bit equal to their solo runs, the smallest ones
    against the oracle."""
    circuits = W.batched()
    b, states, _ = make_batch(hq, circuits)
    b.run(zero_init=True)
    norms = [s.norm() for s in states]
    assert max(abs(x - 1.0) for x in norms) < 1e-4
    order = sorted(range(len(circuits)), key=lambda i: circuits[i][0])
    for i in order[:6]:
        n, desc = circuits[i]
        check(oracle, oracle.run_f64(n, desc), states[i].store())
    for i in order[-3:]:
        n, desc = circuits[i]
        c = hq.Circuit(n)
        c.addGates(W.to_gates(desc))
        c.compile("oshm", specialize=0)
        alone = hq.State(n)
        c.run_on(alone)
        assert np.max(np.abs(alone.store().astype(np.complex128) - states[i].store())) <= 1e-6


def test_batch_bounded_wait_reports_timeout(hq, oracle):
    """Failure detection without a GPU fault: an item made to wait for a count
    that is never reached gives up after its bounded wait; the run returns
    HQ_ERR_TIMEOUT and the next run of the same batch is correct."""
    import time
    circuits = small_mix(seed=91, count=4, nmin=14, nmax=15, dmin=10, dmax=12)
    b, states, _ = make_batch(hq, circuits)
    assert b.info()["groups"] > len(circuits)  # some items wait on a predecessor
    b.inject_stall()
    t0 = time.time()
    with pytest.raises(hq.HQError) as e:
        b.run(zero_init=True)
    assert e.value.code == -5  # HQ_ERR_TIMEOUT
    assert time.time() - t0 < 30
    b.run(zero_init=True)
    for (n, desc), s in zip(circuits, states):
        check(oracle, oracle.run_f64(n, desc), s.store())


def test_batch_empty_and_single_tile(hq, oracle):
    """An empty batch runs as a no-op; a lone 10-qubit circuit is one tile and
    one group (every qubit local)."""
    b = hq.Batch()
    b.compile()
    assert b.info()["circuits"] == 0 and b.info()["items"] == 0
    b.run()
    circuits = [(10, W.ry_rz_cz(W.SplitMix64(101), 10, 12))]
    b2, states, _ = make_batch(hq, circuits)
    info = b2.info()
    assert info["groups"] == 1 and info["items"] == 1 and info["tile_qubits"] == [10]
    b2.run()
    check(oracle, oracle.run_f64(*circuits[0]), states[0].store())
