"""GPU parity: every CUDA path against the FP64 oracle (and the reference's own
fused-unitary outputs in tests/golden).  Tolerance for the complex64 state:
max |d amp| <= 1e-5 and 1 - fidelity <= 1e-6."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = 1e-5
FID = 1e-6
ALL_TYPES = list(range(22))
NPARAMS = {W.CRX: 1, W.CRY: 1, W.CU1: 1, W.CRZ: 1, W.U1: 1, W.U2: 2, W.U3: 3, W.RX: 1, W.RY: 1, W.RZ: 1}


def check(O, ref, got, tol=TOL):
    c = O.compare(ref, got)
    assert c["max_abs_err"] <= tol, c
    assert c["one_minus_fidelity"] <= FID, c
    return c


def random_circuit(seed, n, count, types=ALL_TYPES, qubits=None):
    rng = W.SplitMix64(seed)
    qubits = list(range(n)) if qubits is None else qubits
    desc = []
    for _ in range(count):
        t = types[rng.below(len(types))]
        qs = rng.shuffle(qubits)[:3]
        params = tuple(rng.uniform() * W.TWO_PI for _ in range(NPARAMS.get(t, 0)))
        if t == W.CCX:
            desc.append((t, qs[2], qs[0], qs[1], ()))
        elif t <= W.CRZ:
            desc.append((t, qs[1], qs[0], -1, params))
        else:
            desc.append((t, qs[0], -1, -1, params))
    return desc


def test_plain_u3_cnot_n20(hq, oracle):
    n = 20
    desc = W.plain_u3_cnot(1, n, 10)
    s = hq.State(n)
    s.apply_gates(W.to_gates(desc))
    check(oracle, oracle.run_f64(n, desc), s.store())
    assert abs(s.norm() - 1.0) < 1e-5


@pytest.mark.parametrize("backend", ["plain", "oshm"])
def test_graph_replay_matches_direct_run(hq, oracle, backend):
    """A captured CUDA graph replays the compiled schedule (for the plain path one
    kernel node per gate), including SWAPs folded into the layout."""
    n = 16
    desc = W.plain_u3_cnot(3, n, 6)
    desc = desc[:40] + [(W.SWAP, 2, 9, -1, ())] + desc[40:]
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend)
    s = hq.State(n)
    c.capture_graph(s)
    for _ in range(3):
        s.init_zero()
        c.run_on(s)
    check(oracle, oracle.run_f64(n, desc), s.store())


@pytest.mark.parametrize("backend,opts", [("oshm", {}), ("oshm", {"specialize": 0}), ("hybrid", {}),
                                          ("transmm", {"mm_qubits": 7}), ("plain", {})])
def test_serialized_schedule_runs_the_same(hq, oracle, backend, opts):
    """Schedule bytes (Schedule::serialize, src/schedule.cpp:156-325) give a
    circuit that runs exactly as the one compiled, without partitioning; bytes
    planned on the host load the same way."""
    n = 16
    desc = W.grid_random(6, 4, 4, 12)
    desc = desc[:50] + [(W.SWAP, 3, 12, -1, ())] + desc[50:]
    gates = W.to_gates(desc)
    c = hq.Circuit(n)
    c.addGates(gates)
    c.compile(backend, **opts)
    psi = W.random_state(61, n)
    s1 = hq.State(n, zero=False)
    s1.load(psi)
    c.run_on(s1)
    data = c.serialize()
    c2 = hq.Circuit.deserialize(data)
    assert c2.schedule() == c.schedule()
    s2 = hq.State(n, zero=False)
    s2.load(psi)
    c2.run_on(s2)
    assert np.array_equal(s1.store(), s2.store())
    c3 = hq.Circuit.deserialize(hq.plan_schedule(n, gates, backend=backend, **opts))
    s3 = hq.State(n, zero=False)
    s3.load(psi)
    c3.run_on(s3)
    assert np.array_equal(s1.store(), s3.store())
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s1.store(),
          tol=5e-5 if backend == "transmm" else TOL)


def test_async_readback_orders_with_later_writes(hq, oracle):
    """hq_state_store_async: the copy holds the state as it was when it was
    queued, even when a circuit, an init or a load writes the state right after;
    a circuit on another state runs meanwhile."""
    n = 20
    d1 = W.grid_random(7, 4, 5, 10)
    d2 = W.plain_u3_cnot(5, n, 4)
    c1, c2 = hq.Circuit(n), hq.Circuit(n)
    c1.addGates(W.to_gates(d1))
    c2.addGates(W.to_gates(d2))
    c1.compile("oshm")
    c2.compile("oshm")
    a, b = hq.State(n), hq.State(n)
    bufs = [hq.PinnedBuffer(1 << n) for _ in range(3)]
    c1.run_on(a)
    a.store_async(bufs[0].array)
    c2.run_on(a)                       # writes a: waits for the copy on the device
    c2.run_on(b)                       # another state: free to overlap
    b.store_async(bufs[1].array)
    a.store_async(bufs[2].array)
    a.init_zero()
    a.wait()
    b.wait()
    r1 = oracle.run_f64(n, d1)
    check(oracle, r1, bufs[0].array.copy())
    check(oracle, oracle.apply_f64(n, r1, d2), bufs[2].array.copy())
    check(oracle, oracle.run_f64(n, d2), bufs[1].array.copy())
    assert abs(a.amps([0])[0] - 1) < 1e-7
    for x in bufs:
        x.free()


def test_large_pinned_buffer_readback(hq):
    """Synchronous and asynchronous readbacks into a large pinned buffer match a
    readback into ordinary memory."""
    n = 24
    s = hq.State(n, zero=False)
    s.load(W.random_state(3, n))
    buf = hq.PinnedBuffer(1 << n)
    s.store(buf.array)
    plain = s.store()
    assert np.array_equal(buf.array, plain)
    buf.array[:] = 0
    s.store_async(buf.array)
    s.wait()
    assert np.array_equal(buf.array, plain)
    buf.free()


def test_deserialize_refuses_bad_bytes(hq):
    with pytest.raises(hq.HQError):
        hq.Circuit.deserialize(b"HQSC" + bytes(20))


@pytest.mark.parametrize("t", ALL_TYPES)
def test_plain_every_gate_type(hq, oracle, t):
    n = 9
    desc = random_circuit(100 + t, n, 12, types=[t])
    psi = W.random_state(7, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_gates(W.to_gates(desc))
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("t", ALL_TYPES)
def test_oshm_every_gate_type_in_and_out_of_tile(hq, oracle, t):
    """One OShareMem pass (n=15, 13-qubit tile {0..12}): controls and diagonal
    targets may sit outside the tile (qubits 13, 14)."""
    n = 15
    rng = W.SplitMix64(200 + t)
    tile = list(range(13))
    desc = []
    for _ in range(40):
        qs = rng.shuffle(range(n))
        diag = t in (W.CZ, W.CU1, W.CRZ, W.U1, W.Z, W.S, W.SDG, W.T, W.TDG, W.RZ)
        tq = qs[0] if diag else [q for q in qs if q in tile][0]
        others = [q for q in qs if q != tq]
        params = tuple(rng.uniform() * W.TWO_PI for _ in range(NPARAMS.get(t, 0)))
        if t == W.CCX:
            desc.append((t, tq, others[0], others[1], ()))
        elif t <= W.CRZ:
            desc.append((t, tq, others[0], -1, params))
        else:
            desc.append((t, tq, -1, -1, params))
    psi = W.random_state(9, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_oshm_group(W.to_gates(desc), (1 << 13) - 1)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


def every_placement(n, seed):
    """Every gate type at every target and every control position (CCX with a
    rotating second control), parameters seeded."""
    rng = W.SplitMix64(seed)
    desc = []
    for t in ALL_TYPES:
        for tq in range(n):
            params = tuple(rng.uniform() * W.TWO_PI for _ in range(NPARAMS.get(t, 0)))
            if t == W.CCX:
                for c in range(n):
                    c2 = (c + 1 + tq) % n
                    if c != tq and c2 not in (tq, c):
                        desc.append((t, tq, c, c2, ()))
            elif t <= W.CRZ:
                for c in range(n):
                    if c != tq:
                        desc.append((t, tq, c, -1, params))
            else:
                desc.append((t, tq, -1, -1, params))
    return desc


@pytest.mark.parametrize("tile,specialize", [(10, 2), (12, 2), (10, 0)])
def test_every_gate_at_every_position_compiled(hq, oracle, tile, specialize):
    """Exhaustive placements on 12 qubits through the compiled OShareMem path:
    targets and controls inside and outside the tile, on the vector lane, in a
    warp and across warps (12-qubit tiles run 4 warps), generated kernels and
    the interpreter."""
    n = 12
    desc = every_placement(n, 1234)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm", tile_qubits=tile, specialize=specialize)
    psi = W.random_state(77, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("seed", range(6))
def test_oshm_scattered_tile(hq, oracle, seed):
    """Tile = qubit 0 + 12 random qubits of 18; gates of every type with
    non-diagonal targets in the tile, diagonal ones anywhere."""
    n = 18
    rng = W.SplitMix64(300 + seed)
    tile = sorted([0] + rng.shuffle(range(1, n))[:12])
    diag_types = [W.CZ, W.CU1, W.CRZ, W.U1, W.Z, W.S, W.SDG, W.T, W.TDG, W.RZ]
    desc = random_circuit(400 + seed, n, 150, types=[t for t in ALL_TYPES if t not in diag_types],
                          qubits=tile)
    desc += random_circuit(500 + seed, n, 60, types=diag_types)
    order = rng.shuffle(range(len(desc)))
    desc = [desc[i] for i in order]
    mask = sum(1 << q for q in tile)
    psi = W.random_state(11 + seed, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_oshm_group(W.to_gates(desc), mask)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("backend,tile,prec", [
    ("oshm", 13, "bf16x3"), ("oshm", 10, "bf16x3"), ("oshm", 8, "bf16x3"),
    ("transmm", 0, "fp32"), ("transmm", 0, "bf16x3"), ("hybrid", 13, "fp32"),
    ("hybrid", 13, "bf16x3"), ("plain", 0, "fp32")])
@pytest.mark.parametrize("n", [16, 20])
def test_compiled_random_circuits(hq, oracle, backend, tile, prec, n):
    desc = random_circuit(600 + n, n, 400)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend=backend, tile_qubits=tile, precision=prec)
    psi = W.random_state(13, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("n", [6, 7, 8])
def test_golden_reference_outputs(hq, oracle, n):
    """The reference's own fused-unitary result for the same circuit."""
    z = np.load(GOLDEN / f"unitary_n{n}.npz")
    desc = [tuple(x[:4]) + (tuple(x[4]),) for x in json.loads(str(z["desc"]))]
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend="oshm", tile_qubits=n)
    s = hq.State(n, zero=False)
    s.load(z["psi"].astype(np.complex64))
    c.run_on(s)
    check(oracle, z["out_psi"], s.store())
    c.run()
    check(oracle, z["out_zero"], c.result)


def test_swap_folding_and_logical_readout(hq, oracle):
    n = 14
    desc = random_circuit(700, n, 120)
    desc.insert(40, (W.SWAP, 2, 11, -1, ()))
    desc.insert(90, (W.SWAP, 0, 5, -1, ()))
    desc.append((W.SWAP, 3, 13, -1, ()))
    ref = oracle.run_f64(n, desc)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend="oshm", tile_qubits=10)
    c.run(copy_back=False, destroy=False)
    assert c.state.layout() != list(range(n))
    idx = np.array([0, 1, 5, 77, 1000, (1 << n) - 1], dtype=np.uint64)
    got = c.state.amps(idx)
    np.testing.assert_allclose(got, ref[idx.astype(np.int64)], atol=TOL)
    for q in (0, 2, 11):
        p0 = np.sum(np.abs(ref[((np.arange(1 << n) >> q) & 1) == 0]) ** 2)
        assert abs(c.state.prob_zero(q) - p0) < 1e-6
    m = c.state.marginals()
    for q in range(n):
        p1 = np.sum(np.abs(ref[((np.arange(1 << n) >> q) & 1) == 1]) ** 2)
        assert abs(m[q] - p1) < 1e-6
    check(oracle, ref, c.state.store())
    assert c.state.layout() == list(range(n))


def test_marginals_large_state(hq, oracle):
    n = 26  # two reduction levels
    psi = W.random_state(21, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    p = np.abs(psi.astype(np.complex128)) ** 2
    assert abs(s.norm() - p.sum()) < 1e-9
    m = s.marginals()
    idx = np.arange(1 << n)
    for q in (0, 1, 11, 12, 23, 24, 25):
        assert abs(m[q] - p[((idx >> q) & 1) == 1].sum()) < 1e-9


def test_group_unitary_fp64_matches_oracle(hq, oracle):
    desc = random_circuit(800, 7, 90)
    U = hq.group_unitary(W.to_gates(desc), (1 << 7) - 1)
    np.testing.assert_allclose(U, oracle.group_unitary(list(range(7)), desc), atol=1e-12)


# TransMM tolerances per arithmetic: BF16x3 and FP32 meet the 1e-5 bar; TF32
# (10-bit mantissa) is the low-precision comparison variant.
MM_TOL = {"fp32": (TOL, FID), "bf16x3": (TOL, FID), "tf32": (5e-5, 1e-5)}


@pytest.mark.parametrize("prec,m", [("fp32", 4), ("fp32", 5), ("fp32", 6), ("fp32", 7),
                                    ("bf16x3", 4), ("bf16x3", 6), ("tf32", 6), ("bf16x3", 7),
                                    ("tf32", 7), ("fp32", 8), ("bf16x3", 8), ("tf32", 8)])
def test_transmm_single_group(hq, oracle, prec, m):
    n = 17
    rng = W.SplitMix64(900 + m)
    qubits = sorted(rng.shuffle(range(n))[:m])
    desc = random_circuit(910 + m, n, 30 * m, qubits=qubits)
    psi = W.random_state(17, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_transmm_group(W.to_gates(desc), sum(1 << q for q in qubits), prec)
    tol, fid = MM_TOL[prec]
    c = oracle.compare(oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())
    assert c["max_abs_err"] <= tol and c["one_minus_fidelity"] <= fid, c


@pytest.mark.parametrize("prec", ["bf16x3", "tf32", "fp32"])
def test_transmm_8_qubit_group_many_subtiles(hq, oracle, prec):
    """An 8-qubit group on 22 qubits: 1024 sub-tiles over at most one CTA per SM,
    so every CTA runs several sub-tiles and its operand ring wraps."""
    n = 22
    qubits = [0, 3, 5, 9, 12, 16, 19, 21]
    desc = random_circuit(960, n, 200, qubits=qubits)
    psi = W.random_state(23, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_transmm_group(W.to_gates(desc), sum(1 << q for q in qubits), prec)
    tol, fid = MM_TOL[prec]
    c = oracle.compare(oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())
    assert c["max_abs_err"] <= tol and c["one_minus_fidelity"] <= fid, c


@pytest.mark.parametrize("prec", ["bf16x3", "fp32"])
def test_apply_caller_unitary_narrow_group(hq, oracle, prec):
    """A 3-qubit unitary given by the caller, widened to the contraction width."""
    n = 15
    qubits = [2, 7, 11]
    desc = random_circuit(950, n, 40, qubits=qubits)
    U = oracle.group_unitary(qubits, desc)
    psi = W.random_state(19, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    s.apply_unitary(U, sum(1 << q for q in qubits), prec)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("prec,k", [("bf16x3", 6), ("tf32", 6), ("fp32", 6), ("bf16x3", 7),
                                    ("tf32", 7), ("fp32", 7), ("bf16x3", 8), ("tf32", 8),
                                    ("fp32", 8)])
def test_transmm_qft_precision_sweep(hq, oracle, prec, k):
    """The QFT precision sweep at a size the oracle finishes: QFT on a random state,
    TransMM groups of k qubits only, per arithmetic."""
    n = 18
    desc = W.qft(n)
    psi = W.random_state(31, n)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend="transmm", precision=prec, mm_qubits=k)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    tol, fid = MM_TOL[prec]
    r = oracle.compare(oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())
    assert r["max_abs_err"] <= tol and r["one_minus_fidelity"] <= fid, r


def clifford_t_circuit(seed, n, count):
    """Gates the generated kernels run in closed form: H, sqrt(X) / sqrt(Y) as
    RX / RY(pi/2), T, T^dagger, S, X, Z and their controlled forms, CZ."""
    rng = W.SplitMix64(seed)
    half = math.pi / 2
    out = []
    for _ in range(count):
        qs = rng.shuffle(range(n))[:3]
        k = rng.below(12)
        if k == 0:
            out.append((W.H, qs[0], -1, -1, ()))
        elif k == 1:
            out.append((W.RX, qs[0], -1, -1, (half,)))
        elif k == 2:
            out.append((W.RY, qs[0], -1, -1, (half,)))
        elif k == 3:
            out.append((W.T, qs[0], -1, -1, ()))
        elif k == 4:
            out.append((W.TDG, qs[0], -1, -1, ()))
        elif k == 5:
            out.append((W.S, qs[0], -1, -1, ()))
        elif k == 6:
            out.append((W.X, qs[0], -1, -1, ()))
        elif k == 7:
            out.append((W.CZ, qs[1], qs[0], -1, ()))
        elif k == 8:
            out.append((W.CNOT, qs[1], qs[0], -1, ()))
        elif k == 9:
            out.append((W.CRX, qs[1], qs[0], -1, (half,)))
        elif k == 10:
            out.append((W.CU1, qs[1], qs[0], -1, (math.pi / 4,)))
        else:
            out.append((W.U1, qs[0], -1, -1, (-3 * math.pi / 4,)))
    return out


@pytest.mark.parametrize("n,seed", [(14, 1), (17, 2), (20, 3)])
def test_generated_kernels_clifford_t(hq, oracle, n, seed):
    """Closed-form gates in the generated kernels (per-vector scales: T as one add
    per component, H / sqrt(X) / sqrt(Y) absorbing scale ratios) against the oracle."""
    desc = clifford_t_circuit(700 + seed, n, 600)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm")
    psi = W.random_state(40 + seed, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


def lane_heavy_circuit(seed, n, count):
    """Half of the gates on physical qubit 0 (the packed vectors' lane): the
    closed forms and scale bookkeeping of gates there (T and T^dagger as one
    add on the high lane, H / sqrt(X) / sqrt(Y), real and imaginary
    off-diagonal 2x2s and general ones absorbing the lanes' scale ratio, sign
    flips folded into a lane's scale, lane exchanges under register and
    run-time controls), mixed with the same gates on the other qubits."""
    rng = W.SplitMix64(seed)
    half = math.pi / 2
    out = []
    for _ in range(count):
        qs = list(rng.shuffle(range(n))[:3])
        if rng.below(2) == 0:
            j = rng.below(2)
            if 0 in qs:
                qs.remove(0)
            qs.insert(j, 0)
        k = rng.below(16)
        th = rng.uniform() * W.TWO_PI
        one = [(W.H, ()), (W.RX, (half,)), (W.RY, (half,)), (W.T, ()), (W.TDG, ()), (W.S, ()),
               (W.X, ()), (W.Z, ()), (W.Y, ()), (W.RY, (th,)), (W.RX, (th,)),
               (W.U3, (th, 0.3, 1.1))]
        if k < len(one):
            t, p = one[k]
            out.append((t, qs[0], -1, -1, p))
        elif k == 12:
            out.append((W.CZ, qs[1], qs[0], -1, ()))
        elif k == 13:
            out.append((W.CNOT, qs[1], qs[0], -1, ()))
        elif k == 14:
            out.append((W.CNOT, qs[0], qs[1], -1, ()))
        else:
            out.append((W.CU1, qs[0], qs[1], -1, (math.pi / 4,)))
    return out


@pytest.mark.parametrize("specialize", [0, 1])
@pytest.mark.parametrize("n,seed,tile", [(9, 1, 8), (14, 2, 10), (17, 3, 13)])
def test_lane_heavy_circuits(hq, oracle, n, seed, tile, specialize):
    desc = lane_heavy_circuit(800 + seed, n, 700)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm", tile_qubits=tile, specialize=specialize)
    psi = W.random_state(50 + seed, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    check(oracle, oracle.apply_f64(n, psi.astype(np.complex128), desc), s.store())


@pytest.mark.parametrize("rows,cols", [(4, 4), (3, 6)])
def test_grid_circuit_small_vs_oracle(hq, oracle, rows, cols):
    n = rows * cols
    desc = W.grid_random(5, rows, cols, 20)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm")
    s = hq.State(n)
    c.run_on(s)
    check(oracle, oracle.run_f64(n, desc), s.store())


@pytest.mark.parametrize("rows,cols", [(4, 6), (2, 13)])
def test_grid_circuit_24_26_vs_oracle(hq, oracle, rows, cols):
    """The headline circuit family at 24 and 26 qubits (20 cycles, the
    generated OShareMem kernels at the default 13-qubit tiles) against the
    FP64 gate-by-gate oracle on the whole state."""
    n = rows * cols
    desc = W.grid_random(2, rows, cols, 20)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm")
    s = hq.State(n)
    c.run_on(s)
    got = s.store()
    s.free()
    check(oracle, oracle.run_f64(n, desc), got)


def inverse(desc):
    inv = {W.T: W.TDG, W.TDG: W.T, W.S: W.SDG, W.SDG: W.S}
    out = []
    for (t, q, c, c2, p) in reversed(desc):
        if t in (W.RX, W.RY, W.RZ, W.CU1, W.U1, W.CRX, W.CRY, W.CRZ):
            out.append((t, q, c, c2, (-p[0],)))
        else:
            out.append((inv.get(t, t), q, c, c2, p))
    return out


def test_grid30_oshm_vs_plain_full_size(hq, oracle):
    """The 30-qubit grid circuit at full size (8 GiB): the OShareMem schedule and the plain
    per-gate path are independent CUDA paths; they must agree, and the state
    must stay normalised."""
    n = 30
    desc = W.grid_random(2, 5, 6, 20)
    gates = W.to_gates(desc)
    c = hq.Circuit(n)
    c.addGates(gates)
    c.compile(backend="oshm")
    s1 = hq.State(n)
    c.run_on(s1)
    assert abs(s1.norm() - 1.0) < 1e-4
    s2 = hq.State(n)
    s2.apply_gates(gates)
    idx = np.concatenate([np.arange(4096), np.array(W.SplitMix64(5).shuffle(range(1 << 20))[:4096]) << 10])
    idx = idx.astype(np.uint64)
    a, b = s1.amps(idx), s2.amps(idx)
    assert np.max(np.abs(a - b)) < TOL
    m1, m2 = s1.marginals(), s2.marginals()
    assert np.max(np.abs(m1 - m2)) < 1e-5
    # round trip: circuit followed by its inverse returns |0..0>
    ci = hq.Circuit(n)
    ci.addGates(W.to_gates(inverse(desc)))
    ci.compile(backend="oshm")
    ci.run_on(s1)
    amp0 = s1.amps(np.array([0], dtype=np.uint64))[0]
    assert abs(abs(amp0) ** 2 - 1.0) < 1e-4


def test_qft28_analytic_amplitudes(hq, oracle):
    """QFT |x> has amplitudes exp(2 pi i x k / N) / sqrt(N) (with the final
    swaps); checked on sampled k at 28 qubits, a size-independent property."""
    n = 28
    x = 0x5A3C1F7
    desc = [(W.X, q, -1, -1, ()) for q in range(n) if (x >> q) & 1] + W.qft(n)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend="oshm")
    s = hq.State(n)
    c.run_on(s)
    ks = np.array([0, 1, 2, 12345, (1 << n) - 1] + W.SplitMix64(9).shuffle(range(1 << 20))[:64],
                  dtype=np.uint64)
    got = s.amps(ks)
    N = float(1 << n)
    ref = np.exp(2j * np.pi * ((x * ks.astype(np.float64)) % N) / N) / math.sqrt(N)
    assert np.max(np.abs(got - ref)) < 1e-6


def test_max_size_34_qubits(hq, oracle):
    """The largest register on one GB300 (2^34 amplitudes, 128 GiB): 64-bit
    indexing through the OShareMem path, the readout, the FP64 reductions and
    the sampler.  H on every qubit, RZ on every qubit and CZ on a matching give
    amp(x) = 2^(-n/2) prod_q exp(-+i theta_q/2) prod_(a,b) (-1)^(x_a x_b);
    the inverse circuit then returns |0...0>."""
    n = 34
    rng = W.SplitMix64(34)
    theta = [rng.uniform() * W.TWO_PI for _ in range(n)]
    pairs = [(2 * i, 2 * i + 1) for i in range(n // 2)]
    desc = [(W.H, q, -1, -1, ()) for q in range(n)]
    desc += [(W.RZ, q, -1, -1, (theta[q],)) for q in range(n)]
    desc += [(W.CZ, b, a, -1, ()) for a, b in pairs]
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile(backend="oshm")
    s = hq.State(n)
    c.run_on(s)
    xs = np.array([0, 1, (1 << n) - 1, 0x2_5A5A_5A5A] + [int(v) << 11 | 0x3FF for v in
                   W.SplitMix64(7).shuffle(range(1 << 20))[:60]], dtype=np.uint64)
    got = s.amps(xs)
    for x, a in zip(xs.tolist(), got):
        ph = sum((theta[q] / 2) * (1 if (x >> q) & 1 else -1) for q in range(n))
        sign = (-1) ** sum(((x >> p) & 1) & ((x >> q) & 1) for p, q in pairs)
        ref = sign * np.exp(1j * ph) / math.sqrt(2.0 ** n)
        assert abs(a - ref) < 1e-9 + 1e-5 * abs(ref)
    assert abs(s.norm() - 1.0) < 1e-4
    assert np.max(np.abs(s.marginals() - 0.5)) < 1e-4
    shots = s.sample(64, seed=3)
    assert shots.size == 64 and int(shots.max()) < (1 << n)
    ci = hq.Circuit(n)
    ci.addGates(W.to_gates(inverse(desc)))
    ci.compile(backend="oshm")
    ci.run_on(s)
    amp0 = s.amps(np.array([0], dtype=np.uint64))[0]
    assert abs(abs(amp0) ** 2 - 1.0) < 1e-4
    s.free()


def test_blocked_circuit_hybrid_takes_transmm(hq, oracle):
    """Deep dense 7-qubit blocks: the hybrid partitioner fuses blocks into
    TransMM groups (the reference's mix mode, src/compiler.cpp:248-280) and the
    mixed schedule matches the FP64 oracle."""
    n = 21
    desc = W.blocked_u3_cnot(11, n, 7, 10, 2)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("hybrid")
    kinds = [b for (b, _, _, _) in c.schedule()]
    assert hq.BACKEND_TRANSMM in kinds and hq.BACKEND_OSHM in kinds, kinds
    s = hq.State(n)
    s.init_zero()
    c.run_on(s)
    check(oracle, oracle.run_f64(n, desc), s.store())
