"""Compiled-schedule bytes on the host (no GPU): the reference serialises its
Schedule for broadcast (Schedule/GateGroup/State::serialize,
src/schedule.cpp:156-325; Gate::serialize, src/gate.cpp:558-589).  Here the
bytes must carry exactly the partition compile makes, be deterministic, and
be refused when damaged."""
import ctypes as C
import struct

import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W

HQ_ERR_INVALID = -1
HQ_ERR_UNSUPPORTED = -6


def planned_groups(n, gates, **opts):
    """hq_plan_groups: the partition compile makes, for comparison."""
    arr = hq.gate_array(gates)
    o = hq._compile_options(**opts)
    k = max(1, len(gates))
    ng = C.c_int32()
    b, g, w = (C.c_int32 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
    rel, ph, order = (C.c_uint64 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
    hq.check(hq.lib.hq_plan_groups(n, arr, len(gates), C.byref(o), C.byref(ng), b, g, w, rel, ph,
                                   order))
    return [(b[i], g[i], w[i], rel[i]) for i in range(ng.value)]


def fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    for x in data:
        h ^= x
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def reseal(body: bytes) -> bytes:
    """Bytes with a fresh checksum (to plant a bad field past the checksum test)."""
    return body + struct.pack("<Q", fnv1a(body))


def cases():
    rng = W.SplitMix64(77)
    grid = W.grid_random(3, 4, 5, 12)
    swapped = grid[:30] + [(W.SWAP, 1, 17, -1, ())] + grid[30:]
    return [
        ("grid20", 20, W.to_gates(grid), {}),
        ("grid20_swaps", 20, W.to_gates(swapped), {}),
        ("random16_tile10", 16, W.to_gates(W.ry_rz_cz(rng, 16, 20)), {"tile_qubits": 10}),
        ("qft18_transmm", 18, W.to_gates(W.qft(18)), {"backend": "transmm", "mm_qubits": 7}),
        ("qft18_hybrid", 18, W.to_gates(W.qft(18)), {"backend": "hybrid"}),
        ("reference12", 12, W.to_gates(W.ry_rz_cz(rng, 12, 10)), {"reference_grouping": True}),
    ]


@pytest.mark.parametrize("name,n,gates,opts", cases(), ids=[c[0] for c in cases()])
def test_bytes_carry_the_partition(name, n, gates, opts):
    data = hq.plan_schedule(n, gates, **opts)
    assert data[:4] == b"HQSC"
    info = hq.inspect_schedule(data)
    assert info["num_qubits"] == n and info["num_gates"] == len(gates)
    assert info["groups"] == planned_groups(n, gates, **opts)
    assert hq.plan_schedule(n, gates, **opts) == data  # deterministic


def test_plain_and_interpreter_plans():
    n = 14
    gates = W.to_gates(W.ry_rz_cz(W.SplitMix64(5), n, 12))
    plain = hq.inspect_schedule(hq.plan_schedule(n, gates, backend="plain"))
    assert plain["groups"] == [] and plain["num_gates"] == len(gates)
    # the interpreter plan fuses runs of single-qubit gates before grouping
    fused = hq.inspect_schedule(hq.plan_schedule(n, gates, specialize=0))
    assert sum(g for (_, g, _, _) in fused["groups"]) < len(gates)


def test_damaged_bytes_are_refused():
    n = 16
    gates = W.to_gates(W.grid_random(4, 4, 4, 10))
    data = hq.plan_schedule(n, gates)
    body = data[:-8]

    def code(blob):
        with pytest.raises(hq.HQError) as e:
            hq.inspect_schedule(blob)
        return e.value.code

    flipped = bytearray(data)
    flipped[len(data) // 2] ^= 0x40
    assert code(bytes(flipped)) == HQ_ERR_INVALID          # checksum
    assert code(data[:-9]) == HQ_ERR_INVALID               # truncated
    assert code(b"XXXX" + data[4:]) == HQ_ERR_INVALID      # magic
    assert code(b"") == HQ_ERR_INVALID
    assert code(reseal(body[:4] + struct.pack("<I", 9) + body[8:])) == HQ_ERR_UNSUPPORTED  # version
    assert code(reseal(body + b"\0")) == HQ_ERR_INVALID    # trailing bytes
    # the first group's first gate index pointed past the gate list
    # (header 8 + n 4 + options 28, then the gate list, folded list, maps)
    off = 40
    ngates = struct.unpack_from("<I", body, off)[0]
    off += 4 + ngates * 80
    nfold = struct.unpack_from("<I", body, off)[0]
    off += 4 + nfold * 80
    off += 4 + 4 * struct.unpack_from("<I", body, off)[0]   # index map
    off += 4 + 4 * struct.unpack_from("<I", body, off)[0]   # SWAP permutation
    assert struct.unpack_from("<I", body, off)[0] > 0        # groups
    off += 4 + 4 + 4 + 8                                     # backend, width, related
    assert struct.unpack_from("<I", body, off)[0] > 0        # gate count of group 0
    bad = bytearray(body)
    struct.pack_into("<i", bad, off + 4, nfold + 5)
    assert code(reseal(bytes(bad))) == HQ_ERR_INVALID
    # a layout that is not a permutation
    bad = bytearray(body)
    gcount = struct.unpack_from("<I", body, off)[0]
    pos_off = off + 4 + 4 * gcount
    assert struct.unpack_from("<I", body, pos_off)[0] == n
    struct.pack_into("<ii", bad, pos_off + 4, 3, 3)
    assert code(reseal(bytes(bad))) == HQ_ERR_INVALID
    # a gate on a qubit outside the register
    bad = bytearray(body)
    struct.pack_into("<i", bad, 44 + 4, n + 2)               # gate 0 target
    assert code(reseal(bytes(bad))) == HQ_ERR_INVALID


def test_size_query_and_small_buffer():
    n = 12
    gates = W.to_gates(W.ry_rz_cz(W.SplitMix64(9), n, 6))
    arr = hq.gate_array(gates)
    o = hq._compile_options()
    size = C.c_uint64()
    hq.check(hq.lib.hq_plan_serialize(n, arr, len(gates), C.byref(o), None, 0, C.byref(size)))
    assert size.value > 0
    small = C.create_string_buffer(size.value - 1)
    rc = hq.lib.hq_plan_serialize(n, arr, len(gates), C.byref(o), small, size.value - 1,
                                  C.byref(size))
    assert rc == HQ_ERR_INVALID
    assert size.value == len(hq.plan_schedule(n, gates))


def test_mutated_bytes_never_crash():
    """Random field damage past the checksum (bytes resealed) is either a valid
    schedule or a clean HQ_ERR_* error -- the loader never reads out of bounds."""
    n = 14
    gates = W.to_gates(W.grid_random(8, 2, 7, 6))
    body = hq.plan_schedule(n, gates)[:-8]
    rng = W.SplitMix64(2024)
    ok = refused = 0
    for _ in range(400):
        b = bytearray(body)
        for _ in range(1 + rng.below(3)):
            pos = rng.below(len(b))
            b[pos] = rng.below(256)
        if rng.below(4) == 0:  # truncate or extend as well
            b = b[:rng.below(len(b))] if rng.below(2) else b + bytes(rng.below(64))
        try:
            hq.inspect_schedule(reseal(bytes(b)))
            ok += 1
        except hq.HQError as e:
            assert e.code in (HQ_ERR_INVALID, HQ_ERR_UNSUPPORTED)
            refused += 1
    assert refused > 0 and ok + refused == 400
