"""Gate grouping parity with the reference's Compiler (host only, no GPU).

With reference_grouping=1 the partitioner uses the reference's widths (tile 10
qubits, 3 coalesced qubits, MAT 6) and must reproduce, gate for gate, the
groups the reference's Compiler::run produced for the same circuits
(tests/golden/partition_*.json, made by tests/golden/make_golden.py)."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem.replace("partition_", "") for p in GOLDEN.glob("partition_*.json"))


def plan(n, desc, backend, reference=True, tile=0, mm=0):
    gates = W.to_gates(desc)
    arr = hq.gate_array(gates)
    o = hq.hq_compile_options()
    hq.check(hq.lib.hq_compile_options_default(C.byref(o)))
    o.backend = backend
    o.reference_grouping = 1 if reference else 0
    o.tile_qubits = tile
    o.mm_qubits = mm
    k = len(gates)
    ng = C.c_int32()
    b = (C.c_int32 * k)()
    gpg = (C.c_int32 * k)()
    w = (C.c_int32 * k)()
    rel = (C.c_uint64 * k)()
    ph = (C.c_int32 * k)()
    order = (C.c_int32 * k)()
    hq.check(hq.lib.hq_plan_groups(n, arr, k, C.byref(o), C.byref(ng), b, gpg, w, rel, ph, order))
    groups, off = [], 0
    for i in range(ng.value):
        groups.append({"backend": b[i], "gates": list(order[off:off + gpg[i]]), "related": rel[i],
                       "width": w[i], "phases": ph[i]})
        off += gpg[i]
    return groups


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("backend", ["group", "blas"])
def test_reference_grouping_matches_reference(case, backend):
    rec = json.loads((GOLDEN / f"partition_{case}.json").read_text())
    desc = [tuple(x[:4]) + (tuple(x[4]),) for x in rec["desc"]]
    ref = rec["backends"][backend]["groups"]
    ours = plan(rec["n"], desc, hq.BACKEND_OSHM if backend == "group" else hq.BACKEND_TRANSMM)
    assert len(ours) == len(ref)
    for a, b in zip(ours, ref):
        assert a["gates"] == b["gates"]
        assert a["related"] == b["related"]


def test_native_grouping_covers_every_gate_once():
    desc = W.grid_random(2, 5, 6, 20)
    for backend in (hq.BACKEND_OSHM, hq.BACKEND_TRANSMM, hq.BACKEND_HYBRID):
        groups = plan(30, desc, backend, reference=False)
        seen = sorted(x for g in groups for x in g["gates"])
        assert seen == list(range(len(desc)))


def test_native_tile_is_wider_and_needs_fewer_passes():
    desc = W.grid_random(2, 5, 6, 20)
    rec = json.loads((GOLDEN / "partition_grid_5x6_c20.json").read_text())
    ref_groups = len(rec["backends"]["group"]["groups"])
    ours = plan(30, desc, hq.BACKEND_OSHM, reference=False)
    assert len(ours) < ref_groups
    for g in ours:
        assert g["width"] == 13
        assert g["phases"] >= 1


def test_group_order_respects_dependencies():
    """Executing groups in order, gates in group order, equals program order
    for every pair of gates that share a qubit and do not commute."""
    desc = W.plain_u3_cnot(1, 20, 10)
    groups = plan(20, desc, hq.BACKEND_OSHM, reference=False)
    pos = {}
    k = 0
    for g in groups:
        for x in g["gates"]:
            pos[x] = k
            k += 1
    qubits = lambda d: {d[1]} | ({d[2]} if d[2] >= 0 else set())
    for i in range(len(desc)):
        for j in range(i + 1, len(desc)):
            if qubits(desc[i]) & qubits(desc[j]):
                assert pos[i] < pos[j], (i, j)


DIAGONAL = {W.CZ, W.CU1, W.CRZ, W.U1, W.Z, W.S, W.SDG, W.T, W.TDG, W.RZ}


def families():
    out = []
    for s in range(3):
        out.append((f"grid30_{s}", 30, W.grid_random(2 + s, 5, 6, 20)))
        out.append((f"grid28_{s}", 28, W.grid_random(10 + s, 4, 7, 24)))
        out.append((f"ryrz26_{s}", 26, W.ry_rz_cz(W.SplitMix64(20 + s), 26, 30)))
        out.append((f"u3cnot24_{s}", 24, W.plain_u3_cnot(30 + s, 24, 12)))
    out.append(("qft24", 24, [g for g in W.qft(24) if g[0] != W.SWAP]))
    return out


@pytest.mark.parametrize("backend", [hq.BACKEND_OSHM, hq.BACKEND_HYBRID, hq.BACKEND_TRANSMM])
def test_schedules_are_valid_in_either_direction(backend):
    """The partitioner may keep the greedy over the reversed circuit; whichever
    it keeps, every gate runs once, every pair of gates that share a qubit and do
    not commute keeps its program order, and each OShareMem group's
    non-diagonal targets lie in its related qubits."""
    qubits = lambda d: {d[1]} | {q for q in (d[2], d[3]) if q >= 0}
    for name, n, desc in families():
        groups = plan(n, desc, backend, reference=False)
        pos, k = {}, 0
        for g in groups:
            for x in g["gates"]:
                assert x not in pos, (name, x)
                pos[x] = k
                k += 1
            if g["backend"] == hq.BACKEND_OSHM:
                for x in g["gates"]:
                    if desc[x][0] not in DIAGONAL:
                        assert (g["related"] >> desc[x][1]) & 1, (name, x)
        assert sorted(pos) == list(range(len(desc))), name
        by_qubit = {}
        for i, d in enumerate(desc):
            for q in qubits(d):
                by_qubit.setdefault(q, []).append(i)
        for q, idx in by_qubit.items():
            last_any = last_nondiag = -1  # latest schedule positions so far on q
            for b in idx:
                diag = desc[b][0] in DIAGONAL
                assert pos[b] > (last_nondiag if diag else last_any), (name, q, b)
                last_any = max(last_any, pos[b])
                if not diag:
                    last_nondiag = max(last_nondiag, pos[b])


def test_package_plan_groups_matches_the_abi():
    desc = W.grid_random(2, 5, 6, 20)
    gates = W.to_gates(desc)
    for ref in (True, False):
        a = hq.plan_groups(30, gates, reference_grouping=ref)
        b = plan(30, desc, hq.BACKEND_OSHM, reference=ref)
        assert [(g["backend"], g["gates"], g["related"]) for g in a] == \
               [(g["backend"], g["gates"], g["related"]) for g in b]
    assert len(hq.plan_groups(30, gates, reference_grouping=True)) == 17
