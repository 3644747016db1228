"""The reference's own single-GPU runs as recorded traces (oracle/ref_gpu/):
the reference's host code, linked against a recording CUDA runtime, writes the
device work it issues.  These CPU tests read the traces of the benchmark
circuits: one OShareMem kernel launch and one __constant__ gate upload per gate
group (src/executor.cpp:462-493), one plain-path kernel per gate
(src/kernelSimple.cu:335-446), the "Time Cost" region bracketed by
cudaProfilerStart/Stop (src/circuit.cpp:17-52), and a group count equal to the
reference grouping this library reproduces."""
import json
import struct
from pathlib import Path

import pytest

import oracle as O
from hyquas_gb300 import workloads as W

REF = Path(O.__file__).resolve().parent / "_ref"


def read_trace(name):
    b = (REF / f"trace_{name}.bin").read_bytes()
    assert b[:4] == b"HQRT"
    p = 8
    recs = []

    def u32():
        nonlocal p
        v = struct.unpack_from("<I", b, p)[0]
        p += 4
        return v

    def u64():
        nonlocal p
        v = struct.unpack_from("<Q", b, p)[0]
        p += 8
        return v

    def s():
        nonlocal p
        k = u32()
        v = b[p:p + k].decode()
        p += k
        return v

    while True:
        kind = u32()
        if kind == 0:
            break
        if kind == 1:
            recs.append(("info", u32()))
        elif kind == 2:
            recs.append(("malloc", u64(), u64()))
        elif kind == 3:
            recs.append(("free", u64()))
        elif kind == 4:
            recs.append(("memset", u64(), u32(), u64(), u64()))
        elif kind == 5:
            dst, _, _, k = u64(), u64(), u32(), u64()
            p += k
            recs.append(("h2d", dst, k))
        elif kind == 6:
            recs.append(("d2h", u64(), u64()))
        elif kind == 7:
            recs.append(("d2d", u64(), u64(), u64(), u64()))
        elif kind == 8:
            name, off, _, k = s(), u64(), u64(), u64()
            p += k
            recs.append(("symbol", name, off, k))
        elif kind == 9:
            name = s()
            grid = (u32(), u32(), u32())
            block = (u32(), u32(), u32())
            u64(), u64()
            nargs = u32()
            for _ in range(nargs):
                sz, _ = u32(), u32()
                p += sz
            recs.append(("launch", name, grid, block, nargs))
        elif kind == 10:
            recs.append(("sync", u64()))
        elif kind == 11:
            recs.append(("begin",))
        elif kind == 12:
            recs.append(("end",))
        elif kind == 13:
            n = u32()
            recs.append(("layout", list(struct.unpack_from(f"<{n}i", b, p))))
            p += 4 * n
        else:
            raise AssertionError(f"unknown record {kind}")
    assert p == len(b)
    return recs


def region(recs):
    i0 = [i for i, r in enumerate(recs) if r[0] == "begin"]
    i1 = [i for i, r in enumerate(recs) if r[0] == "end"]
    assert len(i0) == 1 and len(i1) == 1 and i0[0] < i1[0]
    return recs[i0[0] + 1:i1[0]]


needs_traces = pytest.mark.skipif(not (REF / "trace_grid30_group.bin").exists(),
                                  reason="traces are built where the reference checkout is present")


@needs_traces
def test_grid30_trace_is_one_kernel_per_reference_group():
    import hyquas_gb300 as hq
    n = 30
    recs = read_trace("grid30_group")
    meta = json.loads((REF / "trace_grid30_group.json").read_text())
    inside = region(recs)
    launches = [r for r in inside if r[0] == "launch"]
    uploads = [r for r in inside if r[0] == "symbol"]
    assert len(launches) == meta["groups"] == len(uploads)
    assert all(r[1] == "deviceGates" for r in uploads)
    # run<128>: 2^(n-10) CTAs of 128 threads, 8 arguments (src/kernelOpt.cu:426-433)
    assert all(r[2] == (1 << (n - 10), 1, 1) and r[3] == (128, 1, 1) and r[4] == 8 for r in launches)
    assert len({r[1] for r in launches}) == 1
    # the state: one 8 GiB allocation, zeroed, amplitude 0 set (src/kernelSimple.cu:9-37)
    assert ("malloc" in {r[0] for r in recs}) and any(r[0] == "malloc" and r[2] == 8 << n for r in recs)
    # the same group count as this library's reproduction of the reference grouping
    gates = W.to_gates(W.grid_random(2, 5, 6, 20))
    assert meta["groups"] == len(hq.plan_groups(n, gates, reference_grouping=True))
    lay = [r for r in recs if r[0] == "layout"][0][1]
    assert sorted(lay) == list(range(n))


@needs_traces
def test_plain20_trace_is_one_kernel_per_gate():
    recs = read_trace("plain20_serial")
    desc = W.plain_u3_cnot(1, 20, 10)
    launches = [r for r in region(recs) if r[0] == "launch"]
    assert len(launches) == len(desc)
    # 2^(n-1) pairs, 128 threads per CTA
    assert all(r[2][0] * r[3][0] == 1 << 19 for r in launches)
    assert region(recs)[-1][0] == "sync"  # kernelExecSimple ends with a device synchronise
