"""CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/liboracle.so (built from oracle/oracle.c by `make -C oracle`).
Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline leg and
the --impl reference arm) import this package, as the checker or the CPU
baseline.  The product library never links or calls it.

Gate descriptions are the tuples of hyquas_gb300.workloads:
(type, target, control, control2, params); matrices are computed here by the
oracle's own restatement of the reference factories (src/gate.cpp:9-342), not
by the product library.  SWAP (an extension) is applied as three CNOTs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SWAP = 28
CNOT = 1


class oracle_gate(C.Structure):
    _fields_ = [("type", C.c_int32), ("target", C.c_int32), ("control", C.c_int32),
                ("control2", C.c_int32), ("mat", C.c_double * 8)]


def build():
    src = HERE / "oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-C", str(HERE), "liboracle.so"], check=True, capture_output=True)


def _load():
    build()
    lib = C.CDLL(str(LIB))
    P = C.c_void_p
    lib.oracle_gate_matrix.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_apply_f64.argtypes = [C.c_int, P, P, C.c_int, C.c_int]
    lib.oracle_apply_f32.argtypes = [C.c_int, P, P, C.c_int, C.c_int]
    lib.oracle_prob_zero_f32.argtypes = [C.c_int, P, C.c_int, C.c_int]
    lib.oracle_prob_zero_f32.restype = C.c_double
    lib.oracle_group_unitary.argtypes = [C.c_int, P, P, C.c_int, P]
    lib.oracle_apply_f64_blocked.argtypes = [C.c_int, P, P, C.c_int, C.c_int, C.c_int]
    lib.oracle_apply_f64_blocked.restype = C.c_int
    lib.oracle_compare_c64.argtypes = [C.c_int64, P, P, C.c_int, P]
    lib.oracle_compare_c64.restype = None
    for f in ("oracle_gate_matrix", "oracle_apply_f64", "oracle_apply_f32", "oracle_group_unitary"):
        getattr(lib, f).restype = C.c_int
    return lib


lib = _load()
NTHREADS = int(os.environ.get("HQ_ORACLE_THREADS", str(os.cpu_count() or 1)))


def gate_matrix(t: int, params=()) -> np.ndarray:
    p = (C.c_double * 3)(*(list(params) + [0.0] * (3 - len(params))))
    m = (C.c_double * 8)()
    if lib.oracle_gate_matrix(t, p, m) != 0:
        raise ValueError(f"oracle: unknown gate type {t}")
    return np.array(list(m))


def expand(desc):
    """Replace SWAP extension gates by three CNOTs."""
    out = []
    for (t, q, c, c2, p) in desc:
        if t == SWAP:
            out += [(CNOT, c, q, -1, ()), (CNOT, q, c, -1, ()), (CNOT, c, q, -1, ())]
        else:
            out.append((t, q, c, c2, p))
    return out


def gate_structs(desc):
    desc = expand(desc)
    arr = (oracle_gate * max(1, len(desc)))()
    for i, (t, q, c, c2, p) in enumerate(desc):
        arr[i].type, arr[i].target, arr[i].control, arr[i].control2 = t, q, c, c2
        m = gate_matrix(t, p)
        for k in range(8):
            arr[i].mat[k] = m[k]
    return arr, len(desc)


BLOCK_QUBITS = 14  # 2^14 complex128 = 256 KiB per thread: a block stays in cache


def apply_f64(n: int, state: np.ndarray, desc, threads: int | None = None,
              blocked: bool | None = None, copy: bool = True) -> np.ndarray:
    """Gates in order, FP64.  From 18 qubits up the blocked form runs (the
    same operations on every amplitude, bit-identical results, cache-sized
    blocks); `blocked` forces either form."""
    a = np.ascontiguousarray(state, dtype=np.complex128)
    if copy:
        a = a.copy()
    arr, k = gate_structs(desc)
    if blocked is None:
        blocked = n >= 18
    if blocked:
        rc = lib.oracle_apply_f64_blocked(n, a.ctypes.data, arr, k, threads or NTHREADS,
                                          BLOCK_QUBITS)
    else:
        rc = lib.oracle_apply_f64(n, a.ctypes.data, arr, k, threads or NTHREADS)
    if rc != 0:
        raise ValueError("oracle_apply_f64 rejected the circuit")
    return a


def apply_f32(n: int, state: np.ndarray, desc, threads: int | None = None,
              structs=None) -> np.ndarray:
    a = np.ascontiguousarray(state, dtype=np.complex64)
    arr, k = structs if structs is not None else gate_structs(desc)
    rc = lib.oracle_apply_f32(n, a.ctypes.data, arr, k, threads or NTHREADS)
    if rc != 0:
        raise ValueError("oracle_apply_f32 rejected the circuit")
    return a


def zero_state(n: int, dtype=np.complex128) -> np.ndarray:
    a = np.zeros(1 << n, dtype=dtype)
    a[0] = 1
    return a


def run_f64(n: int, desc, init: np.ndarray | None = None) -> np.ndarray:
    if init is None:
        return apply_f64(n, zero_state(n), desc, copy=False)
    return apply_f64(n, init, desc)


def group_unitary(qubits, desc) -> np.ndarray:
    """U (2^m x 2^m) with U[r, c] = <r|U|c>; local bit j <-> qubits[j]."""
    m = len(qubits)
    q = (C.c_int * m)(*qubits)
    arr, k = gate_structs(desc)
    out = np.empty((1 << m) * (1 << m), dtype=np.complex128)
    if lib.oracle_group_unitary(m, q, arr, k, out.ctypes.data) != 0:
        raise ValueError("oracle_group_unitary failed")
    return out.reshape(1 << m, 1 << m).T


def compare(ref: np.ndarray, got: np.ndarray) -> dict:
    """max |d amp| and 1 - fidelity (|<ref|got>|^2 / (|ref|^2 |got|^2))."""
    if (ref.dtype == np.complex128 and got.dtype == np.complex64 and ref.size == got.size
            and ref.flags.c_contiguous and got.flags.c_contiguous):
        out = (C.c_double * 5)()
        lib.oracle_compare_c64(ref.size, ref.ctypes.data, got.ctypes.data, NTHREADS, out)
        mx, ore, oim, rr, gg = list(out)
        fid = (ore * ore + oim * oim) / (rr * gg) if rr > 0 and gg > 0 else 0.0
        return {"max_abs_err": mx, "one_minus_fidelity": float(1.0 - fid)}
    r = ref.astype(np.complex128)
    g = got.astype(np.complex128)
    err = float(np.max(np.abs(r - g))) if r.size else 0.0
    ov = np.vdot(r, g)
    fid = abs(ov) ** 2 / (np.vdot(r, r).real * np.vdot(g, g).real)
    return {"max_abs_err": err, "one_minus_fidelity": float(1.0 - fid)}


def _mix64_uniforms(seed: int, shots: int) -> np.ndarray:
    """The SplitMix64 stream of `seed` (Steele, Lea, Flood 2014), 53-bit
    uniforms in [0, 1): the draws the product sampler makes."""
    mask = (1 << 64) - 1
    s = seed & mask
    out = np.empty(shots, dtype=np.float64)
    for i in range(shots):
        s = (s + 0x9E3779B97F4A7C15) & mask
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        out[i] = (z >> 11) * (1.0 / (1 << 53))
    return out


SAMPLE_BLOCK = 1 << 12  # amplitudes per block of the sampler's cumulative distribution


def _block_sums(p: np.ndarray) -> np.ndarray:
    """FP64 sum of each block of 4096 probabilities in the sampler's order:
    256 partial sums (partial t adds elements t, t + 256, ... in turn), then a
    pairwise tree (t += t + w for w = 128, 64, ..., 1)."""
    nb = (p.size + SAMPLE_BLOCK - 1) // SAMPLE_BLOCK
    q = np.zeros(nb * SAMPLE_BLOCK, dtype=np.float64)
    q[:p.size] = p
    q = q.reshape(nb, SAMPLE_BLOCK // 256, 256)
    s = np.zeros((nb, 256), dtype=np.float64)
    for j in range(SAMPLE_BLOCK // 256):
        s = s + q[:, j, :]
    w = 128
    while w > 0:
        s[:, :w] = s[:, :w] + s[:, w:2 * w]
        w >>= 1
    return s[:, 0].copy()


def _block_scan(v: np.ndarray) -> np.ndarray:
    """Inclusive scan in the sampler's order: 1024 chunks of ceil(nb/1024)
    are scanned sequentially, chunk offsets are an exclusive sequential scan
    of the chunk totals, and each element adds its chunk's offset."""
    nb = v.size
    per = (nb + 1023) // 1024
    out = np.empty_like(v)
    totals = np.zeros(1024, dtype=np.float64)
    for t in range(1024):
        lo, hi = t * per, min(t * per + per, nb)
        if lo >= hi:
            continue
        run = 0.0
        for i in range(lo, hi):
            run = run + float(v[i])
            out[i] = run
        totals[t] = run
    off = 0.0
    offs = np.zeros(1024, dtype=np.float64)
    for t in range(1024):
        offs[t] = off
        off = off + float(totals[t])
    for t in range(1024):
        lo, hi = t * per, min(t * per + per, nb)
        if lo < hi:
            out[lo:hi] = out[lo:hi] + offs[t]
    return out


def sample(amps: np.ndarray, shots: int, seed: int) -> np.ndarray:
    """Inverse-CDF sampling of basis indices from |amp|^2 in FP64, with the
    same draws (SplitMix64 stream of `seed`) and the same order of FP64
    additions as hq_state_sample, so the indices must agree exactly: block
    sums of 4096 amplitudes, a chunked scan into a block CDF, a binary search
    for the first block whose cumulative sum exceeds u * total, then a scan
    of that block in runs of 32 for the first non-zero amplitude whose running
    sum exceeds the remainder (the block's last non-zero amplitude when
    rounding leaves the remainder past the block's sum)."""
    a = np.ascontiguousarray(amps, dtype=np.complex64)
    # |a|^2 of complex64 amplitudes: both products are exact in FP64
    p = a.real.astype(np.float64) * a.real.astype(np.float64) + \
        a.imag.astype(np.float64) * a.imag.astype(np.float64)
    cdf = _block_scan(_block_sums(p))
    nb = cdf.size
    total = float(cdf[-1])
    u = _mix64_uniforms(seed, shots)
    out = np.empty(shots, dtype=np.uint64)
    for s_i in range(shots):
        target = float(u[s_i]) * total
        blk = int(np.searchsorted(cdf, target, side="right"))
        blk = min(blk, nb - 1)
        rem = target - (float(cdf[blk - 1]) if blk else 0.0)
        base = blk * SAMPLE_BLOCK
        end = min(base + SAMPLE_BLOCK, p.size)
        nch = (end - base + 31) // 32
        x = np.zeros(nch * 32, dtype=np.float64)
        x[:end - base] = p[base:end]
        x = x.reshape(nch, 32)
        run = x.copy()  # per-run doubling scan, all runs at once
        d = 1
        while d < 32:
            prev = run.copy()
            run[:, d:] = prev[:, d:] + prev[:, :-d]
            d <<= 1
        pick, last_nz = None, base
        for ch in range(nch):
            pos = x[ch] > 0.0
            nz = np.nonzero(pos)[0]
            if nz.size:
                last_nz = base + ch * 32 + int(nz[-1])
            hit = np.nonzero(pos & (run[ch] > rem))[0]
            if hit.size:
                pick = base + ch * 32 + int(hit[0])
                break
            rem = rem - float(run[ch, 31])
        out[s_i] = pick if pick is not None else last_nz
    return out


# ---------------------------------------------------------------------------
# The reference's own single-GPU runs, replayed on a GPU (oracle/ref_replay.cu).
# oracle/_ref/trace_<name>.bin is the device work the reference's host code
# issued for one circuit (recorded by `make -C oracle ref-gpu` and
# oracle/make_ref_traces.py where the reference checkout is present); the
# cubins are the reference's kernels compiled from its sources.

REF_DIR = HERE / "_ref"
REPLAY_LIB = HERE / "libref_replay.so"
REF_CUBINS = ("kernelOpt.cubin", "kernelSimple.cubin")


def ref_gpu_available(name: str) -> bool:
    return (REPLAY_LIB.exists() and (REF_DIR / f"trace_{name}.bin").exists()
            and all((REF_DIR / c).exists() for c in REF_CUBINS))


def ref_gpu_meta(name: str) -> dict:
    import json
    return json.loads((REF_DIR / f"trace_{name}.json").read_text())


def to_logical(state: np.ndarray, pos) -> np.ndarray:
    """Amplitudes in logical index order from a state whose logical qubit q
    sits at physical bit pos[q] (the reference's Circuit::toPhysicalID,
    src/circuit.cpp:95-104)."""
    n = len(pos)
    if list(pos) == list(range(n)):
        return state
    # numpy axis k of the (2,)*n view is bit n-1-k
    t = state.reshape([2] * n).transpose([n - 1 - pos[n - 1 - k] for k in range(n)])
    return np.ascontiguousarray(t).reshape(-1)


def ref_gpu_run(name: str, repeats: int = 3, want_state: bool = True) -> dict:
    """Replay trace `name` on the current GPU: `repeats` timed runs after one
    untimed run.  Returns the reference's "Time Cost" (host clock, best and
    mean, ms), the CUDA-event time of the same region, its kernel launches, and
    (want_state) the final state in logical order."""
    lib = C.CDLL(str(REPLAY_LIB))
    lib.ref_replay_run.argtypes = [C.c_char_p, C.POINTER(C.c_char_p), C.c_int, C.c_int, C.c_void_p,
                                   C.c_uint64, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    lib.ref_replay_run.restype = C.c_int
    meta = ref_gpu_meta(name)
    n = meta["num_qubits"]
    state = np.empty(1 << n, dtype=np.complex64) if want_state else None
    layout = (C.c_int32 * n)()
    out = (C.c_double * 5)()
    err = C.create_string_buffer(1024)
    cubins = (C.c_char_p * len(REF_CUBINS))(*[str(REF_DIR / c).encode() for c in REF_CUBINS])
    rc = lib.ref_replay_run(str(REF_DIR / f"trace_{name}.bin").encode(), cubins, len(REF_CUBINS),
                            repeats, state.ctypes.data if want_state else None,
                            state.nbytes if want_state else 0, layout, out, err, len(err))
    if rc != 0:
        raise RuntimeError(f"reference replay {name}: {err.value.decode()}")
    res = {"time_cost_ms_best": out[0], "time_cost_ms_mean": out[1], "device_ms_best": out[2],
           "launches": int(out[3]), "num_qubits": int(out[4]), "groups": meta.get("groups"),
           "gates": meta.get("gates"), "backend": meta.get("backend"), "layout": list(layout)}
    if want_state:
        res["state"] = to_logical(state, list(layout))
    return res
