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


def apply_f64(n: int, state: np.ndarray, desc, threads: int | None = None) -> np.ndarray:
    a = np.ascontiguousarray(state, dtype=np.complex128).copy()
    arr, k = gate_structs(desc)
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
    return apply_f64(n, zero_state(n) if init is None else init, desc)


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


def sample(amps: np.ndarray, shots: int, seed: int) -> np.ndarray:
    """Inverse-CDF sampling of basis indices from |amp|^2 in FP64 with the
    same draws as hq_state_sample (first index whose cumulative probability
    exceeds u * total)."""
    a = np.asarray(amps)
    p = a.real.astype(np.float64) ** 2 + a.imag.astype(np.float64) ** 2
    cdf = np.cumsum(p)
    u = _mix64_uniforms(seed, shots)
    idx = np.searchsorted(cdf, u * cdf[-1], side="right")
    return np.minimum(idx, a.size - 1).astype(np.uint64)
