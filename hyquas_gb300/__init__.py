"""hyquas_gb300: GB300-native single-GPU state-vector simulator.

Python mirror of the reference's user API (thu-pacman/HyQuas src/circuit.h:20-46,
src/gate.h:11-66) over the C ABI in include/hyquas_gb300.h:

    c = Circuit(n)
    c.addGate(Gate.H(0)); c.addGate(Gate.CNOT(0, 1))
    c.compile()
    us = c.run()            # device time in microseconds ("Time Cost")
    c.ampAt(3)              # ResultItem(idx, amp)

The native library (libhyquas_gb300.so, built by hyquas_gb300/build.py) is the
only implementation: importing this module without it raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libhyquas_gb300.so"

# reference GateType ordinals (src/gate.h:7-9) + SWAP extension
CCX, CNOT, CY, CZ, CRX, CRY, CU1, CRZ, U1, U2, U3, H, X, Y, Z, S, SDG, T, TDG, RX, RY, RZ = range(22)
ID = 23
SWAP = 28

BACKEND_PLAIN, BACKEND_OSHM, BACKEND_TRANSMM, BACKEND_HYBRID = 0, 1, 3, 4
MM_BF16X3, MM_TF32, MM_FP32 = 0, 1, 2
_BACKENDS = {"plain": 0, "serial": 0, "oshm": 1, "group": 1, "transmm": 3, "blas": 3,
             "hybrid": 4, "mix": 4}
_PRECISIONS = {"bf16x3": 0, "tf32": 1, "fp32": 2}

ERR = {0: "ok", -1: "invalid", -2: "cuda", -3: "nomem", -4: "state", -5: "timeout",
       -6: "unsupported", -7: "busy"}


class HQError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERR.get(code, code)}] {msg}")
        self.code = code


class hq_gate(C.Structure):
    _fields_ = [("type", C.c_int32), ("target", C.c_int32), ("control", C.c_int32),
                ("control2", C.c_int32), ("mat", C.c_double * 8)]


class hq_compile_options(C.Structure):
    _fields_ = [("backend", C.c_int32), ("tile_qubits", C.c_int32), ("coalesce", C.c_int32),
                ("mm_qubits", C.c_int32), ("mm_precision", C.c_int32),
                ("reference_grouping", C.c_int32), ("specialize", C.c_int32)]


class hq_cost_params(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("pass_floor", "oshm_gate", "oshm_diag", "oshm_ctrl_diag",
                                         "mm_bf16x3", "mm_tf32", "mm_fp32", "launch")]


class hq_server_options(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("step_budget_us", C.c_double),
                ("planner_threads", C.c_int32), ("tile_qubits", C.c_int32),
                ("jit_min_qubits", C.c_int32)]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"native library missing: {LIB_PATH} (run hyquas_gb300/build.py)")
    lib = C.CDLL(str(LIB_PATH))
    P, I32, I64, U64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
    sig = {
        "hq_init": [C.c_int],
        "hq_device_info": [C.POINTER(I32), C.POINTER(U64), C.POINTER(I32)],
        "hq_set_hbm_budget": [U64],
        "hq_hbm_in_use": [C.POINTER(U64)],
        "hq_gate_make": [I32, I32, I32, I32, C.POINTER(D), C.POINTER(hq_gate)],
        "hq_state_create": [I32, C.POINTER(P)],
        "hq_state_destroy": [P],
        "hq_state_init_zero": [P],
        "hq_state_load": [P, P],
        "hq_state_store": [P, P],
        "hq_state_store_async": [P, P],
        "hq_state_wait": [P],
        "hq_state_amps": [P, P, I64, P],
        "hq_state_layout": [P, P],
        "hq_state_num_qubits": [P, C.POINTER(I32)],
        "hq_state_device_ptr": [P, C.POINTER(P)],
        "hq_state_prob_zero": [P, I32, C.POINTER(D)],
        "hq_state_norm": [P, C.POINTER(D)],
        "hq_state_marginals": [P, P],
        "hq_state_sample": [P, I32, U64, P],
        "hq_state_remap": [P, P],
        "hq_apply_gates": [P, P, I32],
        "hq_compile_options_default": [C.POINTER(hq_compile_options)],
        "hq_circuit_create": [I32, C.POINTER(P)],
        "hq_circuit_destroy": [P],
        "hq_circuit_add_gates": [P, P, I32],
        "hq_circuit_num_gates": [P, C.POINTER(I32)],
        "hq_circuit_compile": [P, C.POINTER(hq_compile_options)],
        "hq_circuit_schedule": [P, C.POINTER(I32), P, P, P, P],
        "hq_circuit_group_gates": [P, I32, P, I32, C.POINTER(I32)],
        "hq_circuit_run": [P, P, C.POINTER(D)],
        "hq_circuit_run_to_host": [P, P, P, C.POINTER(D)],
        "hq_circuit_enqueue": [P, P],
        "hq_circuit_profile": [P, P, P],
        "hq_circuit_predict": [P, P],
        "hq_circuit_program_bytes": [P, C.POINTER(U64)],
        "hq_host_alloc": [U64, C.POINTER(P)],
        "hq_host_free": [P],
        "hq_plan_groups": [I32, P, I32, C.POINTER(hq_compile_options), C.POINTER(I32), P, P, P, P,
                           P, P],
        "hq_circuit_capture_graph": [P, P],
        "hq_circuit_serialize": [P, P, U64, C.POINTER(U64)],
        "hq_plan_serialize": [I32, P, I32, C.POINTER(hq_compile_options), P, U64, C.POINTER(U64)],
        "hq_schedule_inspect": [P, U64, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32), P, P, P, P],
        "hq_circuit_deserialize": [P, U64, C.POINTER(P)],
        "hq_synchronize": [],
        "hq_apply_oshm_group": [P, P, I32, U64],
        "hq_apply_transmm_group": [P, P, I32, U64, I32],
        "hq_apply_unitary": [P, P, U64, I32],
        "hq_group_unitary": [P, I32, U64, P],
        "hq_qasm_parse": [C.c_char_p, C.POINTER(I32), P, I32, C.POINTER(I32)],
        "hq_cost_params_get": [C.POINTER(hq_cost_params)],
        "hq_cost_params_set": [C.POINTER(hq_cost_params)],
        "hq_autotune": [I32, C.POINTER(hq_cost_params)],
        "hq_server_options_default": [C.POINTER(hq_server_options)],
        "hq_server_check": [C.POINTER(hq_server_options), I32, P, I32],
        "hq_server_create": [C.POINTER(hq_server_options), C.POINTER(P)],
        "hq_server_destroy": [P],
        "hq_server_submit": [P, I32, P, I32, C.POINTER(I64)],
        "hq_server_wait": [P, I64, D, C.POINTER(I32)],
        "hq_server_poll": [P, P, I32, C.POINTER(I32)],
        "hq_server_state": [P, I64, C.POINTER(P)],
        "hq_server_times": [P, I64, C.POINTER(D), C.POINTER(D), C.POINTER(D)],
        "hq_server_release": [P, I64],
        "hq_server_steps": [P, I64, C.POINTER(I64), C.POINTER(I64)],
        "hq_server_plan_cache": [P, C.POINTER(I64), C.POINTER(I64)],
        "hq_server_stats": [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64), C.POINTER(U64),
                            C.POINTER(U64)],
        "hq_batch_create": [C.POINTER(P)],
        "hq_batch_destroy": [P],
        "hq_batch_add": [P, P, P, C.POINTER(I32)],
        "hq_batch_compile": [P, C.POINTER(hq_compile_options)],
        "hq_batch_run": [P, I32, C.POINTER(D)],
        "hq_batch_enqueue": [P, I32],
        "hq_batch_capture_graph": [P, I32],
        "hq_batch_inject_stall": [P],
        "hq_batch_info": [P, C.POINTER(I32), C.POINTER(I64), C.POINTER(I64), C.POINTER(U64), P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = I32
    lib.hq_last_error.restype = C.c_char_p
    lib.hq_last_error.argtypes = []
    lib.hq_version.restype = C.c_char_p
    lib.hq_version.argtypes = []
    return lib


lib = _load()


def check(code: int):
    if code != 0:
        raise HQError(code, lib.hq_last_error().decode())


def synchronize():
    check(lib.hq_synchronize())


def init(device: int = 0):
    check(lib.hq_init(device))


def device_info():
    sm, hbm, smem = C.c_int32(), C.c_uint64(), C.c_int32()
    check(lib.hq_device_info(C.byref(sm), C.byref(hbm), C.byref(smem)))
    return {"sm_count": sm.value, "hbm_bytes": hbm.value, "smem_per_block": smem.value}


class _PinnedView:
    """The numpy view's base: it holds the PinnedBuffer, so the memory stays
    allocated while any view of it is alive (unless free() is called)."""

    def __init__(self, owner, ptr: int, count: int, dtype):
        self.owner = owner
        self.__array_interface__ = {"shape": (int(count),), "typestr": np.dtype(dtype).str,
                                    "data": (ptr, False), "version": 3}


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array (`array`).  The buffer
    lives as long as the buffer object or any view of `array`."""

    def __init__(self, count: int, dtype=np.complex64):
        self.ptr = C.c_void_p()
        nbytes = int(count) * np.dtype(dtype).itemsize
        check(lib.hq_host_alloc(nbytes, C.byref(self.ptr)))
        self.array = np.asarray(_PinnedView(self, self.ptr.value, count, dtype))

    def numa_nodes(self, samples: int = 16) -> list[int] | None:
        """NUMA node of `samples` pages spread over the buffer (move_pages with
        no target nodes only reports where each page is); None where the
        query is unavailable."""
        import platform
        nr = {"x86_64": 279, "aarch64": 239}.get(platform.machine())
        if nr is None or not self.ptr:
            return None
        libc = C.CDLL(None, use_errno=True)
        page = os.sysconf("SC_PAGE_SIZE")
        nbytes = self.array.nbytes
        addrs = [(self.ptr.value + (nbytes - 1) * i // max(1, samples - 1)) // page * page
                 for i in range(samples)]
        pages = (C.c_void_p * samples)(*addrs)
        status = (C.c_int * samples)()
        rc = libc.syscall(C.c_long(nr), C.c_int(0), C.c_ulong(samples), pages, None, status,
                          C.c_int(0))
        if rc != 0:
            return None
        return sorted(set(int(x) for x in status))

    def free(self):
        if self.ptr:
            lib.hq_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def set_hbm_budget(nbytes: int):
    check(lib.hq_set_hbm_budget(int(nbytes)))


def hbm_in_use() -> int:
    v = C.c_uint64()
    check(lib.hq_hbm_in_use(C.byref(v)))
    return v.value


# --------------------------------------------------------------------------- gates

class Gate:
    """A gate; factories follow the reference's argument order (control first)."""

    __slots__ = ("g",)

    def __init__(self, g: hq_gate):
        self.g = g

    @staticmethod
    def _make(t, target, control=-1, control2=-1, params=()):
        g = hq_gate()
        arr = (C.c_double * 3)(*(list(params) + [0.0] * (3 - len(params))))
        check(lib.hq_gate_make(t, target, control, control2, arr, C.byref(g)))
        return Gate(g)

    # two-qubit and three-qubit gates: control(s) first, as in src/gate.h:30-38
    @staticmethod
    def CCX(c1, c2, t): return Gate._make(CCX, t, c1, c2)
    @staticmethod
    def CNOT(c, t): return Gate._make(CNOT, t, c)
    @staticmethod
    def CY(c, t): return Gate._make(CY, t, c)
    @staticmethod
    def CZ(c, t): return Gate._make(CZ, t, c)
    @staticmethod
    def CRX(c, t, angle): return Gate._make(CRX, t, c, params=(angle,))
    @staticmethod
    def CRY(c, t, angle): return Gate._make(CRY, t, c, params=(angle,))
    @staticmethod
    def CU1(c, t, lam): return Gate._make(CU1, t, c, params=(lam,))
    @staticmethod
    def CRZ(c, t, angle): return Gate._make(CRZ, t, c, params=(angle,))
    @staticmethod
    def U1(t, lam): return Gate._make(U1, t, params=(lam,))
    @staticmethod
    def U2(t, phi, lam): return Gate._make(U2, t, params=(phi, lam))
    @staticmethod
    def U3(t, theta, phi, lam): return Gate._make(U3, t, params=(theta, phi, lam))
    @staticmethod
    def H(t): return Gate._make(H, t)
    @staticmethod
    def X(t): return Gate._make(X, t)
    @staticmethod
    def Y(t): return Gate._make(Y, t)
    @staticmethod
    def Z(t): return Gate._make(Z, t)
    @staticmethod
    def S(t): return Gate._make(S, t)
    @staticmethod
    def SDG(t): return Gate._make(SDG, t)
    @staticmethod
    def T(t): return Gate._make(T, t)
    @staticmethod
    def TDG(t): return Gate._make(TDG, t)
    @staticmethod
    def RX(t, angle): return Gate._make(RX, t, params=(angle,))
    @staticmethod
    def RY(t, angle): return Gate._make(RY, t, params=(angle,))
    @staticmethod
    def RZ(t, angle): return Gate._make(RZ, t, params=(angle,))
    @staticmethod
    def ID(t): return Gate._make(ID, t)
    # extensions (no reference factory)
    @staticmethod
    def SWAP(a, b): return Gate._make(SWAP, a, b)
    @staticmethod
    def SX(t): return Gate.RX(t, math.pi / 2)
    @staticmethod
    def SY(t): return Gate.RY(t, math.pi / 2)

    @property
    def type(self): return self.g.type
    @property
    def targetQubit(self): return self.g.target
    @property
    def controlQubit(self): return self.g.control
    @property
    def controlQubit2(self): return self.g.control2
    @property
    def mat(self):
        m = list(self.g.mat)
        return np.array([[m[0] + 1j * m[1], m[2] + 1j * m[3]], [m[4] + 1j * m[5], m[6] + 1j * m[7]]])

    def isDiagonal(self) -> bool:
        return self.g.type in (CZ, CU1, CRZ, U1, Z, S, SDG, T, TDG, RZ)

    def __repr__(self):
        return f"Gate(type={self.g.type}, t={self.g.target}, c={self.g.control}, c2={self.g.control2})"


def gate_array(gates) -> C.Array:
    arr = (hq_gate * max(1, len(gates)))()
    for i, g in enumerate(gates):
        arr[i] = g.g if isinstance(g, Gate) else g
    return arr


def _compile_options(backend="oshm", tile_qubits=0, coalesce=0, mm_qubits=0, precision="bf16x3",
                     reference_grouping=False, specialize=2) -> hq_compile_options:
    o = hq_compile_options()
    check(lib.hq_compile_options_default(C.byref(o)))
    o.backend = _BACKENDS[backend] if isinstance(backend, str) else backend
    o.tile_qubits = tile_qubits
    o.coalesce = coalesce
    o.mm_qubits = mm_qubits
    o.mm_precision = _PRECISIONS[precision] if isinstance(precision, str) else precision
    o.reference_grouping = 1 if reference_grouping else 0
    o.specialize = specialize
    return o


def plan_groups(num_qubits: int, gates, **options) -> list[dict]:
    """Host only: the gate groups compile would make (hq_plan_groups), each as
    {backend, gates (indices), width, related, phases}."""
    arr = gate_array(gates)
    o = _compile_options(**options)
    k = max(1, len(gates))
    ng = C.c_int32()
    b, g, w = (C.c_int32 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
    rel, ph, order = (C.c_uint64 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
    check(lib.hq_plan_groups(num_qubits, arr, len(gates), C.byref(o), C.byref(ng), b, g, w, rel, ph,
                             order))
    out, off = [], 0
    for i in range(ng.value):
        out.append({"backend": b[i], "gates": list(order[off:off + g[i]]), "width": w[i],
                    "related": rel[i], "phases": ph[i]})
        off += g[i]
    return out


def plan_schedule(num_qubits: int, gates, **options) -> bytes:
    """Host only: the schedule bytes compile would make for these gates (the
    reference's Schedule::serialize, src/schedule.cpp:156-325)."""
    arr = gate_array(gates)
    o = _compile_options(**options)
    n = C.c_uint64()
    check(lib.hq_plan_serialize(num_qubits, arr, len(gates), C.byref(o), None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value)
    check(lib.hq_plan_serialize(num_qubits, arr, len(gates), C.byref(o), buf, n.value, C.byref(n)))
    return buf.raw[:n.value]


def inspect_schedule(data: bytes) -> dict:
    """Host only: check schedule bytes and list their groups."""
    nq, ngates, ng = C.c_int32(), C.c_int32(), C.c_int32()
    check(lib.hq_schedule_inspect(data, len(data), C.byref(nq), C.byref(ngates), C.byref(ng),
                                  None, None, None, None))
    k = max(1, ng.value)
    b, g, w = (C.c_int32 * k)(), (C.c_int32 * k)(), (C.c_int32 * k)()
    r = (C.c_uint64 * k)()
    check(lib.hq_schedule_inspect(data, len(data), None, None, None, b, g, w, r))
    return {"num_qubits": nq.value, "num_gates": ngates.value,
            "groups": [(b[i], g[i], w[i], r[i]) for i in range(ng.value)]}


def cost_params() -> dict:
    """The cost model's constants (seconds per amplitude per pass, and per launch)."""
    p = hq_cost_params()
    check(lib.hq_cost_params_get(C.byref(p)))
    return {k: getattr(p, k) for k, _ in hq_cost_params._fields_}


def set_cost_params(params: dict):
    p = hq_cost_params()
    check(lib.hq_cost_params_get(C.byref(p)))
    for k, v in params.items():
        setattr(p, k, float(v))
    check(lib.hq_cost_params_set(C.byref(p)))


def autotune(num_qubits: int = 0) -> dict:
    """Measure the cost model on this GPU and install it (replaces the
    reference's offline calibration and parameter files)."""
    p = hq_cost_params()
    check(lib.hq_autotune(num_qubits, C.byref(p)))
    return {k: getattr(p, k) for k, _ in hq_cost_params._fields_}


def parse_qasm(text: str) -> tuple[int, list]:
    """OpenQASM 2 text -> (num_qubits, [Gate]); the reference parser's subset
    (main.cpp:12-230) plus u2, id, swap and skipped creg/barrier/measure."""
    b = text.encode()
    n, cnt = C.c_int32(), C.c_int32()
    check(lib.hq_qasm_parse(b, C.byref(n), None, 0, C.byref(cnt)))
    arr = (hq_gate * max(1, cnt.value))()
    check(lib.hq_qasm_parse(b, C.byref(n), arr, cnt.value, C.byref(cnt)))
    return n.value, [Gate(arr[i]) for i in range(cnt.value)]


# --------------------------------------------------------------------------- state

class State:
    """A device-resident complex64 state vector of n qubits."""

    def __init__(self, n: int, zero: bool = True):
        self.n = n
        self._h = C.c_void_p()
        check(lib.hq_state_create(n, C.byref(self._h)))
        if zero:
            self.init_zero()

    @classmethod
    def _borrow(cls, handle, n: int) -> "State":
        """A view of a state owned by the library (e.g. a served result)."""
        st = cls.__new__(cls)
        st.n = n
        st._h = C.c_void_p(handle)
        st._borrowed = True
        return st

    @property
    def handle(self):
        return self._h

    def init_zero(self):
        check(lib.hq_state_init_zero(self._h))

    def load(self, amps: np.ndarray):
        a = np.ascontiguousarray(amps, dtype=np.complex64)
        assert a.size == (1 << self.n)
        check(lib.hq_state_load(self._h, a.ctypes.data))

    def store(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(1 << self.n, dtype=np.complex64)
        assert out.dtype == np.complex64 and out.size == (1 << self.n) and out.flags.c_contiguous
        check(lib.hq_state_store(self._h, out.ctypes.data))
        return out

    def store_async(self, out: np.ndarray) -> np.ndarray:
        """Start the readback into `out` (pinned memory for full speed) and
        return at once; `wait()` before reading `out`."""
        assert out.dtype == np.complex64 and out.size == (1 << self.n) and out.flags.c_contiguous
        check(lib.hq_state_store_async(self._h, out.ctypes.data))
        self._pending_out = out  # kept alive until the copy lands
        return out

    def wait(self):
        check(lib.hq_state_wait(self._h))
        self._pending_out = None

    def amps(self, idx) -> np.ndarray:
        idx = np.ascontiguousarray(idx, dtype=np.uint64)
        out = np.empty(idx.size, dtype=np.complex64)
        check(lib.hq_state_amps(self._h, idx.ctypes.data, idx.size, out.ctypes.data))
        return out

    def layout(self) -> list[int]:
        pos = (C.c_int32 * self.n)()
        check(lib.hq_state_layout(self._h, pos))
        return list(pos)

    def norm(self) -> float:
        v = C.c_double()
        check(lib.hq_state_norm(self._h, C.byref(v)))
        return v.value

    def prob_zero(self, q: int) -> float:
        v = C.c_double()
        check(lib.hq_state_prob_zero(self._h, q, C.byref(v)))
        return v.value

    def marginals(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float64)
        check(lib.hq_state_marginals(self._h, out.ctypes.data))
        return out

    def sample(self, shots: int, seed: int = 0) -> np.ndarray:
        """`shots` logical basis indices drawn from |amp|^2 (seeded SplitMix64 draws)."""
        out = np.empty(max(1, shots), dtype=np.uint64)
        check(lib.hq_state_sample(self._h, shots, seed, out.ctypes.data))
        return out[:shots]

    def remap(self, new_pos):
        arr = (C.c_int32 * self.n)(*new_pos)
        check(lib.hq_state_remap(self._h, arr))

    def apply_gates(self, gates):
        arr = gate_array(gates)
        check(lib.hq_apply_gates(self._h, arr, len(gates)))

    def apply_oshm_group(self, gates, tile_mask: int):
        arr = gate_array(gates)
        check(lib.hq_apply_oshm_group(self._h, arr, len(gates), tile_mask))

    def apply_transmm_group(self, gates, group_mask: int, precision: str = "bf16x3"):
        arr = gate_array(gates)
        check(lib.hq_apply_transmm_group(self._h, arr, len(gates), group_mask,
                                         _PRECISIONS[precision]))

    def apply_unitary(self, U: np.ndarray, group_mask: int, precision: str = "bf16x3"):
        u = np.ascontiguousarray(np.asarray(U, dtype=np.complex128).T)  # column-major
        check(lib.hq_apply_unitary(self._h, u.ctypes.data, group_mask, _PRECISIONS[precision]))

    def free(self):
        if self._h and not getattr(self, "_borrowed", False):
            lib.hq_state_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def group_unitary(gates, group_mask: int) -> np.ndarray:
    """FP64 fused unitary of gates on the qubits of group_mask (composed on the GPU)."""
    m = bin(group_mask).count("1")
    out = np.empty((1 << m) * (1 << m), dtype=np.complex128)
    arr = gate_array(gates)
    check(lib.hq_group_unitary(arr, len(gates), group_mask, out.ctypes.data))
    return out.reshape(1 << m, 1 << m).T  # stored column-major


# --------------------------------------------------------------------------- circuit

@dataclass
class ResultItem:
    """src/circuit.h:9-18"""
    idx: int
    amp: complex

    def __str__(self):
        def zw(x):  # zero_wrapper, src/utils.cpp:77-84
            return 0.0 if -1e-14 < x < 1e-14 else x
        p = abs(self.amp) ** 2
        return f"{self.idx} {p:.12f}: {zw(self.amp.real):.12f} {zw(self.amp.imag):.12f}"


class Circuit:
    """Circuit(n) / addGate / compile / run / ampAt, src/circuit.h:20-46."""

    def __init__(self, numQubits: int):
        self.numQubits = numQubits
        self._h = C.c_void_p()
        check(lib.hq_circuit_create(numQubits, C.byref(self._h)))
        self.state: State | None = None
        self.result: np.ndarray | None = None
        self.gates: list[Gate] = []

    @classmethod
    def from_qasm(cls, text: str) -> "Circuit":
        """parse_circuit, main.cpp:65-230."""
        n, gates = parse_qasm(text)
        c = cls(n)
        c.addGates(gates)
        return c

    @classmethod
    def deserialize(cls, data: bytes) -> "Circuit":
        """A compiled circuit from schedule bytes (no partitioning)."""
        h = C.c_void_p()
        check(lib.hq_circuit_deserialize(data, len(data), C.byref(h)))
        nq = C.c_int32()
        check(lib.hq_schedule_inspect(data, len(data), C.byref(nq), None, None, None, None, None,
                                      None))
        c = cls.__new__(cls)
        c.numQubits = nq.value
        c._h = h
        c.state = None
        c.result = None
        c.gates = []
        return c

    def serialize(self) -> bytes:
        """The compiled schedule as bytes (Schedule::serialize, src/schedule.cpp:156-325)."""
        n = C.c_uint64()
        check(lib.hq_circuit_serialize(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        check(lib.hq_circuit_serialize(self._h, buf, n.value, C.byref(n)))
        return buf.raw[:n.value]

    @property
    def handle(self):
        return self._h

    def addGate(self, gate: Gate):
        self.gates.append(gate)
        check(lib.hq_circuit_add_gates(self._h, C.byref(gate.g), 1))

    def addGates(self, gates):
        self.gates.extend(gates)
        arr = gate_array(gates)
        check(lib.hq_circuit_add_gates(self._h, arr, len(gates)))

    def compile(self, backend: str | int = "oshm", tile_qubits: int = 0, coalesce: int = 0,
                mm_qubits: int = 0, precision: str | int = "bf16x3", reference_grouping: bool = False,
                specialize: int = 2):
        o = _compile_options(backend, tile_qubits, coalesce, mm_qubits, precision, reference_grouping,
                             specialize)
        check(lib.hq_circuit_compile(self._h, C.byref(o)))

    def schedule(self):
        """List of (backend, num_gates, width, related_mask) per gate group."""
        ng = C.c_int32()
        check(lib.hq_circuit_schedule(self._h, C.byref(ng), None, None, None, None))
        k = ng.value
        b = (C.c_int32 * max(1, k))()
        g = (C.c_int32 * max(1, k))()
        w = (C.c_int32 * max(1, k))()
        r = (C.c_uint64 * max(1, k))()
        check(lib.hq_circuit_schedule(self._h, C.byref(ng), b, g, w, r))
        return [(b[i], g[i], w[i], r[i]) for i in range(k)]

    def group_gates(self, gi: int) -> list[int]:
        cnt = C.c_int32()
        check(lib.hq_circuit_group_gates(self._h, gi, None, 0, C.byref(cnt)))
        arr = (C.c_int32 * max(1, cnt.value))()
        check(lib.hq_circuit_group_gates(self._h, gi, arr, cnt.value, C.byref(cnt)))
        return list(arr[: cnt.value])

    def run_on(self, state: State) -> float:
        us = C.c_double()
        check(lib.hq_circuit_run(self._h, state.handle, C.byref(us)))
        return us.value

    def run_to_host(self, state: State, out: np.ndarray) -> float:
        """Run on `state` and leave the final state (logical order) in `out`, a
        complex64 array of 2^n entries; device time in us.  With a pinned
        `out` (PinnedBuffer.array) the last group writes it in the same pass."""
        if out.dtype != np.complex64 or out.size != (1 << self.numQubits) or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous complex64 array of 2^n amplitudes")
        us = C.c_double()
        check(lib.hq_circuit_run_to_host(self._h, state.handle, C.c_void_p(out.ctypes.data), C.byref(us)))
        return us.value

    def profile(self, state: State) -> np.ndarray:
        """Per-group device time (us) of one run on `state`."""
        k = len(self.schedule())
        out = np.zeros(max(1, k), dtype=np.float64)
        check(lib.hq_circuit_profile(self._h, state.handle, out.ctypes.data))
        return out[:k]

    def predict(self) -> np.ndarray:
        """The cost model's device time (us) of each group (hq_circuit_predict)."""
        k = len(self.schedule())
        out = np.zeros(max(1, k), dtype=np.float64)
        check(lib.hq_circuit_predict(self._h, out.ctypes.data))
        return out[:k]

    def program_bytes(self) -> int:
        v = C.c_uint64()
        check(lib.hq_circuit_program_bytes(self._h, C.byref(v)))
        return v.value

    def capture_graph(self, state: State):
        check(lib.hq_circuit_capture_graph(self._h, state.handle))

    def enqueue(self, state: State):
        check(lib.hq_circuit_enqueue(self._h, state.handle))

    def run(self, copy_back: bool = True, destroy: bool = True) -> float:
        """src/circuit.cpp:16-71: init |0..0>, run, optional copy-back; returns us."""
        if self.state is None:
            self.state = State(self.numQubits, zero=True)
        else:
            self.state.init_zero()
        us = self.run_on(self.state)
        if copy_back:
            self.result = self.state.store()
        if destroy:
            self.state.free()
            self.state = None
        return us

    def ampAt(self, idx: int) -> ResultItem:
        assert self.result is not None, "run(copy_back=True) first"
        return ResultItem(idx, complex(self.result[idx]))

    def ampAtGPU(self, idx: int) -> complex:
        assert self.state is not None, "run(destroy=False) first"
        return complex(self.state.amps([idx])[0])

    def printState(self):
        """src/circuit.cpp:285-308: amplitudes 0..127, then |a|^2 > 0.001 above 127."""
        assert self.result is not None
        for i in range(min(128, self.result.size)):
            print(self.ampAt(i))
        p = np.abs(self.result) ** 2
        for i in np.nonzero(p > 0.001)[0]:
            if i >= 128:
                print(self.ampAt(int(i)))

    def __del__(self):
        try:
            if self._h:
                lib.hq_circuit_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass


REQ_STATUS = {0: "planning", 1: "queued", 2: "running", 3: "done", 4: "failed"}


def server_options(hbm_budget: int | None = None, step_budget_us: float = 0.0,
                   planner_threads: int = 0, tile_qubits: int = 0,
                   jit_min_qubits: int = 0) -> hq_server_options:
    o = hq_server_options()
    check(lib.hq_server_options_default(C.byref(o)))
    if jit_min_qubits:
        o.jit_min_qubits = jit_min_qubits
    if hbm_budget is not None:
        o.hbm_budget = hbm_budget
    if step_budget_us:
        o.step_budget_us = step_budget_us
    if planner_threads:
        o.planner_threads = planner_threads
    o.tile_qubits = tile_qubits
    return o


def server_check(n: int, gates, **kw):
    """Host-only admission checks of a request (raises HQError)."""
    o = server_options(**kw)
    arr = gate_array(gates)
    check(lib.hq_server_check(C.byref(o), n, arr, len(gates)))


class Server:
    """Request loop: submit circuits, get results back as they finish.

    Arriving requests are admitted while their states fit `hbm_budget` and
    run in continuous batches (one persistent launch per step over every
    admitted request's next gate groups)."""

    def __init__(self, hbm_budget: int | None = None, step_budget_us: float = 0.0,
                 planner_threads: int = 0, tile_qubits: int = 0, jit_min_qubits: int = 0):
        self._h = C.c_void_p()
        o = server_options(hbm_budget, step_budget_us, planner_threads, tile_qubits,
                           jit_min_qubits)
        check(lib.hq_server_create(C.byref(o), C.byref(self._h)))
        self._n: dict[int, int] = {}

    def submit(self, n: int, gates) -> int:
        """gates: Gate objects, or an array made by gate_array() beforehand."""
        arr = gates if isinstance(gates, C.Array) else gate_array(gates)
        rid = C.c_int64()
        check(lib.hq_server_submit(self._h, n, arr, len(gates), C.byref(rid)))
        self._n[rid.value] = n
        return rid.value

    def wait(self, rid: int, timeout: float = 60.0) -> str:
        st = C.c_int32()
        check(lib.hq_server_wait(self._h, rid, timeout, C.byref(st)))
        return REQ_STATUS[st.value]

    def poll(self, cap: int = 4096) -> list[int]:
        ids = (C.c_int64 * cap)()
        k = C.c_int32()
        check(lib.hq_server_poll(self._h, ids, cap, C.byref(k)))
        return list(ids[: k.value])

    def state(self, rid: int) -> State:
        h = C.c_void_p()
        check(lib.hq_server_state(self._h, rid, C.byref(h)))
        return State._borrow(h.value, self._n[rid])

    def times(self, rid: int) -> tuple[float, float, float]:
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        check(lib.hq_server_times(self._h, rid, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def steps(self, rid: int) -> tuple[int, int]:
        """(first, last) step index the request's work ran in."""
        a, b = C.c_int64(), C.c_int64()
        check(lib.hq_server_steps(self._h, rid, C.byref(a), C.byref(b)))
        return a.value, b.value

    def release(self, rid: int):
        check(lib.hq_server_release(self._h, rid))

    def stats(self) -> dict:
        v = [C.c_int64(), C.c_int64(), C.c_int64(), C.c_uint64(), C.c_uint64()]
        check(lib.hq_server_stats(self._h, *[C.byref(x) for x in v]))
        return dict(zip(["steps", "items", "finished", "resident_bytes", "peak_resident_bytes"],
                        [x.value for x in v]))

    def plan_cache(self) -> dict:
        h, e = C.c_int64(), C.c_int64()
        check(lib.hq_server_plan_cache(self._h, C.byref(h), C.byref(e)))
        return {"hits": h.value, "entries": e.value}

    def close(self):
        if self._h:
            lib.hq_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many circuits (uneven qubit counts) in one persistent launch.

    add(circuit, state) pairs a circuit with the state it runs on; compile()
    plans every circuit as OShareMem groups (tile width per circuit from the
    cost model unless tile_qubits is given); run() executes all of them."""

    def __init__(self):
        self._h = C.c_void_p()
        check(lib.hq_batch_create(C.byref(self._h)))
        self._keep: list = []  # circuits and states must outlive the batch's runs

    @property
    def handle(self):
        return self._h

    def add(self, circuit: "Circuit", state: State) -> int:
        idx = C.c_int32()
        check(lib.hq_batch_add(self._h, circuit.handle, state.handle, C.byref(idx)))
        self._keep.append((circuit, state))
        return idx.value

    def compile(self, tile_qubits: int = 0, coalesce: int = 0):
        o = hq_compile_options()
        check(lib.hq_compile_options_default(C.byref(o)))
        o.tile_qubits = tile_qubits
        o.coalesce = coalesce
        check(lib.hq_batch_compile(self._h, C.byref(o)))

    def run(self, zero_init: bool = True) -> float:
        """Run every circuit once; returns device microseconds."""
        us = C.c_double()
        check(lib.hq_batch_run(self._h, 1 if zero_init else 0, C.byref(us)))
        return us.value

    def enqueue(self, zero_init: bool = True):
        check(lib.hq_batch_enqueue(self._h, 1 if zero_init else 0))

    def capture_graph(self, zero_init: bool = True):
        check(lib.hq_batch_capture_graph(self._h, 1 if zero_init else 0))

    def inject_stall(self):
        """Test hook: the next direct run's bounded device wait expires (HQ_ERR_TIMEOUT)."""
        check(lib.hq_batch_inject_stall(self._h))

    def info(self) -> dict:
        nc, ng, ni, pb = C.c_int32(), C.c_int64(), C.c_int64(), C.c_uint64()
        check(lib.hq_batch_info(self._h, C.byref(nc), C.byref(ng), C.byref(ni), C.byref(pb), None))
        tiles = (C.c_int32 * max(1, nc.value))()
        check(lib.hq_batch_info(self._h, None, None, None, None, tiles))
        return {"circuits": nc.value, "groups": ng.value, "items": ni.value,
                "pass_bytes": pb.value, "tile_qubits": list(tiles[: nc.value])}

    def free(self):
        if self._h:
            lib.hq_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


__all__ = ["Circuit", "Batch", "Server", "Gate", "State", "parse_qasm", "autotune",
           "cost_params", "set_cost_params", "ResultItem", "HQError", "init", "device_info",
           "group_unitary", "set_hbm_budget", "hbm_in_use", "lib", "LIB_PATH"]
