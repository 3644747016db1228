"""C-ABI surface, host-side gate factories and error behaviour (no GPU needed)."""
import ctypes as C
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import hyquas_gb300 as hq

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)  # drop comments
        names |= set(re.findall(r"\b(hq_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    out = subprocess.run(["nm", "-D", "--defined-only", str(hq.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (hq_[a-z0-9_]+)$", out, re.M))
    declared = declared_symbols()
    assert len(declared) > 30
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    for name in declared:
        assert hasattr(hq.lib, name)


def test_gate_factories_match_reference_matrices():
    recs = json.loads((GOLDEN / "matrices.json").read_text())
    for r in recs:
        g = hq.hq_gate()
        p = (C.c_double * 3)(*(list(r["params"]) + [0.0] * (3 - len(r["params"]))))
        t = r["type"]
        c, c2 = (0, 1) if t == 0 else ((0, -1) if t <= 7 else (-1, -1))
        hq.check(hq.lib.hq_gate_make(t, 2, c, c2, p, C.byref(g)))
        np.testing.assert_allclose(list(g.mat), r["mat"], rtol=0, atol=1e-15, err_msg=str(r))


def test_factory_argument_order_follows_reference():
    g = hq.Gate.CNOT(3, 5)  # control first (src/gate.h:31)
    assert (g.controlQubit, g.targetQubit) == (3, 5)
    g = hq.Gate.CCX(1, 2, 7)
    assert (g.controlQubit, g.controlQubit2, g.targetQubit) == (1, 2, 7)
    g = hq.Gate.CU1(0, 4, 0.5)
    assert (g.controlQubit, g.targetQubit) == (0, 4)
    assert hq.Gate.T(0).isDiagonal() and not hq.Gate.H(0).isDiagonal()


def test_errors_are_codes_not_exits():
    g = hq.hq_gate()
    assert hq.lib.hq_gate_make(99, 0, -1, -1, None, C.byref(g)) == -1
    assert b"unknown gate type" in hq.lib.hq_last_error()
    assert hq.lib.hq_gate_make(hq.CNOT, 0, -1, -1, None, C.byref(g)) == -1
    assert hq.lib.hq_gate_make(hq.H, 0, -1, -1, None, None) == -1
    with pytest.raises(hq.HQError):
        hq.Gate.CCX(0, -1, 2)


def test_circuit_rejects_out_of_range_gates():
    c = hq.Circuit(4)
    with pytest.raises(hq.HQError):
        c.addGate(hq.Gate.H(4))
    with pytest.raises(hq.HQError):
        c.addGate(hq.Gate.CNOT(2, 2))
    c.addGate(hq.Gate.H(3))
    n = C.c_int32()
    hq.check(hq.lib.hq_circuit_num_gates(c.handle, C.byref(n)))
    assert n.value == 1
    with pytest.raises(hq.HQError):
        hq.Circuit(37)


def test_compile_options_validated_without_device():
    gates = hq.gate_array([hq.Gate.H(0)])
    o = hq.hq_compile_options()
    hq.check(hq.lib.hq_compile_options_default(C.byref(o)))
    o.tile_qubits = 20
    ng = C.c_int32()
    assert hq.lib.hq_plan_groups(10, gates, 1, C.byref(o), C.byref(ng), None, None, None, None,
                                 None, None) == -1
    o.tile_qubits = 0
    o.backend = 7
    assert hq.lib.hq_plan_groups(10, gates, 1, C.byref(o), C.byref(ng), None, None, None, None,
                                 None, None) == -1


def test_pinned_view_keeps_its_buffer_alive():
    """PinnedBuffer.array's base holds the PinnedBuffer, so a view taken from a
    temporary buffer object does not outlive the memory (host-only check of
    the view mechanism, on ordinary memory)."""
    import gc
    import weakref
    import numpy as np
    import hyquas_gb300 as hq

    class Owner:
        pass

    backing = np.arange(8, dtype=np.complex64)
    owner = Owner()
    ref = weakref.ref(owner)
    view = np.asarray(hq._PinnedView(owner, backing.ctypes.data, 8, np.complex64))
    del owner
    gc.collect()
    assert ref() is not None
    assert view.dtype == np.complex64 and view.shape == (8,) and view[3] == backing[3]
    del view
    gc.collect()
    assert ref() is None
