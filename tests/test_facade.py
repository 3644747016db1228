"""The header-only C++ facade (hyquas_gb300/circuit.hpp): it compiles against
the C ABI, its gate factories give the oracle's matrices (host only), and on a
GPU a Circuit built through it matches the FP64 oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def facade_bin(tmp_path_factory):
    out = tmp_path_factory.mktemp("facade") / "facade_main"
    lib = hq.LIB_PATH
    subprocess.run(["g++", "-O2", "-std=c++17", str(ROOT / "tests/cpp/facade_main.cpp"),
                    "-o", str(out), f"-L{lib.parent}", "-lhyquas_gb300",
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    return out


def test_factories_match_oracle(facade_bin, oracle):
    txt = subprocess.run([str(facade_bin), "gates"], check=True, capture_output=True,
                         text=True).stdout
    params = {"CRX": (0.3,), "CRY": (0.4,), "CU1": (0.5,), "CRZ": (0.6,), "U1": (0.7,),
              "U2": (0.8, 0.9), "U3": (1.0, 1.1, 1.2), "RX": (1.3,), "RY": (1.4,), "RZ": (1.5,)}
    types = {"CCX": W.CCX, "CNOT": W.CNOT, "CY": W.CY, "CZ": W.CZ, "CRX": W.CRX, "CRY": W.CRY,
             "CU1": W.CU1, "CRZ": W.CRZ, "U1": W.U1, "U2": W.U2, "U3": W.U3, "H": W.H, "X": W.X,
             "Y": W.Y, "Z": W.Z, "S": W.S, "SDG": W.SDG, "T": W.T, "TDG": W.TDG, "RX": W.RX,
             "RY": W.RY, "RZ": W.RZ, "ID": 23}
    seen = 0
    for line in txt.splitlines():
        name, *vals = line.split()
        got = np.array([float(x) for x in vals])
        ref = oracle.gate_matrix(types[name], params.get(name, ()))
        assert np.allclose(got, ref, atol=1e-15), name
        seen += 1
    assert seen == 23


@pytest.mark.gpu
@pytest.mark.parametrize("n", [9, 14])
def test_facade_circuit_matches_oracle(facade_bin, oracle, n):
    txt = subprocess.run([str(facade_bin), "run", str(n), "7"], check=True, capture_output=True,
                         text=True).stdout
    v = np.array([[float(x) for x in ln.split()] for ln in txt.splitlines()])
    got = (v[:, 0] + 1j * v[:, 1]).astype(np.complex64)
    # the same circuit, generated the same way
    s = 7
    mask = (1 << 64) - 1

    def uni():
        nonlocal s
        s = (s * 6364136223846793005 + 1442695040888963407) & mask
        return (s >> 11) * (1.0 / 9007199254740992.0) * 6.283185307179586
    desc = []
    for layer in range(4):
        for q in range(n):
            a, b, d = uni(), uni(), uni()
            desc.append((W.U3, q, -1, -1, (a, b, d)))
        for q in range(layer & 1, n - 1, 2):
            desc.append((W.CNOT, q + 1, q, -1, ()))
    c = oracle.compare(oracle.run_f64(n, desc), got)
    assert c["max_abs_err"] <= 1e-5 and c["one_minus_fidelity"] <= 1e-6, c


@pytest.mark.gpu
def test_facade_schedule_round_trip(facade_bin):
    """Circuit::serialize / Circuit::deserialize through the C++ facade: the
    loaded circuit gives the same amplitudes, bit for bit."""
    txt = subprocess.run([str(facade_bin), "roundtrip", "14", "9"], check=True, capture_output=True,
                         text=True).stdout
    assert txt.startswith("ok "), txt
