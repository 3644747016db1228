"""OpenQASM 2 front-end (the reference parser's subset, main.cpp:12-230):
parsing on the host against hand-written expectations, through the C++
facade, and (GPU) a parsed QFT against the FP64 oracle."""
import math
import subprocess

import numpy as np
import pytest

import hyquas_gb300 as hq
from hyquas_gb300 import workloads as W

TEXT = """OPENQASM 2.0;
include "qelib1.inc";
// a comment line
qreg q[5];
creg c[5];
h q[0];
cx q[0],q[1];
ccx q[0],q[1],q[2];
cy q[3],q[4];
cz q[2],q[4];
x q[1]; y q[2];
s q[3];
sdg q[3];
t q[4];
tdg q[4];
crx(pi/2) q[0],q[3];
cry(pi*0.25) q[1],q[3];
crz(0.125) q[2],q[3];
cu1(pi/4) q[3],q[0];
u1(pi*1.5) q[2];
u2(0.5,-pi/2) q[1];
u3(0.1,0.2,0.3) q[0];
rx(-0.75) q[4];
ry(pi/3) q[0];
rz(pi*2) q[1];
barrier q[0],q[1];
swap q[0],q[4];
measure q[0] -> c[0];
"""


def expected():
    pi = math.pi
    G = hq.Gate
    return [G.H(0), G.CNOT(0, 1), G.CCX(0, 1, 2), G.CY(3, 4), G.CZ(2, 4), G.X(1), G.S(3),
            G.SDG(3), G.T(4), G.TDG(4), G.CRX(0, 3, pi / 2), G.CRY(1, 3, pi * 0.25),
            G.CRZ(2, 3, 0.125), G.CU1(3, 0, pi / 4), G.U1(2, pi * 1.5), G.U2(1, 0.5, -pi / 2),
            G.U3(0, 0.1, 0.2, 0.3), G.RX(4, -0.75), G.RY(0, pi / 3), G.RZ(1, pi * 2),
            G.SWAP(0, 4)]


def key(g):
    return (g.g.type, g.g.target, g.g.control, g.g.control2, tuple(round(x, 15) for x in g.g.mat))


def test_parse_matches_factories():
    n, gates = hq.parse_qasm(TEXT)
    assert n == 5
    # `x q[1]; y q[2];` is one line: the reference reads one statement per line
    assert [key(g) for g in gates] == [key(g) for g in expected()]


@pytest.mark.parametrize("bad", [
    "qreg q[3];\nfoo q[0];\n",            # unknown gate
    "h q[0];\n",                          # gate before qreg
    "qreg q[3];\ncx q[0];\n",             # wrong qubit count
    "qreg q[3];\nrx(pi/0) q[0];\n",       # bad parameter
    "qreg q[3];\nu3(0.1,0.2) q[0];\n",    # wrong parameter count
    "qreg q[3];\nh q[3];\n",              # qubit out of range
    "// nothing\n",                       # no qreg
])
def test_parse_errors(bad):
    with pytest.raises(hq.HQError):
        hq.parse_qasm(bad)


def test_error_names_the_line():
    with pytest.raises(hq.HQError) as e:
        hq.parse_qasm("qreg q[4];\nh q[0];\nh q[1];\nbogus q[2];\n")
    assert "line 4" in str(e.value)


def qft_qasm(n):
    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', f"qreg q[{n}];"]
    for j in range(n - 1, -1, -1):
        lines.append(f"h q[{j}];")
        for k in range(j - 1, -1, -1):
            lines.append(f"cu1(pi/{1 << (j - k)}) q[{k}],q[{j}];")
    for i in range(n // 2):
        lines.append(f"swap q[{i}],q[{n - 1 - i}];")
    return "\n".join(lines) + "\n"


def test_qft_text_equals_workload():
    n, gates = hq.parse_qasm(qft_qasm(10))
    ref = W.to_gates(W.qft(10))
    assert [key(g) for g in gates] == [key(g) for g in ref]


def test_facade_parse_circuit(tmp_path):
    from test_facade import ROOT
    src = tmp_path / "c.qasm"
    src.write_text(TEXT)
    out = tmp_path / "facade_main"
    lib = hq.LIB_PATH
    subprocess.run(["g++", "-O2", "-std=c++17", str(ROOT / "tests/cpp/facade_main.cpp"), "-o",
                    str(out), f"-L{lib.parent}", "-lhyquas_gb300", f"-Wl,-rpath,{lib.parent}"],
                   check=True)
    txt = subprocess.run([str(out), "qasm", str(src)], check=True, capture_output=True,
                         text=True).stdout.splitlines()
    assert len(txt) == len(expected())
    assert txt[2] == "type 0 target 2 control 0 control2 1"


@pytest.mark.gpu
def test_parsed_qft_runs(hq, oracle):
    n = 12
    c = hq.Circuit.from_qasm(qft_qasm(n))
    c.compile("oshm")
    psi = W.random_state(5, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    c.run_on(s)
    ref = np.fft.ifft(psi.astype(np.complex128)) * np.sqrt(1 << n)
    cmp = oracle.compare(ref, s.store())
    assert cmp["max_abs_err"] <= 1e-5 and cmp["one_minus_fidelity"] <= 1e-6, cmp


def test_mutated_text_never_crashes():
    """Damaged QASM (random characters replaced, cut short, lines repeated) is
    either parsed or refused with an error -- the parser never misbehaves."""
    rng = W.SplitMix64(99)
    alphabet = "qc[](),;.*/+-0123456789 piuxyzhtsdgcrOPENQASM\n"
    ok = refused = 0
    for _ in range(300):
        t = list(TEXT)
        for _ in range(1 + rng.below(6)):
            t[rng.below(len(t))] = alphabet[rng.below(len(alphabet))]
        text = "".join(t)
        if rng.below(3) == 0:
            text = text[:rng.below(len(text))]
        try:
            n, gates = hq.parse_qasm(text)
            assert 0 < n <= 36
            for g in gates:
                assert 0 <= g.g.target < n
            ok += 1
        except hq.HQError:
            refused += 1
    assert ok + refused == 300 and refused > 0
