"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs oracle/_ref/ref_driver_{group,blas,mix} -- the reference's CPU sources
(src/gate.cpp, src/compiler.cpp, src/evaluator.cpp, src/schedule.cpp) compiled
where they lie by `make -C oracle ref` -- on seeded circuits and stores:

  matrices.json     every factory's 2x2 matrix for a set of angles
                    (Gate::* in src/gate.cpp:9-342)
  unitary_*.npz     small circuits run through GateGroup::initCPUMatrix
                    (src/schedule.cpp:578-702): output states for |0..0> and a
                    random input
  partition_*.json  Compiler::run (src/compiler.cpp:70-165) group partitions
                    for the group (OShareMem), blas (TransMM) and, at 28
                    qubits, mix backends

Needs the reference checkout, so it runs in the development container only;
its outputs are committed and the tests read only those.
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
from hyquas_gb300 import workloads as W  # noqa: E402

REF = ROOT / "oracle" / "_ref"
ALL_TYPES = list(range(22))  # CCX .. RZ
NPARAMS = {W.CRX: 1, W.CRY: 1, W.CU1: 1, W.CRZ: 1, W.U1: 1, W.U2: 2, W.U3: 3, W.RX: 1, W.RY: 1, W.RZ: 1}


def run_driver(backend: str, n: int, desc, cmd: str, psi=None) -> str:
    lines = [f"n {n}"]
    for (t, q, c, c2, p) in desc:
        pp = list(p) + [0.0] * (3 - len(p))
        lines.append(f"g {t} {q} {c} {c2} {pp[0]:.17g} {pp[1]:.17g} {pp[2]:.17g}")
    if psi is not None:
        for a in psi:
            lines.append(f"s {a.real:.17g} {a.imag:.17g}")
    lines.append(f"cmd {cmd}")
    r = subprocess.run([str(REF / f"ref_driver_{backend}")], input="\n".join(lines) + "\n",
                       capture_output=True, text=True, check=True)
    return r.stdout


def random_circuit(rng: W.SplitMix64, n: int, count: int, types=ALL_TYPES):
    desc = []
    for _ in range(count):
        t = types[rng.below(len(types))]
        qs = rng.shuffle(range(n))[:3]
        params = tuple(rng.uniform() * W.TWO_PI for _ in range(NPARAMS.get(t, 0)))
        if t == W.CCX:
            desc.append((t, qs[2], qs[0], qs[1], ()))
        elif t <= W.CRZ:
            desc.append((t, qs[1], qs[0], -1, params))
        else:
            desc.append((t, qs[0], -1, -1, params))
    return desc


def make_matrices():
    rng = W.SplitMix64(11)
    out = []
    for t in ALL_TYPES:
        for trial in range(3):
            params = tuple(rng.uniform() * W.TWO_PI - math.pi for _ in range(NPARAMS.get(t, 0)))
            if t == W.CCX:
                desc = [(t, 2, 0, 1, params)]
            elif t <= W.CRZ:
                desc = [(t, 1, 0, -1, params)]
            else:
                desc = [(t, 0, -1, -1, params)]
            txt = run_driver("group", 3, desc, "matrices")
            vals = [float(x) for x in txt.split()[1:9]]
            out.append({"type": t, "params": list(params), "mat": vals})
    (HERE / "matrices.json").write_text(json.dumps(out, indent=0))
    print("matrices.json", len(out))


def make_unitaries():
    rng = W.SplitMix64(12)
    cases = [(4, 30), (5, 60), (6, 80), (7, 120), (8, 160)]
    for idx, (n, count) in enumerate(cases):
        desc = random_circuit(rng, n, count)
        zero = run_driver("blas", n, desc, "unitary")
        out0 = np.array([complex(float(a), float(b)) for (_, a, b) in
                         (ln.split() for ln in zero.strip().splitlines())])
        psi = W.random_state(100 + idx, n).astype(np.complex128)
        txt = run_driver("blas", n, desc, "unitary", psi=psi)
        out1 = np.array([complex(float(a), float(b)) for (_, a, b) in
                         (ln.split() for ln in txt.strip().splitlines())])
        np.savez_compressed(HERE / f"unitary_n{n}.npz", desc=np.array(json.dumps(desc)),
                            out_zero=out0, psi=psi, out_psi=out1)
        print(f"unitary_n{n}.npz", len(desc))


def parse_partition(txt: str):
    groups, final = [], None
    for ln in txt.strip().splitlines():
        tok = ln.split()
        if tok[0] == "group":
            colon = tok.index(":")
            posi = tok.index("pos")
            groups.append({"backend": tok[1], "related": int(tok[3]), "matqubit": int(tok[5]),
                           "gates": [int(x) for x in tok[colon + 1:posi]]})
        elif tok[0] == "final":
            final = [int(x) for x in tok[1:]]
    return groups, final


def make_partitions():
    cases = []
    rng = W.SplitMix64(13)
    no_ccx = [t for t in ALL_TYPES if t != W.CCX]
    for n, count in ((12, 300), (16, 600), (20, 900)):
        cases.append((f"random_n{n}", n, random_circuit(rng, n, count, no_ccx), ("group", "blas")))
    cases.append(("grid_5x6_c20", 30, W.grid_random(2, 5, 6, 20), ("group", "blas")))
    cases.append(("u3cnot_n20", 20, W.plain_u3_cnot(1, 20, 10), ("group", "blas")))
    cases.append(("qft_n28", 28, [g for g in W.qft(28) if g[0] != W.SWAP], ("group", "blas", "mix")))
    cases.append(("grid_4x7_c20", 28, W.grid_random(2, 4, 7, 20), ("group", "blas", "mix")))
    for name, n, desc, backends in cases:
        rec = {"name": name, "n": n, "desc": desc, "backends": {}}
        for b in backends:
            groups, final = parse_partition(run_driver(b, n, desc, "compile"))
            rec["backends"][b] = {"groups": groups, "final": final}
        (HERE / f"partition_{name}.json").write_text(json.dumps(rec))
        print(f"partition_{name}.json", {b: len(v["groups"]) for b, v in rec["backends"].items()})


if __name__ == "__main__":
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref"], check=True, capture_output=True)
    make_matrices()
    make_unitaries()
    make_partitions()
