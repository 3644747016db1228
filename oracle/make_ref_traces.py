#!/usr/bin/env python3
"""Trace the reference's own single-GPU runs -- TEST INFRASTRUCTURE ONLY.

Runs oracle/_ref/ref_trace_{group,serial} (the reference's host code linked
against oracle/ref_gpu/fake_cuda.cpp, built by `make -C oracle ref-gpu`) on the
benchmark circuits and on small test circuits, writing
oracle/_ref/trace_<name>.bin (the device work the reference issues) and
oracle/_ref/trace_<name>.json (its log: group counts, compile time).
oracle/ref_replay.cu replays the traces on a GPU with the reference's kernels.

Circuits come from hyquas_gb300/workloads.py (loaded by path; no native code).
"""
from __future__ import annotations

import importlib.util
import json
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"


def workloads():
    spec = importlib.util.spec_from_file_location("hq_workloads_trace",
                                                  HERE.parent / "hyquas_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def mixed_circuit(W, seed: int, n: int, count: int):
    """Every gate type the reference's two single-GPU paths apply as their
    factories define (SDG/TDG and CCX left out: the reference runs SDG/TDG
    through the S/T kernels and its grouping ignores CCX's second control)."""
    rng = W.SplitMix64(seed)
    types = [t for t in range(22) if t not in (W.CCX, W.SDG, W.TDG)]
    nparams = {W.CRX: 1, W.CRY: 1, W.CU1: 1, W.CRZ: 1, W.U1: 1, W.U2: 2, W.U3: 3, W.RX: 1,
               W.RY: 1, W.RZ: 1}
    desc = []
    for _ in range(count):
        t = types[rng.below(len(types))]
        qs = rng.shuffle(list(range(n)))[:2]
        params = tuple(rng.uniform() * W.TWO_PI for _ in range(nparams.get(t, 0)))
        if t <= W.CRZ:
            desc.append((t, qs[1], qs[0], -1, params))
        else:
            desc.append((t, qs[0], -1, -1, params))
    return desc


def circuits():
    W = workloads()
    return {
        # benchmark circuits (the grid30 and plain20 workloads of bench.py)
        "grid30_group": (30, W.grid_random(2, 5, 6, 20), "group"),
        "plain20_serial": (20, W.plain_u3_cnot(1, 20, 10), "serial"),
        # small cases for the GPU tests
        "grid16_group": (16, W.grid_random(5, 4, 4, 20), "group"),
        "mixed14_group": (14, mixed_circuit(W, 77, 14, 400), "group"),
        "mixed14_serial": (14, mixed_circuit(W, 77, 14, 400), "serial"),
    }


def circuit_text(n, desc) -> str:
    lines = [f"n {n}"]
    for (t, q, c, c2, p) in desc:
        pp = list(p) + [0.0] * (3 - len(p))
        lines.append(f"g {t} {q} {c} {c2} {pp[0]!r} {pp[1]!r} {pp[2]!r}")
    return "\n".join(lines) + "\n"


def main() -> int:
    for name, (n, desc, backend) in circuits().items():
        exe = OUT / f"ref_trace_{backend}"
        if not exe.exists():
            print(f"missing {exe}: run make -C oracle ref-gpu", file=sys.stderr)
            return 1
        trace = OUT / f"trace_{name}.bin"
        r = subprocess.run([str(exe), str(trace)], input=circuit_text(n, desc),
                           capture_output=True, text=True)
        if r.returncode != 0:
            print(f"{name}: trace failed\n{r.stdout}\n{r.stderr}", file=sys.stderr)
            return 1
        log = [ln for ln in r.stdout.splitlines() if ln.strip()]
        groups = None
        for ln in log:
            if "Total Groups:" in ln:
                groups = int(ln.split("Total Groups:")[1].split()[1])
        meta = {"name": name, "num_qubits": n, "backend": backend, "gates": len(desc),
                "groups": groups, "log": log}
        (OUT / f"trace_{name}.json").write_text(json.dumps(meta, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
