#!/usr/bin/env python3
"""Benchmark: 30-qubit random grid circuit (5x6, 20 cycles) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--backend oshm|hybrid|transmm] [--no-cpu-baseline]

A step = one full circuit (845 gates: sqrt(X)/sqrt(Y)/T per qubit and CZ on
the cycle's coupler pattern) applied to a complex64 state resident in HBM
(2^30 amplitudes = 8 GiB, larger than L2, so no flush is needed).  `value` is
circuits per second over all ranks; ms_per_step is device time per circuit.

  roofline      the OShareMem kernel: algorithmic bytes per launch (read + write
                of every amplitude = 16 * 2^30 B) over its mean launch time,
                measured with CUDA events on the library stream, against the
                measured HBM copy bandwidth (MEASURED_PEAKS.json).
  e2e           the same metric through the public API with host buffers: per
                step Circuit(30) + addGates + compile (program upload = H2D),
                |0..0> init, run, copy-back of the full state into pinned host
                memory (D2H) -- the reference's Circuit::run(copy_back=true).
  cpu_baseline  the oracle's complex64 OpenMP gate-by-gate port on this host's
                cores, on a bounded sample (the circuit's first gates), scaled
                to circuits/s.
  --impl reference   the same CPU port as the reference arm (the reference
                has no CPU implementation of the path; its GPU build needs
                sources that are not on the GPU machine).

Multi-GPU: replicas only (the single-GPU path does not shard); each rank runs
its own circuit on its own GPU, barrier + max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_QUBITS = 30
WORKLOAD = "grid 5x6 (30 qubits), 20 cycles of sqrt(X)/sqrt(Y)/T + CZ (4 coupler patterns), complex64"
METRIC = "30q grid circuit throughput (circuits/s)"
UNIT = "circuits/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = []
        for ln in Path(self.f.name).read_text().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_sample(n: int, desc, budget_s: float, threads: int):
    """Time the oracle's complex64 gate-by-gate port on the first gates of the
    circuit; returns (seconds per gate, gates run)."""
    import oracle as O
    state = np.zeros(1 << n, dtype=np.complex64)
    state[0] = 1
    k = 0
    t_total = 0.0
    # warm one gate (first touch of the 8 GiB buffer is not the algorithm)
    O.apply_f32(n, state, desc[:1], threads=threads)
    while k < len(desc) and (t_total < budget_s or k < 4):
        chunk = desc[k:k + 4]
        t0 = time.perf_counter()
        O.apply_f32(n, state, chunk, threads=threads)
        t_total += time.perf_counter() - t0
        k += len(chunk)
    return t_total / k, k


def run_reference(args, dist: Dist):
    """Reference arm: the CPU gate-by-gate port on all host cores."""
    from hyquas_gb300 import workloads as W
    if dist.rank != 0:
        return
    desc = W.grid_random(2, 5, 6, 20)
    threads = os.cpu_count() or 1
    per_step_budget = 1.5
    for _ in range(args.warmup):
        cpu_sample(N_QUBITS, desc, per_step_budget, threads)
    rates = []
    gates_run = 0
    for _ in range(args.steps):
        spg, k = cpu_sample(N_QUBITS, desc, per_step_budget, threads)
        gates_run = k
        rates.append(1.0 / (spg * len(desc)))
    value = float(np.mean(rates))
    sample = (f"each step: first {gates_run} of {len(desc)} gates at n=30 (complex64, in place, "
              f"OpenMP over amplitude pairs), time scaled to the full circuit")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "implementation":
                                        "oracle complex64 OpenMP port of the reference gate "
                                        "semantics (the reference has no CPU path)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, dist: Dist):
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W

    hq.init(dist.local)
    rows, cols = args.grid
    n = rows * cols
    desc = W.grid_random(2, rows, cols, 20)
    gates = W.to_gates(desc)
    circ = hq.Circuit(n)
    circ.addGates(gates)
    t0 = time.perf_counter()
    circ.compile(backend=args.backend)
    compile_ms = (time.perf_counter() - t0) * 1000.0
    sched = circ.schedule()
    state = hq.State(n)

    # warm-up
    for _ in range(args.warmup):
        circ.run_on(state)

    # timed region: K circuits, device time per circuit from CUDA events on the
    # library stream; barrier + max over ranks
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    wall0 = time.perf_counter()
    dev_us = [circ.run_on(state) for _ in range(args.steps)]
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    dist.barrier()
    total_s = dist.max(sum(dev_us) * 1e-6)
    value = dist.ws * args.steps / total_s
    ms_per_step = total_s * 1000.0 / args.steps

    # roofline of the dominant kernel (OShareMem): per-group CUDA-event times
    prof = circ.profile(state)
    kinds = [b for (b, _, _, _) in sched]
    peak, peak_kind = measured_peaks()
    bytes_per_pass = 16.0 * (1 << n)
    oshm_t = [t for t, b in zip(prof, kinds) if b == hq.BACKEND_OSHM]
    mm_t = [t for t, b in zip(prof, kinds) if b == hq.BACKEND_TRANSMM]
    dom = oshm_t if oshm_t else mm_t
    achieved = bytes_per_pass / (np.mean(dom) * 1e-6) / 1e9 if dom else None
    traffic = None
    tfile = ROOT / "profiles" / "oshm_grid30_traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get("bytes_per_launch")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "kernel": "k_oshm<13,5>" if oshm_t else "transmm",
                "peak_source": peak_kind,
                "launches_per_circuit": len(dom)}

    # e2e through the public API with host buffers
    pinned = hq.PinnedBuffer(1 << n) if not args.no_e2e else None
    e2e_times = []
    h2d = 0
    for i in range(0 if args.no_e2e else args.steps):
        t0 = time.perf_counter()
        c2 = hq.Circuit(n)
        c2.addGates(gates)
        c2.compile(backend=args.backend)
        h2d = c2.program_bytes()
        state.init_zero()
        c2.run_on(state)
        state.store(pinned.array)
        e2e_times.append(time.perf_counter() - t0)
        del c2
    e2e = None
    if not args.no_e2e:
        e2e_s = dist.max(sum(e2e_times))
        e2e = {"value": dist.ws * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(8 * (1 << n))}
        pinned.free()

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        state.free()
        spg, k = cpu_sample(n, desc, args.cpu_budget, threads)
        if (rows, cols) != (5, 6):
            cpu = None
        cpu = {"value": 1.0 / (spg * len(desc)), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"first {k} of {len(desc)} gates at n=30 (complex64 OpenMP gate-by-gate "
                         f"port of the reference semantics), scaled to the full circuit"}

    groups_oshm = sum(1 for b in kinds if b == hq.BACKEND_OSHM)
    workload = WORKLOAD if (rows, cols) == (5, 6) else WORKLOAD.replace(
        "grid 5x6 (30 qubits)", f"grid {rows}x{cols} ({n} qubits)")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": workload, "backend": args.backend, "passes": len(sched),
                   "oshm_groups": groups_oshm, "transmm_groups": len(sched) - groups_oshm,
                   "reference_groups_tile10": 17, "compile_ms": compile_ms,
                   "l2": f"state ({8 << n >> 20} MiB) larger than L2; no flush",
                   "parallelism": f"replicas x{dist.ws}"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": len(sched) * args.steps,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--backend", default="oshm", choices=["oshm", "hybrid", "transmm"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU sampling")
    ap.add_argument("--grid", default="5x6", help="grid RxC of the circuit (5x6 = the 30-qubit "
                    "benchmark; smaller grids are for profiler captures)")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    args.grid = tuple(int(x) for x in args.grid.lower().split("x"))
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
