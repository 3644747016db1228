#!/usr/bin/env python3
"""Benchmarks on one GB300 (default: the 30-qubit random grid circuit).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload grid30|plain20|qft28|batch|serve|remap|dense28|blocked28]
                    [--backend oshm|hybrid|transmm] [--no-cpu-baseline]

grid30 (default, the headline): a step = one full circuit (845 gates:
sqrt(X)/sqrt(Y)/T per qubit and CZ on the cycle's coupler pattern) applied to a
complex64 state resident in HBM (2^30 amplitudes = 8 GiB, larger than L2, so no
flush is needed).  `value` is circuits per second over all ranks;
ms_per_step is device time per circuit.

  roofline      the OShareMem kernel: algorithmic bytes per launch (read + write
                of every amplitude = 16 * 2^30 B) over its mean launch time,
                measured with CUDA events on the library stream, against the
                measured HBM copy bandwidth (MEASURED_PEAKS.json).
  e2e           the same metric through the public API with host buffers: per
                step Circuit(30) + addGates + compile (program upload = H2D),
                |0..0> init, run, copy-back of the full state into pinned host
                memory (D2H) -- the reference's Circuit::run(copy_back=true).
                Two states alternate so that a circuit's readback (a copy
                kernel on 4 SMs) runs beside the next circuit; also recorded:
                the same steps one after another through Circuit.run_to_host,
                and a new circuit every step (its kernels compiling meanwhile).
  cpu_baseline  the oracle's complex64 OpenMP gate-by-gate port on this host's
                cores, on a bounded sample (the circuit's first gates), scaled
                to circuits/s.
  --impl reference   the same CPU port as the reference arm (the reference
                has no CPU implementation of the path, and it is a CMake
                C++/CUDA project that does not install as a package).

The other workloads print one line each with their own metric:
  plain20  20 qubits, 10 layers of U3 on every qubit + CNOT matching, plain
           gate-by-gate path (the state is 8 MiB and L2-resident).
  qft28    28-qubit QFT on a seeded random state: TransMM groups k = 6, 7, 8 in
           split-BF16 (3 products), TF32 and FP32 SIMT, with max |d amp| and
           1 - fidelity against the exact transform.
  batch    512 circuits (n 10..22, depth 8..40, RY/RZ + CZ) in one persistent
           launch, against each circuit run alone.
  serve    Poisson streams at 200, 1000 and 5000 circuits/s (n log-uniform
           12..32, depth 10..60) through the request loop; circuits/s and
           p50/p99 latency against one-at-a-time execution.
  remap    one in-place pass moving 8 physical bits of a 30-qubit state, and
           back; GB/s against the measured copy bandwidth.
  dense28  28 qubits, 10 layers of U3 + CNOT matching: OShareMem-only, hybrid,
           TransMM-only.
  blocked28  28 qubits in 7-qubit blocks of deep U3 + CNOT layers joined by
           single CNOTs, where the hybrid takes TransMM for every group.

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


def replica_throughput(dist: "Dist", units_per_rank: float, seconds: float):
    """Whole-job throughput of N independent replicas: every rank did
    `units_per_rank` units in `seconds`; the job takes the slowest rank's time.
    Returns (units per second over all ranks, that time)."""
    total_s = dist.max(seconds)
    return dist.ws * units_per_rank / total_s, total_s


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


_CPU_STATE: dict = {}


def cpu_sample(n: int, desc, budget_s: float, threads: int):
    """Time the oracle's complex64 gate-by-gate port on the first gates of the
    circuit; returns (seconds per gate, gates run).  The state buffer is made
    once per qubit count."""
    import oracle as O
    state = _CPU_STATE.get(n)
    if state is None:
        state = np.zeros(1 << n, dtype=np.complex64)
        state[0] = 1
        _CPU_STATE.clear()
        _CPU_STATE[n] = state
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


def workloads_module():
    """hyquas_gb300/workloads.py loaded by path: the generators are plain
    Python, and importing the package would load the native library, which
    the CPU arms do not use."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("hq_workloads_cpu",
                                                  ROOT / "hyquas_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference(args, dist: Dist):
    """Reference arm: the CPU gate-by-gate port on all host cores."""
    W = workloads_module()
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


def reference_gpu_leg(name: str, ref) -> dict:
    """The reference's own single-GPU run on this GPU, outside the timed region:
    its schedule and kernels (src/kernelOpt.cu run<128> for OShareMem groups,
    src/kernelSimple.cu for the plain path), traced from its host code and
    replayed (oracle/ref_replay.cu).  Its "Time Cost" (src/circuit.cpp:46-52),
    the device time of the same region, its launches, and its state against the
    FP64 oracle when `ref` is given."""
    import oracle as O
    if not O.ref_gpu_available(name):
        return {"unavailable": f"no trace or cubins for {name} (built where the reference "
                               "checkout is present: make -C oracle ref-if-present)"}
    try:
        r = O.ref_gpu_run(name, repeats=3, want_state=ref is not None)
    except Exception as e:  # reported, not fatal: it is a baseline
        return {"unavailable": str(e)}
    out = {"time_cost_ms": r["time_cost_ms_best"], "time_cost_ms_mean": r["time_cost_ms_mean"],
           "device_ms": r["device_ms_best"], "launches": r["launches"], "groups": r["groups"],
           "backend": r["backend"],
           "how": "reference host code traced against a recording CUDA runtime, its kernels "
                  "compiled from its sources for sm_103a, replayed on this GPU (best of 3)"}
    if ref is not None:
        out.update({"vs_oracle_" + k: v for k, v in O.compare(ref, r["state"]).items()})
    return out


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
    circ.compile(backend=args.backend, specialize=args.specialize, tile_qubits=args.tile_qubits,
                 coalesce=args.coalesce)
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
    value, total_s = replica_throughput(dist, args.steps, sum(dev_us) * 1e-6)
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
    if tfile.exists() and oshm_t and n == 30:  # the capture covers the OShareMem kernel at 30 qubits
        traffic = json.loads(tfile.read_text()).get("bytes_per_launch")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "kernel": "hq_oshm_group (generated per group)" if oshm_t else "k_transmm_tc",
                "peak_source": peak_kind,
                "launches_per_circuit": len(dom)}

    # e2e through the public API with host buffers: per step compile, run from
    # |0..0> and read the whole state back into pinned host memory, as the
    # reference's Circuit::run + result does (src/circuit.cpp:46-62).  Two
    # states alternate: step k's readback (State.store_async: a copy kernel on
    # a few SMs) runs beside step k+1's compile and run on the other SMs; the
    # region ends when the last readback has landed.
    e2e = None
    if not args.no_e2e:
        states = [state, hq.State(n)]
        pinned = [hq.PinnedBuffer(1 << n), hq.PinnedBuffer(1 << n)]
        # the host link's rate, and the first transfer into each buffer's fresh
        # pinned pages, out of the timed region
        tr = time.perf_counter()
        states[1].store(pinned[1].array)
        readback_gbs = 8.0 * (1 << n) / (time.perf_counter() - tr) / 1e9
        states[0].store(pinned[0].array)
        h2d = 0
        parts = []  # per step (ms): compile, readback age at reuse, init, enqueue
        issued = [None, None]
        live = []  # circuits whose runs may still be in flight
        t0 = time.perf_counter()
        for i in range(args.steps):
            st = states[i % 2]
            ta = time.perf_counter()
            # the host's planning overlaps the previous step's run; uploading the
            # program waits for that run (one stream)
            c2 = hq.Circuit(n)
            c2.addGates(gates)
            c2.compile(backend=args.backend, specialize=args.specialize,
                       tile_qubits=args.tile_qubits, coalesce=args.coalesce)
            h2d = c2.program_bytes()
            tb = time.perf_counter()
            age = 0.0
            if issued[i % 2] is not None:  # the state's previous readback has landed
                st.wait()
                age = (time.perf_counter() - issued[i % 2]) * 1e3
            tw = time.perf_counter()
            st.init_zero()
            td = time.perf_counter()
            c2.enqueue(st)  # the run, asynchronous
            st.store_async(pinned[i % 2].array)  # its readback, ordered after the run
            issued[i % 2] = time.perf_counter()
            live.append(c2)
            if len(live) > 2:
                live.pop(0)
            parts.append([round((tb - ta) * 1e3, 1), round(age, 1), round((td - tw) * 1e3, 1),
                          round((issued[i % 2] - td) * 1e3, 1)])
        hq.synchronize()  # the last run done, the device error word checked
        for s_ in states:
            s_.wait()
        live.clear()
        e2e_s = dist.max(time.perf_counter() - t0)
        # the same steps without overlap: run_to_host writes the final state to
        # HBM and to the pinned buffer in the last group's pass
        seq_steps = max(1, min(args.steps, 5))
        seq_ms = []
        f0 = time.perf_counter()
        for i in range(seq_steps):
            c2 = hq.Circuit(n)
            c2.addGates(gates)
            c2.compile(backend=args.backend, specialize=args.specialize,
                       tile_qubits=args.tile_qubits, coalesce=args.coalesce)
            state.init_zero()
            seq_ms.append(round(c2.run_to_host(state, pinned[0].array) / 1e3, 2))
            del c2
        seq_s = dist.max(time.perf_counter() - f0)
        # a new circuit every step (same shape, another seed): the compile
        # includes generating and compiling its group kernels
        fresh_steps = max(1, min(args.steps, 5))
        fresh_parts = []
        f0 = time.perf_counter()
        for i in range(fresh_steps):
            st = states[i % 2]
            ta = time.perf_counter()
            c2 = hq.Circuit(n)
            c2.addGates(W.to_gates(W.grid_random(1000 + 97 * i + dist.rank, rows, cols, 20)))
            # kernels not compiled before are compiled on a host thread; the
            # run uses the interpreter for groups whose kernel is not in yet
            c2.compile(backend=args.backend, specialize=3 if args.specialize == 2 else args.specialize,
                       tile_qubits=args.tile_qubits, coalesce=args.coalesce)
            tb = time.perf_counter()
            st.init_zero()
            c2.run_on(st)
            tc = time.perf_counter()
            st.store_async(pinned[i % 2].array)
            del c2
            fresh_parts.append([round((tb - ta) * 1e3, 1), round((tc - tb) * 1e3, 1)])
        for s_ in states:
            s_.wait()
        fresh_s = dist.max(time.perf_counter() - f0)
        e2e = {"value": dist.ws * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(8 * (1 << n)),
               "readback": "State.store_async: a copy kernel on 4 SMs writes the pinned buffer "
                           "while the next step runs on the other SMs; two states alternate; "
                           "runs are enqueued, so the next step's host planning overlaps the run",
               "readback_gbs": readback_gbs,
               "pinned_numa_nodes": [b.numa_nodes() for b in pinned],
               "step_parts_ms": {"compile_incl_wait_for_previous_run": [p[0] for p in parts],
                                 "readback_age_at_reuse": [p[1] for p in parts],
                                 "init": [p[2] for p in parts],
                                 "enqueue_run_and_readback": [p[3] for p in parts]},
               "sequential_run_to_host": {"value": dist.ws * seq_steps / seq_s, "unit": UNIT,
                                          "steps": seq_steps, "device_run_readback_ms": seq_ms},
               "fresh_circuit": {"value": dist.ws * fresh_steps / fresh_s, "unit": UNIT,
                                 "steps": fresh_steps,
                                 "compile_ms": [p[0] for p in fresh_parts],
                                 "init_run_ms": [p[1] for p in fresh_parts],
                                 "what": "a new seeded circuit of the same shape every step: "
                                         "planning inside the step; its group kernels compile "
                                         "on a host thread (specialize=3) while the run uses "
                                         "the interpreter for groups not compiled yet"}}
        states[1].free()
        for b in pinned:
            b.free()

    # accuracy against the FP64 gate-by-gate oracle (outside the timed region):
    # one fresh run from |0..0>, the whole state read back
    accuracy = None
    ref_gpu = None
    if not args.no_accuracy:
        import oracle as O
        state.init_zero()
        circ.run_on(state)
        got = np.empty(1 << n, dtype=np.complex64)
        state.store(got)
        ta = time.perf_counter()
        ref = O.run_f64(n, desc)
        oracle_s = time.perf_counter() - ta
        accuracy = O.compare(ref, got)
        accuracy.update({"against": "FP64 gate-by-gate oracle (reference gate matrices), "
                                    "whole state", "oracle_s": round(oracle_s, 1),
                         "oracle_threads": O.NTHREADS})
        del got
        if (rows, cols) == (5, 6) and not args.no_reference_gpu:
            ref_gpu = reference_gpu_leg("grid30_group", ref)
        del ref
    elif (rows, cols) == (5, 6) and not args.no_reference_gpu:
        ref_gpu = reference_gpu_leg("grid30_group", None)

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
        "config": {"workload": workload, "backend": args.backend, "specialize": args.specialize,
                   "tile_qubits": args.tile_qubits or 13, "coalesce": args.coalesce or 3,
                   "passes": len(sched),
                   "oshm_groups": groups_oshm, "transmm_groups": len(sched) - groups_oshm,
                   "reference_groups_tile10": len(hq.plan_groups(n, gates, reference_grouping=True)),
                   "compile_ms": compile_ms,
                   "group_ms": [round(t / 1000.0, 3) for t in prof],
                   "group_ms_predicted": [round(t / 1000.0, 3) for t in circ.predict()],
                   "l2": f"state ({8 << n >> 20} MiB) larger than L2; no flush",
                   "parallelism": f"replicas x{dist.ws}"},
        "accuracy": accuracy,
        "reference_gpu": ref_gpu,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": len(sched) * args.steps,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def base_line(args, dist, metric, value, unit, ms, hib, workload, extra_cfg=None):
    cfg = {"workload": workload, "parallelism": f"replicas x{dist.ws}"}
    cfg.update(extra_cfg or {})
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": dist.ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": hib, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic", "config": cfg}


def run_plain20(args, dist: Dist):
    """20 qubits, plain gate-by-gate path, |0..0>, full state out."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    import oracle as O
    hq.init(dist.local)
    n = 20
    desc = W.plain_u3_cnot(1, n, 10)
    gates = W.to_gates(desc)
    circ = hq.Circuit(n)
    circ.addGates(gates)
    circ.compile("plain")
    state = hq.State(n)
    circ.capture_graph(state)  # one kernel node per gate: replays without a host launch per gate
    flush = hq.State(28)  # 2 GiB written between steps: the state is L2-sized
    for _ in range(args.warmup):
        state.init_zero()
        circ.run_on(state)
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    dev = []
    for _ in range(args.steps):
        flush.init_zero()
        state.init_zero()
        dev.append(circ.run_on(state))
    clk = clocks.stop()
    dist.barrier()
    value, total_s = replica_throughput(dist, args.steps, sum(dev) * 1e-6)
    ref = O.run_f64(n, desc)
    got = state.store()
    err = O.compare(ref, got)
    ref_gpu = None if args.no_reference_gpu else reference_gpu_leg("plain20_serial", ref)
    peak, peak_kind = measured_peaks()
    per_gate_s = total_s / args.steps / len(desc)
    achieved = 16.0 * (1 << n) / per_gate_s / 1e9
    pinned = hq.PinnedBuffer(1 << n)
    e2e = []
    h2d = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        c2 = hq.Circuit(n)
        c2.addGates(gates)
        c2.compile("plain")
        state.init_zero()
        c2.run_on(state)
        state.store(pinned.array)
        e2e.append(time.perf_counter() - t0)
        h2d = sum(64 for _ in gates)  # gate records passed by value per launch
    pinned.free()
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        a = O.zero_state(n, np.complex64)
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < min(args.cpu_budget, 10.0) or reps == 0:
            O.apply_f32(n, a, desc, threads=threads)
            reps += 1
        cpu = {"value": reps / (time.perf_counter() - t0), "unit": "circuits/s", "cores": threads,
               "kind": "port", "sample": f"{reps} full circuits (complex64 OpenMP gate by gate)"}
    line = base_line(args, dist, "20q plain U3+CNOT circuit throughput (circuits/s)", value,
                     "circuits/s", total_s * 1000 / args.steps, True,
                     "plain path, 20 qubits, 10 layers of U3 on every qubit + CNOT on a random "
                     "matching (200 1q + 100 2q gates), |0..0>",
                     {"l2": "state 8 MiB is L2-resident; a 2 GiB buffer is written between steps",
                      "max_abs_err": err["max_abs_err"],
                      "one_minus_fidelity": err["one_minus_fidelity"]})
    line.update({
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel": "k_plain_gate",
                     "peak_source": peak_kind,
                     "note": "per-gate passes over an L2-resident 8 MiB state: frac above 1 "
                             "measures L2, not HBM"},
        "cpu_baseline": cpu,
        "reference_gpu": ref_gpu,
        "accuracy": err,
        "e2e": {"value": dist.ws * args.steps / dist.max(sum(e2e)), "unit": "circuits/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(8 << n)},
        "gpu_launches": (len(desc) + 1) * args.steps, "clocks": clk})
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_qft28(args, dist: Dist):
    """QFT-28 precision sweep on a seeded random state."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    hq.init(dist.local)
    n = args.qft_qubits
    desc = W.qft(n)
    gates = W.to_gates(desc)
    psi = W.random_state(3, n)
    N = 1 << n
    # exact transform: QFT|x> = sum_k e^{2 pi i x k / N} |k> / sqrt(N)
    ref = np.fft.ifft(psi.astype(np.complex128)) * np.sqrt(N)
    refn = np.vdot(ref, ref).real
    state = hq.State(n, zero=False)
    out = np.empty(N, dtype=np.complex64)
    sweep = []
    cases = [("oshm", 0, "fp32")]
    for k in (6, 7, 8):
        for prec in ("bf16x3", "tf32", "fp32"):
            cases.append(("transmm", k, prec))
    if args.qft_cases:  # e.g. "transmm:8:bf16x3,oshm:0:fp32"
        cases = [(b, int(k), p) for b, k, p in (x.split(":") for x in args.qft_cases.split(","))]
    best = None
    for backend, k, prec in cases:
        rec = {"backend": backend, "k": k, "precision": prec}
        try:
            c = hq.Circuit(n)
            c.addGates(gates)
            if backend == "oshm":
                c.compile("oshm")
            else:
                c.compile("transmm", mm_qubits=k, precision=prec)
            ts = []
            for i in range(max(args.warmup, 1) + args.steps):
                state.load(psi)
                t = c.run_on(state)
                if i >= max(args.warmup, 1):
                    ts.append(t)
            state.store(out)
            g = out.astype(np.complex128)
            ov = np.vdot(ref, g)
            rec.update({"ms": float(np.mean(ts)) / 1000.0, "passes": len(c.schedule()),
                        "max_abs_err": float(np.max(np.abs(g - ref))),
                        "one_minus_fidelity": float(1 - abs(ov) ** 2 / (refn * np.vdot(g, g).real))})
            # headline: split BF16 at the default tensor-core width (7 qubits)
            if best is None or (backend == "transmm" and prec == "bf16x3" and k == 7):
                best = rec
        except hq.HQError as e:
            rec["not_built"] = str(e)
        sweep.append(rec)
        if dist.rank == 0:
            print(json.dumps({"qft_case": rec}), file=sys.stderr, flush=True)
    value = best["ms"] if best else None
    peak, peak_kind = measured_peaks()
    achieved = (best["passes"] * 16.0 * N / (best["ms"] * 1e-3) / 1e9) if best else None
    title = (f"TransMM {best['precision']} k={best['k']}" if best and best["backend"] == "transmm"
             else "OShareMem")
    line = base_line(args, dist, f"{n}q QFT time (ms), {title}", value, "ms", value,
                     False, f"QFT-{n} (H + CU1 for all pairs + swaps folded into the layout) on an "
                     "iid complex Gaussian normalised state; reference = exact transform (FP64 FFT)",
                     {"sweep": sweep})
    line.update({"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak if achieved else None, "traffic": None,
                              "kernel": ("hq_oshm_group" if best and best["backend"] == "oshm" else
                                         "k_transmm_tcs" if best and best["k"] >= 7 else "k_transmm_tc")
                              + " (circuit average)", "peak_source": peak_kind},
                 "cpu_baseline": None, "e2e": None,
                 "gpu_launches": best["passes"] * args.steps if best else None})
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_batch(args, dist: Dist):
    """512 circuits in one persistent launch vs each alone."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    import oracle as O
    hq.init(dist.local)
    circuits = W.batched(4 + dist.rank, args.batch_count)
    arrays = [W.to_gates(d) for _, d in circuits]
    t0 = time.perf_counter()
    b = hq.Batch()
    states, circs = [], []
    for (n, _), g in zip(circuits, arrays):
        c = hq.Circuit(n)
        c.addGates(g)
        s = hq.State(n, zero=False)
        b.add(c, s)
        states.append(s)
        circs.append(c)
    b.compile()
    compile_s = time.perf_counter() - t0
    info = b.info()
    b.capture_graph(True)
    for _ in range(args.warmup):
        b.run()
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    dev = [b.run() for _ in range(args.steps)]
    clk = clocks.stop()
    dist.barrier()
    value, total_s = replica_throughput(dist, len(circuits) * args.steps, sum(dev) * 1e-6)
    # correctness: the smallest circuits against the FP64 oracle, all norms
    order = sorted(range(len(circuits)), key=lambda i: circuits[i][0])
    errs = [O.compare(O.run_f64(*circuits[i]), states[i].store())["max_abs_err"] for i in order[:8]]
    norm_dev = max(abs(s.norm() - 1.0) for s in states)
    # each circuit alone (same kernels: compiled schedule, one launch per group)
    for c in circs:
        c.compile("oshm", specialize=0)
    for c, s in zip(circs[:4], states[:4]):
        c.run_on(s)
    hq.synchronize()
    w0 = time.perf_counter()
    alone_dev = sum(c.run_on(s) for c, s in zip(circs, states))
    alone_wall = time.perf_counter() - w0
    peak, peak_kind = measured_peaks()
    achieved = info["pass_bytes"] / (total_s / args.steps) / 1e9
    # e2e: build, plan, run and read every state back to pinned host memory
    e2e = []
    d2h = sum(8 << n for n, _ in circuits)
    bufs = {n: hq.PinnedBuffer(1 << n) for n in set(n for n, _ in circuits)}
    for _ in range(args.steps):
        t0 = time.perf_counter()
        b2 = hq.Batch()
        for c, s in zip(circs, states):
            b2.add(c, s)
        b2.compile()
        b2.run()
        for (n, _), s in zip(circuits, states):
            s.store(bufs[n].array)
        e2e.append(time.perf_counter() - t0)
        b2.free()
    for x in bufs.values():
        x.free()
    gates_total = sum(len(d) for _, d in circuits)
    line = base_line(args, dist, f"batched circuits/s ({len(circuits)} circuits, n 10-22, depth 8-40)", value,
                     "circuits/s", total_s * 1000 / args.steps, True,
                     f"{len(circuits)} RY/RZ+CZ circuits, n uniform 10..22, depth uniform 8..40, one persistent "
                     "launch (CUDA graph), states start at |0..0>",
                     {"groups": info["groups"], "items": info["items"],
                      "pass_bytes": info["pass_bytes"], "gates": gates_total,
                      "tile_qubits_histogram": np.bincount(info["tile_qubits"]).tolist(),
                      "compile_s": compile_s,
                      "alone_device_ms": alone_dev / 1000.0, "alone_wall_ms": alone_wall * 1000.0,
                      "speedup_vs_alone_wall": alone_wall / (total_s / args.steps),
                      "max_abs_err_smallest8": max(errs), "max_norm_dev": norm_dev,
                      "l2": "2.4 GB of states, larger than L2"})
    line.update({"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak, "traffic": None,
                              "kernel": "k_oshm_batch<13,5>", "peak_source": peak_kind},
                 "cpu_baseline": None,
                 "e2e": {"value": dist.ws * len(circuits) * args.steps / dist.max(sum(e2e)),
                         "unit": "circuits/s", "h2d_bytes_per_step": None,
                         "d2h_bytes_per_step": int(d2h)},
                 "gpu_launches": args.steps, "clocks": clk})
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_dense28(args, dist: Dist):
    """Dense circuits at 28 qubits, OShareMem-only, TransMM-only and the hybrid
    choice, each against the FP64 oracle.  dense28: the 20-qubit plain-path
    family (U3 on every qubit, then CNOT on a random matching, per layer);
    blocked28: deep U3+CNOT blocks of 7 qubits joined by single CNOTs, where
    a block's layers fuse into one 7-qubit unitary (the reference's mix mode,
    src/compiler.cpp:248-280)."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    import oracle as O
    hq.init(dist.local)
    n = args.dense_qubits
    blocked = args.workload == "blocked28"
    if blocked:
        desc = W.blocked_u3_cnot(11, n, 7, args.dense_layers, 2)
        what = (f"{n} qubits in blocks of 7, 2 rounds of {args.dense_layers} layers per block (U3 on "
                "every qubit + CNOTs on alternating neighbour pairs inside the block, then one CNOT "
                "joining neighbouring blocks), |0..0>")
    else:
        desc = W.plain_u3_cnot(1, n, args.dense_layers)
        what = (f"{n} qubits, {args.dense_layers} layers of U3 on every qubit + CNOT on a random "
                "matching, |0..0>")
    gates = W.to_gates(desc)
    ref = O.run_f64(n, desc)
    state = hq.State(n)
    got = np.empty(1 << n, dtype=np.complex64)
    rows = []
    for backend in ("oshm", "hybrid", "transmm"):
        c = hq.Circuit(n)
        c.addGates(gates)
        c.compile(backend)
        kinds = [b for (b, _, _, _) in c.schedule()]
        for _ in range(max(args.warmup, 1)):
            state.init_zero()
            c.run_on(state)
        ts = []
        for _ in range(args.steps):
            state.init_zero()
            ts.append(c.run_on(state))
        state.init_zero()
        c.run_on(state)
        state.store(got)
        acc = O.compare(ref, got)
        rows.append({"backend": backend, "ms": float(np.median(ts)) / 1000.0,
                     "passes": len(kinds), "transmm_groups": sum(1 for b in kinds if b == hq.BACKEND_TRANSMM),
                     "predicted_ms": float(np.sum(c.predict())) / 1000.0, **acc})
        if dist.rank == 0:
            print(json.dumps({"dense_case": rows[-1]}), file=sys.stderr, flush=True)
    best = min(rows, key=lambda r: r["ms"])
    peak, peak_kind = measured_peaks()
    achieved = best["passes"] * 16.0 * (1 << n) / (best["ms"] * 1e-3) / 1e9
    line = base_line(args, dist, f"{n}q {'blocked ' if blocked else ''}U3+CNOT circuit time (ms), "
                     "best backend", best["ms"], "ms", best["ms"], False,
                     what + "; OShareMem-only, hybrid and TransMM-only (split BF16, 7-qubit groups), "
                     "each checked against the FP64 oracle",
                     {"cases": rows, "best_backend": best["backend"]})
    line.update({"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak, "traffic": None,
                              "kernel": "circuit average over its passes", "peak_source": peak_kind},
                 "cpu_baseline": None, "e2e": None, "gpu_launches": best["passes"] * args.steps})
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_remap(args, dist: Dist):
    """In-HBM qubit remap (the single-GPU form of the reference's global-qubit
    exchange, src/executor.cpp:59-179): a step moves 8 physical bits of a
    resident state in one in-place pass and the next step moves them back."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    hq.init(dist.local)
    n = args.remap_qubits
    s = hq.State(n, zero=False)
    psi = W.random_state(21, n)
    s.load(psi)
    ident = list(range(n))
    moved = [3, 7, 12, 17, n - 6, n - 4, n - 2, n - 1]  # a cycle over 8 bits
    fwd = ident.copy()
    for a, b in zip(moved, moved[1:] + moved[:1]):
        fwd[a] = b
    layouts = [fwd, ident]
    for i in range(args.warmup):
        s.remap(layouts[i % 2])
    if args.warmup % 2:
        s.remap(ident)
    hq.synchronize()
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    t0 = time.perf_counter()
    for i in range(args.steps):
        s.remap(layouts[i % 2])
    hq.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    dist.barrier()
    value, total_s = replica_throughput(dist, args.steps, dt)
    if args.steps % 2:
        s.remap(ident)
    idx = np.array(W.SplitMix64(3).shuffle(range(1 << 16))[:2048], dtype=np.uint64) << np.uint64(n - 16)
    exact = bool(np.array_equal(s.amps(idx), psi[idx.astype(np.int64)]))
    # a whole reversal (every bit moves): passes of up to 13 tile bits
    rev = ident[::-1]
    t1 = time.perf_counter()
    s.remap(rev)
    hq.synchronize()
    rev_ms = (time.perf_counter() - t1) * 1e3
    s.remap(ident)
    peak, peak_kind = measured_peaks()
    per_step = total_s / args.steps
    achieved = 16.0 * (1 << n) / per_step / 1e9
    line = base_line(args, dist, f"{n}q in-HBM remap of 8 qubits (remaps/s)", value, "remaps/s",
                     per_step * 1e3, True,
                     f"{n}-qubit complex64 state (8 << {n} bytes, larger than L2): 8 physical bits "
                     "moved by one in-place pass, then moved back",
                     {"amplitudes_exact_after_round_trips": exact,
                      "full_reversal_ms": rev_ms,
                      "l2": "state larger than L2; no flush"})
    line.update({"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak, "traffic": None,
                              "kernel": "k_permute_bits (timed with host clock around "
                                        "synchronised steps)", "peak_source": peak_kind},
                 "cpu_baseline": None, "e2e": None, "gpu_launches": args.steps, "clocks": clk})
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def serve_once(hq, stream, arrays):
    """Run `stream` (arrival s, n, gates) through a fresh request loop in real
    time: submit each request at its arrival, read its result (one amplitude
    and 16 samples) and release it on completion.  Returns circuits/s over the
    span from first submission to last completion, p50/p99 latency (ms) and
    the loop's statistics."""
    sv = hq.Server()
    w = sv.submit(12, [])
    sv.wait(w, 60)
    sv.release(w)
    sv.poll()
    count = len(stream)
    t0 = time.perf_counter()
    times = {}
    i = 0
    while len(times) < count:
        now = time.perf_counter() - t0
        while i < count and stream[i][0] <= now:
            sv.submit(stream[i][1], arrays[i])
            i += 1
        for rid in sv.poll():
            if sv.wait(rid, 0) == "done":
                st = sv.state(rid)
                st.amps([0])
                st.sample(16, seed=rid)
            times[rid] = sv.times(rid)
            sv.release(rid)
        time.sleep(0.0002)
    lat = np.array([d - s for (s, a, d) in times.values()]) / 1e3
    first = min(s for s, a, d in times.values())
    last = max(d for s, a, d in times.values())
    out = {"circuits_per_s": count / ((last - first) * 1e-6),
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "steps": sv.stats()["steps"], "peak_resident_gb": sv.stats()["peak_resident_bytes"] / 1e9}
    sv.close()
    return out


def fifo(stream, service):
    """One server, first come first served: each request starts at the later
    of its arrival and the previous request's end and takes its measured
    service time.  Circuits/s over the span and p50/p99 latency (ms)."""
    fin, lat = 0.0, []
    for (t, _, _), sv_t in zip(stream, service):
        fin = max(fin, t) + sv_t
        lat.append(fin - t)
    span = fin - stream[0][0]
    return {"circuits_per_s": len(stream) / span, "p50_ms": float(np.percentile(lat, 50)) * 1e3,
            "p99_ms": float(np.percentile(lat, 99)) * 1e3}


def run_serve(args, dist: Dist):
    """Poisson streams of circuits through the request loop, against the
    reference's plain gate-by-gate path run one request at a time."""
    import hyquas_gb300 as hq
    from hyquas_gb300 import workloads as W
    hq.init(dist.local)
    count, nmax = args.serve_count, args.serve_nmax
    rates = [200.0, 1000.0, 5000.0]
    results, subset = {}, {}
    base = W.served_stream(5 + dist.rank, count, 1000.0, 12, nmax)
    arrays = [hq.gate_array(W.to_gates(d)) for _, _, d in base]
    m = min(args.serve_plain_count, count)
    for rate in rates:
        stream = W.served_stream(5 + dist.rank, count, rate, 12, nmax)
        results[rate] = serve_once(hq, stream, arrays)
        subset[rate] = serve_once(hq, stream[:m], arrays[:m])
        if dist.rank == 0:
            print(json.dumps({"serve_rate": rate, **results[rate], "subset": subset[rate]}),
                  file=sys.stderr, flush=True)
    # the plain path (src/kernelSimple.cu:335-446), measured: each of the first
    # m requests alone -- state, one launch per gate, result read -- in turn
    plain_service = []
    for (t, n, _), arr in zip(base[:m], arrays[:m]):
        a = time.perf_counter()
        s = hq.State(n)
        s.apply_gates(arr)
        s.amps([0])
        s.sample(16, seed=7)
        plain_service.append(time.perf_counter() - a)
        s.free()
    # compiled one request at a time (same kernels as the loop, no batching)
    comp_service = []
    for (t, n, _), arr in zip(base[:m], arrays[:m]):
        a = time.perf_counter()
        c = hq.Circuit(n)
        c.addGates(arr)
        c.compile("oshm", specialize=0)
        s = hq.State(n)
        c.run_on(s)
        s.amps([0])
        s.sample(16, seed=7)
        comp_service.append(time.perf_counter() - a)
        s.free()
    plain_r, comp_r = {}, {}
    for rate in rates:
        stream = W.served_stream(5 + dist.rank, count, rate, 12, nmax)[:m]
        plain_r[rate] = fifo(stream, plain_service)
        comp_r[rate] = fifo(stream, comp_service)
    head = results[1000.0]
    line = base_line(args, dist, "served circuits/s at 1000/s arrivals (p50/p99 in config)",
                     head["circuits_per_s"], "circuits/s", None, True,
                     f"{count} Poisson requests per rate, n log-uniform 12..{nmax}, depth 10..60 "
                     "RY/RZ+CZ; admission by 2^n x 8 B against 150 GB; results read (amplitude + "
                     "16 samples) and released on completion",
                     {"rates": {str(int(r)): results[r] for r in rates},
                      "subset_requests": m,
                      "subset_rates": {str(int(r)): subset[r] for r in rates},
                      "plain_one_at_a_time_measured": {str(int(r)): plain_r[r] for r in rates},
                      "compiled_one_at_a_time_measured": {str(int(r)): comp_r[r] for r in rates},
                      "plain_service_s_total": sum(plain_service),
                      "comparison": f"the first {m} requests of each stream: the request loop "
                                    "(measured, real time) against each request run alone in "
                                    "arrival order (measured service times, FIFO queue)",
                      "speedup_vs_plain": {str(int(r)): subset[r]["circuits_per_s"] /
                                           plain_r[r]["circuits_per_s"] for r in rates},
                      "speedup_vs_compiled": {str(int(r)): subset[r]["circuits_per_s"] /
                                              comp_r[r]["circuits_per_s"] for r in rates}})
    line.update({"roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None})
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
    ap.add_argument("--tile-qubits", type=int, default=0,
                    help="OShareMem tile width (0: the library default, 13)")
    ap.add_argument("--coalesce", type=int, default=0,
                    help="low physical qubits kept in every tile (0: the library default)")
    ap.add_argument("--specialize", type=int, default=2, choices=[0, 1, 2, 3],
                    help="OShareMem kernels: 0 interpreter, 1 generated, 2 generated where "
                         "possible (grid30)")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the replay of the reference's own GPU run")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 oracle comparison (grid30: about a minute of CPU)")
    ap.add_argument("--workload", default="grid30",
                    choices=["grid30", "plain20", "qft28", "batch", "serve", "remap", "dense28",
                             "blocked28"])
    ap.add_argument("--dense-qubits", type=int, default=28)
    ap.add_argument("--dense-layers", type=int, default=10)
    ap.add_argument("--remap-qubits", type=int, default=30)
    ap.add_argument("--qft-qubits", type=int, default=28)
    ap.add_argument("--qft-cases", default="",
                    help="backend:k:precision list for --workload qft28 (default: the full sweep)")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--serve-count", type=int, default=200)
    ap.add_argument("--serve-nmax", type=int, default=32)
    ap.add_argument("--serve-plain-count", type=int, default=50,
                    help="requests of each stream also run one at a time on the plain path")
    args = ap.parse_args()
    args.grid = tuple(int(x) for x in args.grid.lower().split("x"))
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "grid30":
            run_ours(args, dist)
        else:
            {"plain20": run_plain20, "qft28": run_qft28, "batch": run_batch,
             "serve": run_serve, "remap": run_remap, "dense28": run_dense28,
             "blocked28": run_dense28}[args.workload](args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
