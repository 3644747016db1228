/* hyquas_gb300 -- GB300-native single-GPU state-vector simulator, C ABI.
 *
 * This is the drop-in boundary for the single-GPU path of thu-pacman/HyQuas.
 * Every entry point names the reference interface it replaces (path:line in
 * the reference tree).  The header-only C++ facade in hyquas_gb300/circuit.hpp
 * re-creates the reference's Circuit/Gate API (src/circuit.h:20-46,
 * src/gate.h:11-66) on top of these functions; ctypes bindings in
 * hyquas_gb300/__init__.py do the same for Python.
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, int32/int64/uint64, float, double.
 *   - Every function returns an hq_status (0 = success).  hq_last_error()
 *     returns a thread-local message for the last failure.  The reference
 *     exits the process on any error (src/utils.h:106-144); here errors are
 *     returned and the library stays usable.
 *   - State vectors are complex64, interleaved (re, im), 2^n amplitudes, the
 *     reference's qComplex layout for the FP32 build (src/utils.h:24-31).
 *     Amplitude index bit q is qubit q.
 *   - After a compiled run the amplitudes may sit in a permuted qubit layout
 *     (the reference keeps its final State, src/circuit.cpp:95-113).  All
 *     readout functions take LOGICAL indices and apply the layout.
 *   - Objects are not thread-safe; use one object per host thread.
 */
#ifndef HYQUAS_GB300_H
#define HYQUAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t hq_status;
#define HQ_OK 0
#define HQ_ERR_INVALID (-1)     /* bad argument: qubit index, size, null pointer */
#define HQ_ERR_CUDA (-2)        /* a CUDA runtime/driver call failed */
#define HQ_ERR_NOMEM (-3)       /* device allocation failed or over the HBM budget */
#define HQ_ERR_STATE (-4)       /* object in the wrong state (e.g. run before compile) */
#define HQ_ERR_TIMEOUT (-5)     /* a bounded device-side wait expired (error flag set) */
#define HQ_ERR_UNSUPPORTED (-6) /* feature not available on this device/configuration */
#define HQ_ERR_BUSY (-7)        /* serving queue full / slot not ready */

/* Gate type ordinals follow the reference GateType (src/gate.h:7-9). */
enum hq_gate_type {
    HQ_CCX = 0, HQ_CNOT = 1, HQ_CY = 2, HQ_CZ = 3, HQ_CRX = 4, HQ_CRY = 5, HQ_CU1 = 6,
    HQ_CRZ = 7, HQ_U1 = 8, HQ_U2 = 9, HQ_U3 = 10, HQ_H = 11, HQ_X = 12, HQ_Y = 13,
    HQ_Z = 14, HQ_S = 15, HQ_SDG = 16, HQ_T = 17, HQ_TDG = 18, HQ_RX = 19, HQ_RY = 20,
    HQ_RZ = 21, HQ_ID = 23,
    /* Extension (no reference counterpart): exchange of qubits `target` and
     * `control`.  The compiler folds it into the qubit layout (no data pass). */
    HQ_SWAP = 28
};

/* One gate: the fields of the reference Gate (src/gate.h:11-20) without the
 * name/id.  mat = row-major 2x2 complex in double: re00 im00 re01 im01 re10
 * im10 re11 im11.  control/control2 = -1 when absent. */
typedef struct hq_gate {
    int32_t type;
    int32_t target;
    int32_t control;
    int32_t control2;
    double mat[8];
} hq_gate;

typedef struct hq_state_s* hq_state;
typedef struct hq_circuit_s* hq_circuit;

/* ---- context ---------------------------------------------------------- */

/* Select the device and create the library's stream.  Replaces
 * MyGlobalVars::init (src/utils.cpp:17-60) for one GPU; idempotent. */
hq_status hq_init(int device);
/* Thread-local message for the last failing call ("" when none). */
const char* hq_last_error(void);
/* Library version string. */
const char* hq_version(void);
/* Device facts: SM count, HBM bytes, max shared memory per block. */
hq_status hq_device_info(int32_t* sm_count, uint64_t* hbm_bytes, int32_t* smem_per_block);
/* Set the HBM budget (bytes) that state allocation is admitted against;
 * 0 = no budget.  No reference counterpart (the reference has no admission). */
hq_status hq_set_hbm_budget(uint64_t bytes);
/* Device bytes the library holds (states, programs, scratch). */
hq_status hq_hbm_in_use(uint64_t* bytes);

/* Page-locked host buffers for fast state transfers: from 64 MiB up an
 * anonymous mapping with transparent huge pages requested, page-locked and
 * device-mapped with cudaHostRegister, every page then written once through
 * the mapping (so the first readback into it runs at full rate; contents are
 * zero-filled words per 4 KB, otherwise undefined); smaller ones (or where
 * that fails) from cudaHostAlloc. */
hq_status hq_host_alloc(uint64_t bytes, void** out);
/* Frees a buffer from hq_host_alloc. */
hq_status hq_host_free(void* p);

/* ---- gates (src/gate.cpp:9-342, the Gate::* factories) ---------------- */

/* Fill `out` with the gate of `type` on the given qubits; params = the
 * factory's angle arguments in order (theta/phi/lambda/angle), may be NULL
 * for gates without angles.  Argument order of the reference factories is
 * control-then-target; here qubits are passed by role. */
hq_status hq_gate_make(int32_t type, int32_t target, int32_t control, int32_t control2,
                       const double* params, hq_gate* out);

/* Parse OpenQASM 2 text: the subset the reference's parser reads
 * (parse_circuit, main.cpp:12-230: qreg; cx ccx cy cz h x y z s sdg t tdg;
 * crx cry crz cu1 u1 u3 rx ry rz with pi*x / pi/x / decimal parameters),
 * plus u2, id, swap, -pi*x / -pi/x, and skipped creg / barrier / measure.
 * *num_qubits = the qreg size; the gates go to out[0..cap) and *count is
 * their number (out may be NULL to ask for the count).  Errors name the line. */
hq_status hq_qasm_parse(const char* text, int32_t* num_qubits, hq_gate* out, int32_t cap,
                        int32_t* count);

/* ---- state vector (src/kernelSimple.cu:9-37, 518-529) ------------------ */

/* Allocate a 2^n complex64 state (no initialisation).  kernelInit's cudaMalloc,
 * src/kernelSimple.cu:9-37. */
hq_status hq_state_create(int32_t num_qubits, hq_state* out);
/* kernelDestroy, src/kernelSimple.cu:527-529. */
hq_status hq_state_destroy(hq_state s);
/* |0..0>: kernelInit's memset + amp[0]=1, src/kernelSimple.cu:14-31. */
hq_status hq_state_init_zero(hq_state s);
/* Upload 2^n interleaved complex64 amplitudes in logical order; resets the
 * layout to identity.  No reference counterpart (random initial states). */
hq_status hq_state_load(hq_state s, const float* host_amps);
/* Download all 2^n amplitudes in LOGICAL order (undoing the layout on the
 * device first).  kernelDeviceToHost + Circuit::ampAt, src/kernelSimple.cu:523-525,
 * src/circuit.cpp:54-64, 115-118. */
hq_status hq_state_store(hq_state s, float* host_amps);
/* The same copy without waiting: it runs on the library's copy stream after
 * the work already queued on s, so a circuit on another state overlaps it.
 * host_amps must stay valid (and should be pinned, hq_host_alloc) until
 * hq_state_wait(s); later work that writes s waits for the copy on the device.
 * Into pinned memory of 64 MiB or more the copy is a kernel on 4 SMs, and the
 * library's group kernels launch on the other SMs while it is in flight;
 * otherwise copy-engine transfers.  hq_state_store's asynchronous form, for
 * pipelined readback. */
hq_status hq_state_store_async(hq_state s, float* host_amps);
/* Block until s's pending asynchronous copy has landed in host memory. */
hq_status hq_state_wait(hq_state s);
/* Download the amplitudes at `count` logical indices.  Circuit::ampAtGPU /
 * kernelGetAmp, src/circuit.cpp:120-142, src/kernelSimple.cu:518-522. */
hq_status hq_state_amps(hq_state s, const uint64_t* logical_idx, int64_t count, float* out);
/* Current logical->physical qubit map (State::pos, src/schedule.h:15-34). */
hq_status hq_state_layout(hq_state s, int32_t* pos);
/* Circuit::numQubits for a state (src/circuit.h:20-46). */
hq_status hq_state_num_qubits(hq_state s, int32_t* n);
/* Device pointer of the amplitudes (physical order); for zero-copy users. */
hq_status hq_state_device_ptr(hq_state s, void** dev_ptr);

/* P(qubit q = 0) with an FP64 reduction: kernelMeasure, src/kernelSimple.cu:497-516. */
hq_status hq_state_prob_zero(hq_state s, int32_t logical_qubit, double* p0);
/* sum |a|^2 (FP64 reduction). */
hq_status hq_state_norm(hq_state s, double* norm);
/* P(qubit q = 1) for every logical qubit, one FP64 pass. */
hq_status hq_state_marginals(hq_state s, double* p1);
/* Draw `shots` outcomes from |amp|^2: out[i] = logical basis index.  The
 * draws are the SplitMix64 stream of `seed` (u = output >> 11 scaled to
 * [0, 1)), inverted through an FP64 cumulative distribution in logical
 * index order (the state is brought to the identity layout first).  No reference
 * counterpart (it measures one qubit, src/kernelSimple.cu:497-516). */
hq_status hq_state_sample(hq_state s, int32_t shots, uint64_t seed, uint64_t* out);
/* Allocation-free form of hq_state_marginals, for callers that cannot call
 * cudaMalloc: code whose device memory belongs to another allocator (a
 * framework's caching pool, or an HBM budget already handed out in full) and
 * latency-critical paths that must not take cudaMalloc's implicit device
 * synchronisation.  No counterpart in the reference.
 *   d_state  caller's device array of 2^num_qubits complex64 amplitudes
 *            (16-byte aligned), read in physical order;
 *   d_out    caller's device array of num_qubits + 1 doubles, receives
 *            [sum |a|^2, P(bit 0 = 1), ..., P(bit n-1 = 1)] (FP64);
 *   stream   cudaStream_t to run on (NULL = default stream); nothing is
 *            synchronised.
 * Scratch is a static 1.6 MiB device array in the library (held by every GPU
 * that loads it until exit), so num_qubits is limited to 26; larger sizes
 * return HQ_ERR_INVALID.  The first call on a device looks up the array's
 * address with that device current: make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race.
 * d_state, d_out and stream must belong to the current device and its
 * primary context (the one the CUDA runtime uses); a state on another device
 * returns HQ_ERR_INVALID. */
hq_status hq_marginals_noalloc(const void* d_state, int32_t num_qubits, double* d_out,
                               void* stream);
/* ---- plain path (BACKEND=serial): one launch per gate ------------------- */

/* Apply gates one kernel launch each, in order: kernelExecSimple,
 * src/kernelSimple.cu:335-446.  Logical qubits, current layout honoured. */
hq_status hq_apply_gates(hq_state s, const hq_gate* gates, int32_t num_gates);

/* ---- circuits: compile + run (src/circuit.cpp:16-71, 156-210) ------------ */

/* Backends, after the reference's -DBACKEND (CMakeLists.txt:18-35). */
enum hq_backend {
    HQ_BACKEND_PLAIN = 0,   /* serial: one launch per gate */
    HQ_BACKEND_OSHM = 1,    /* group: OShareMem gate groups only */
    HQ_BACKEND_TRANSMM = 3, /* blas: TransMM groups only */
    HQ_BACKEND_HYBRID = 4   /* mix: per-group cost-model choice */
};
/* TransMM arithmetic. */
enum hq_mm_precision {
    HQ_MM_BF16X3 = 0, /* split hi+lo BF16, 3 products, FP32 accumulate (tcgen05) */
    HQ_MM_TF32 = 1,   /* one TF32 product (tcgen05) */
    HQ_MM_FP32 = 2    /* FP32 SIMT */
};

typedef struct hq_compile_options {
    int32_t backend;       /* hq_backend */
    int32_t tile_qubits;   /* OShareMem tile width k (0 = autotuned) */
    int32_t coalesce;      /* low physical qubits always in a tile (0 = default) */
    int32_t mm_qubits;     /* TransMM group width, 4..8 (0 = 7 on the tensor cores, 6 for
                              FP32 SIMT) */
    int32_t mm_precision;  /* hq_mm_precision */
    int32_t reference_grouping; /* 1 = use the reference's widths (tile 10, coalesce 3, MAT 6) */
    int32_t specialize;    /* OShareMem kernels: 0 = interpreter (runs of single-qubit gates
                              on a qubit are fused into one gate first), 1 = one generated
                              kernel per group (NVRTC, error if unavailable), 2 = generated
                              when NVRTC is present, else interpreter (default), 3 = as 2
                              but kernels not compiled before are compiled on a host thread
                              after compile returns; runs use the interpreter for the
                              groups until their kernels are in (a new circuit's first run
                              does not wait for NVRTC) */
} hq_compile_options;

/* OShareMem backend, autotuned widths, split BF16, generated kernels when
 * available (the reference's default build: -DBACKEND=group). */
hq_status hq_compile_options_default(hq_compile_options* opt);

/* Circuit(int numQubits), src/circuit.h:20-46; destroy frees its device program. */
hq_status hq_circuit_create(int32_t num_qubits, hq_circuit* out);
hq_status hq_circuit_destroy(hq_circuit c);
/* Circuit::addGate, src/circuit.h:28-30. */
hq_status hq_circuit_add_gates(hq_circuit c, const hq_gate* gates, int32_t num_gates);
/* Gates added so far (the reference's Circuit::gates.size()). */
hq_status hq_circuit_num_gates(hq_circuit c, int32_t* num_gates);
/* Circuit::compile, src/circuit.cpp:177-210 (Compiler::run, src/compiler.cpp:70-165). */
hq_status hq_circuit_compile(hq_circuit c, const hq_compile_options* opt);
/* Number of gate groups and, per group: backend (HQ_BACKEND_OSHM /
 * HQ_BACKEND_TRANSMM), gate count, tile/group width and related-qubit mask.
 * Arrays may be NULL; they must hold num_groups entries otherwise. */
hq_status hq_circuit_schedule(hq_circuit c, int32_t* num_groups, int32_t* backend,
                              int32_t* gates_per_group, int32_t* width, uint64_t* related);
/* Gate indices (into the added list) of group g, in execution order (a
 * fused run of single-qubit gates is listed by its first gate). */
hq_status hq_circuit_group_gates(hq_circuit c, int32_t g, int32_t* gate_idx, int32_t cap,
                                 int32_t* count);
/* Host-only planning (no device needed): partition `num_gates` gates as
 * hq_circuit_compile would and report, per group, its backend, gate count,
 * width, related-qubit mask and (OShareMem) number of register phases;
 * gate_order receives the gate indices group after group (num_gates
 * entries).  Arrays need room for num_gates groups.  The CPU half of
 * Circuit::compile (src/circuit.cpp:156-175, Compiler::run
 * src/compiler.cpp:70-165). */
hq_status hq_plan_groups(int32_t num_qubits, const hq_gate* gates, int32_t num_gates,
                         const hq_compile_options* opt, int32_t* num_groups, int32_t* backend,
                         int32_t* gates_per_group, int32_t* width, uint64_t* related,
                         int32_t* phases, int32_t* gate_order);
/* ---- compiled-schedule bytes (the reference serialises its Schedule for
 * broadcast: Schedule/GateGroup/State::serialize, src/schedule.cpp:156-325;
 * Gate::serialize, src/gate.cpp:558-589) ----------------------------------
 * The bytes hold the compile options, the gates, the SWAP-folded gates and
 * the partition, with a checksum.  *len receives the size; buf = NULL asks for
 * the size only, otherwise cap must be at least *len. */
hq_status hq_circuit_serialize(hq_circuit c, void* buf, uint64_t cap, uint64_t* len);
/* Host only: plan num_gates gates as hq_circuit_compile would and write the
 * schedule bytes (no device needed). */
hq_status hq_plan_serialize(int32_t num_qubits, const hq_gate* gates, int32_t num_gates,
                            const hq_compile_options* opt, void* buf, uint64_t cap, uint64_t* len);
/* Host only: check schedule bytes (magic, version, checksum, every size and
 * index) and report the register size, gate count and, per group, backend,
 * gate count, width and related-qubit mask (arrays may be NULL, else they need
 * num_groups entries; size them with a first call that passes NULL). */
hq_status hq_schedule_inspect(const void* buf, uint64_t len, int32_t* num_qubits, int32_t* num_gates,
                              int32_t* num_groups, int32_t* backend, int32_t* gates_per_group,
                              int32_t* width, uint64_t* related);
/* A compiled circuit from schedule bytes: the partitioner does not run; the
 * groups are lowered and uploaded as compile would.  Invalid bytes give
 * HQ_ERR_INVALID (HQ_ERR_UNSUPPORTED for another format version). */
hq_status hq_circuit_deserialize(const void* buf, uint64_t len, hq_circuit* out);
/* Bytes of device-resident program (gate-group lowering, fused unitaries)
 * that compile uploaded for this circuit. */
hq_status hq_circuit_program_bytes(hq_circuit c, uint64_t* bytes);
/* Run the compiled schedule on state s (stream-ordered, then synchronised).
 * Circuit::run, src/circuit.cpp:16-71; elapsed_us = device time of the run
 * (the reference's "Time Cost"). */
hq_status hq_circuit_run(hq_circuit c, hq_state s, double* elapsed_us);
/* Run the compiled schedule on s and leave the final state in logical order
 * at host_amps (2 * 2^n floats, interleaved re/im): the reference's run
 * followed by its full-state readback into Circuit::result
 * (src/circuit.cpp:46-62, kernelDeviceToHost).  With a pinned buffer
 * (hq_host_alloc) and a schedule whose last group runs a generated kernel
 * and ends in the canonical layout, that group writes each finished amplitude
 * to HBM and to host_amps in the same pass; otherwise the run is followed by
 * a copy.  s holds the final state afterwards either way.  elapsed_us =
 * device time of run and readback. */
hq_status hq_circuit_run_to_host(hq_circuit c, hq_state s, float* host_amps, double* elapsed_us);
/* Run the compiled schedule on s with a CUDA event pair around every group;
 * group_us[g] = device time of group g (num_groups entries).  The reference's
 * MEASURE_STAGE per-group timing, src/executor.cpp:406-458. */
hq_status hq_circuit_profile(hq_circuit c, hq_state s, double* group_us);
/* The cost model's device time (us) of each group of a compiled circuit, the
 * figure the hybrid partitioner compares (hq_cost_params): the counterpart of
 * the reference's Evaluator::perfPerGate / perfBLAS (src/evaluator.cpp:111-229),
 * to set beside hq_circuit_profile. */
hq_status hq_circuit_predict(hq_circuit c, double* group_us);
/* Enqueue the compiled schedule on the library stream without synchronising. */
hq_status hq_circuit_enqueue(hq_circuit c, hq_state s);
/* Capture the compiled schedule for state s into a CUDA graph (replayed by
 * later hq_circuit_run / hq_circuit_enqueue calls on the same state).  Plain-
 * path circuits are captured too: one kernel node per gate, no host launch per
 * gate on replay. */
hq_status hq_circuit_capture_graph(hq_circuit c, hq_state s);
/* Wait for all work queued on the library stream (cudaDeviceSynchronize in the
 * reference's timed region, src/circuit.cpp:16-71). */
hq_status hq_synchronize(void);

/* ---- cost model and autotuner (replace the reference's V100/A100 parameter
 * files and their calibrator: src/evaluator.h:18-127, src/evaluator.cpp:111-229,
 * evaluator-preprocess/process.cpp:24-176) ---------------------------------
 * Seconds per amplitude of one pass over the state; the hybrid partitioner
 * and the batch/serving planners predict group times with them. */
typedef struct hq_cost_params {
    double pass_floor;      /* OShareMem pass without gates (HBM read + write) */
    double oshm_gate;       /* + per non-diagonal gate */
    double oshm_diag;       /* + per uncontrolled diagonal gate */
    double oshm_ctrl_diag;  /* + per controlled diagonal gate */
    double mm_bf16x3;       /* 6-qubit TransMM pass, split BF16 (tensor cores) */
    double mm_tf32;         /* 6-qubit TransMM pass, TF32 (tensor cores) */
    double mm_fp32;         /* 6-qubit TransMM pass, FP32 SIMT (x 2^(m-6) beyond 6) */
    double launch;          /* seconds per launch */
} hq_cost_params;
/* The cost model in use (defaults fitted on GB300, or hq_autotune's). */
hq_status hq_cost_params_get(hq_cost_params* out);
/* Install cost-model constants (e.g. ones measured earlier by hq_autotune). */
hq_status hq_cost_params_set(const hq_cost_params* p);
/* Measure the parameters on this GPU with a num_qubits-qubit scratch state
 * (0 = 26; a few seconds, including kernel generation) and install them;
 * *out (may be NULL) receives them, e.g. to save and set again later. */
hq_status hq_autotune(int32_t num_qubits, hq_cost_params* out);

/* ---- batched execution (no reference counterpart: the reference runs one
 * circuit per process, src/circuit.cpp:16-71) ------------------------------
 * Many circuits of uneven qubit counts run in ONE persistent launch that pulls
 * (circuit, gate group, tile range) items from a device work queue. */
typedef struct hq_batch_s* hq_batch;
/* An empty batch; destroy frees its device program (not the states). */
hq_status hq_batch_create(hq_batch* out);
hq_status hq_batch_destroy(hq_batch b);
/* Add circuit c (its gates are copied; it need not be compiled) to run on
 * state s (same qubit count; s must outlive the batch's runs). */
hq_status hq_batch_add(hq_batch b, hq_circuit c, hq_state s, int32_t* index);
/* Plan every circuit as OShareMem groups and upload one program.  opt may be
 * NULL; opt->tile_qubits = 0 lets the cost model choose the tile width of
 * each circuit in [10, 13]; circuits below 10 qubits run gate by gate. */
hq_status hq_batch_compile(hq_batch b, const hq_compile_options* opt);
/* One run of every circuit on its state.  zero_init != 0: states start from
 * |0...0> (written by the first group, never read).  elapsed_us may be NULL. */
hq_status hq_batch_run(hq_batch b, int32_t zero_init, double* elapsed_us);
/* Enqueue a run on the library stream without synchronising. */
hq_status hq_batch_enqueue(hq_batch b, int32_t zero_init);
/* Test hook for failure detection: the next direct run makes one work item
 * wait for a completion count that is never reached.  The device-side wait is
 * bounded (about 2 s); the run then returns HQ_ERR_TIMEOUT, and later runs
 * work as before.  No GPU fault is involved. */
hq_status hq_batch_inject_stall(hq_batch b);
/* Capture a run into a CUDA graph; later runs with the same zero_init replay it. */
hq_status hq_batch_capture_graph(hq_batch b, int32_t zero_init);
/* num_circuits, total gate groups, work items and pass bytes (2 x 8 B x 2^n
 * per group summed over circuits); tile_qubits[i] = tile width chosen for
 * circuit i (0 = gate by gate) when not NULL. */
hq_status hq_batch_info(hq_batch b, int32_t* num_circuits, int64_t* num_groups,
                        int64_t* num_items, uint64_t* pass_bytes, int32_t* tile_qubits);

/* ---- serving (no reference counterpart: one circuit per process there,
 * src/main.cpp:12-230) -------------------------------------------------------
 * A request loop: submit() returns at once; planner threads partition and
 * lower each circuit; an engine thread admits planned requests in arrival
 * order while their state bytes (2^n x 8 B) fit hbm_budget and runs steps,
 * each step one persistent batched launch over the next gate groups of every
 * admitted request (continuous batching).  Results stay resident until
 * hq_server_release. */
typedef struct hq_server_s* hq_server;
#define HQ_REQ_PLANNING 0
#define HQ_REQ_QUEUED 1   /* planned, waiting for memory */
#define HQ_REQ_RUNNING 2
#define HQ_REQ_DONE 3
#define HQ_REQ_FAILED 4
typedef struct hq_server_options {
    uint64_t hbm_budget;     /* bytes of resident states admitted at once; 0 = no limit */
    double step_budget_us;   /* estimated device time of one step, split evenly between
                                the admitted requests; a request whose next group is
                                over its share runs a slice of that group's tiles (0 = 2000) */
    int32_t planner_threads; /* 0 = 4 */
    int32_t tile_qubits;     /* 0 = 13 (or n when smaller); else 10..13 */
    int32_t jit_min_qubits;  /* requests of at least this many qubits get generated group
                                kernels (compiled by the planner threads while other work
                                runs) and run them between the batched launches; 0 or
                                > 34 = never.  Pays off when circuits repeat (the plan
                                cache keeps their kernels): compiling a group costs about
                                a CPU-second, more than it saves on one run */
} hq_server_options;
/* Defaults: 150 GB budget, 2000 us steps, 4 planners, tile 13, no generated
 * kernels. */
hq_status hq_server_options_default(hq_server_options* opt);
/* Host-only admission checks of a request (qubit range 10..34, gate indices,
 * state bytes against the budget); the checks hq_server_submit makes. */
hq_status hq_server_check(const hq_server_options* opt, int32_t num_qubits, const hq_gate* gates,
                          int32_t num_gates);
/* Starts the planner threads and the engine thread. */
hq_status hq_server_create(const hq_server_options* opt, hq_server* out);
/* Stops the engine (the step in flight completes) and frees every state. */
hq_status hq_server_destroy(hq_server sv);
/* Queue a circuit (returns at once with its id); planning runs on the
 * planner threads, admission by state bytes against the HBM budget. */
hq_status hq_server_submit(hq_server sv, int32_t num_qubits, const hq_gate* gates,
                           int32_t num_gates, int64_t* id);
/* Wait up to timeout_s for request id to finish; *status = HQ_REQ_*. */
hq_status hq_server_wait(hq_server sv, int64_t id, double timeout_s, int32_t* status);
/* Ids finished (done or failed) since the last call, at most cap of them. */
hq_status hq_server_poll(hq_server sv, int64_t* ids, int32_t cap, int32_t* count);
/* The finished request's state (borrowed: valid until hq_server_release; do
 * not destroy it).  HQ_ERR_BUSY while queued or running; a failed request
 * returns its error. */
hq_status hq_server_state(hq_server sv, int64_t id, hq_state* out);
/* Host clock (microseconds since the server started) of submit, admission
 * and completion. */
hq_status hq_server_times(hq_server sv, int64_t id, double* submit_us, double* admit_us,
                          double* done_us);
/* Index of the first and last step (batched launch) the request ran in; two
 * requests whose ranges meet shared a launch. */
hq_status hq_server_steps(hq_server sv, int64_t id, int64_t* first_step, int64_t* last_step);
/* Plan cache: requests whose circuit (qubit count and gate records) was
 * planned before reuse that plan.  Hits so far and cached plans. */
hq_status hq_server_plan_cache(hq_server sv, int64_t* hits, int64_t* entries);
/* Frees the request's state (finished requests only). */
hq_status hq_server_release(hq_server sv, int64_t id);
/* Engine counters: steps run, work items, finished requests, resident and
 * peak state bytes. */
hq_status hq_server_stats(hq_server sv, int64_t* steps, int64_t* items, int64_t* finished,
                          uint64_t* resident_bytes, uint64_t* peak_resident_bytes);

/* ---- single group entry points (the reference kernel ABI, src/kernel.h) -- */

/* One OShareMem pass over the state applying `num_gates` gates (logical
 * qubits) whose non-diagonal targets lie in `tile_mask` (logical qubit mask,
 * popcount = tile width).  Replaces copyGatesToSymbol + launchExecutor,
 * src/kernel.h:20-25, src/kernelOpt.cu:499-506. */
hq_status hq_apply_oshm_group(hq_state s, const hq_gate* gates, int32_t num_gates,
                              uint64_t tile_mask);
/* One TransMM pass: fuse the gates (all on the qubits of `group_mask`) into a
 * 2^m x 2^m unitary (FP64 composition on the GPU) and apply it with the given
 * arithmetic.  Replaces GateGroup::initMatrix + cuttExecute + cublasGEMM,
 * src/executor.cpp:533-551. */
hq_status hq_apply_transmm_group(hq_state s, const hq_gate* gates, int32_t num_gates,
                                 uint64_t group_mask, int32_t precision);
/* Apply a caller-given 2^m x 2^m unitary (column-major complex128, m =
 * popcount(group_mask), logical qubit j of the mask = local bit j). */
hq_status hq_apply_unitary(hq_state s, const double* unitary, uint64_t group_mask,
                           int32_t precision);
/* Fused FP64 unitary of gates on the qubits of group_mask, composed on the
 * GPU, copied to host (column-major complex128).  GateGroup::initCPUMatrix,
 * src/schedule.cpp:578-702. */
hq_status hq_group_unitary(const hq_gate* gates, int32_t num_gates, uint64_t group_mask,
                           double* unitary_out);
/* Permute qubits in HBM: after the call logical qubit q sits at physical bit
 * new_pos[q].  The single-GPU form of the reference's transpose + all-to-all
 * (src/executor.cpp:59-179). */
hq_status hq_state_remap(hq_state s, const int32_t* new_pos);

#ifdef __cplusplus
}
#endif
#endif
