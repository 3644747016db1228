// State vectors, compiled circuits and the executor that walks a schedule.
// Replaces Executor (src/executor.cpp:33-57, 405-551) and the state handling
// of Circuit (src/circuit.cpp:16-71).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "compiler.h"
#include "jit.h"

struct hq_state_s {
    int n = 0;
    void* d = nullptr;          // float2[2^n], physical order
    size_t bytes = 0;
    std::vector<int> pos;       // logical -> physical
    double* d_scratch = nullptr;  // reduction partials (FP64)
    size_t scratch_doubles = 0;
    // asynchronous readback (state_store_async): the copy runs on the library's
    // copy stream; work that writes the state first waits for copy_done
    cudaEvent_t ready = nullptr, copy_done = nullptr;
    bool copy_pending = false;
};

namespace hq {

// Generated kernels of a circuit being compiled on a host thread while the
// circuit runs interpreted (compile option specialize = 3, kernels not cached).
struct JitJob {
    std::thread th;
    std::mutex mu;
    std::mutex join_mu;             // joins from the installing run and the exit hook
    bool done = false;
    std::vector<OshmProgram> progs;
    std::vector<size_t> groups;     // dgroups index of each program
    std::vector<JitKernel> kernels;
    std::string err;
    void join() {
        std::lock_guard<std::mutex> lk(join_mu);
        if (th.joinable()) th.join();
    }
};

struct DeviceGroup {
    int backend = HQ_BACKEND_OSHM;
    // OShareMem
    OshmProgram prog;
    size_t phase_off = 0, op_off = 0;  // offsets into the circuit's device arrays
    // TransMM
    int mm_m = 0;
    uint64_t mm_rows = 0;        // physical row bits (group qubits)
    uint64_t mm_tile = 0;        // physical tile bits (rows + columns)
    int mm_precision = HQ_MM_BF16X3;
    size_t umat_off = 0;         // offset (doubles) of the FP64 fused unitary
    size_t operand_off = 0;      // offset (bytes) of the precision-specific operand
    std::vector<hq_gate> phys_gates;
    bool has_jit = false;        // a generated kernel replaces the interpreter
    JitKernel jit;
};

}  // namespace hq

struct hq_circuit_s {
    int n = 0;
    std::vector<hq_gate> gates;         // as added (may contain SWAP)
    bool compiled = false;
    hq_compile_options opt{};
    std::vector<hq_gate> folded;        // SWAPs folded away
    std::vector<int> orig_index;        // folded index -> index in `gates`
    std::vector<int> swap_perm;         // user qubit s names physical qubit swap_perm[s]
    hq::Partition part;
    std::vector<hq::DeviceGroup> dgroups;
    hq::OshmPhase* d_phases = nullptr;
    size_t phases_bytes = 0;
    hq::OshmOp* d_ops = nullptr;
    size_t ops_bytes = 0;
    double* d_umats = nullptr;          // fused unitaries (complex128, column-major)
    size_t umats_bytes = 0;
    void* d_mm_scratch = nullptr;       // TransMM operand staging (split BF16 / FP32)
    size_t mm_scratch_bytes = 0;
    // CUDA graph of the schedule for one state
    cudaGraphExec_t graph = nullptr;
    const hq_state_s* graph_state = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool specialized = false;           // OShareMem groups run generated kernels
    std::string specialize_note;        // why not, when requested in auto mode
    std::shared_ptr<hq::JitJob> jit_job;  // generated kernels still compiling
};

namespace hq {

hq_state_s* state_create(int n);
void state_destroy(hq_state_s* s);
void state_canonicalize(hq_state_s* s);
// the library stream waits for a pending asynchronous readback of s (before writing s)
void state_wait_copy(hq_state_s* s);
// canonical-order device -> host copy on the copy stream; returns at once
void state_store_async(hq_state_s* s, void* host);
// block until s's asynchronous readback has landed in host memory
void state_wait_host(hq_state_s* s);
void state_remap(hq_state_s* s, const std::vector<int>& new_pos);
void state_gather(hq_state_s* s, const uint64_t* logical_idx, int64_t count, float* out);
void state_marginals(hq_state_s* s, double* h_out);  // [total, p1(phys bit b)]
// `shots` outcomes (logical basis indices) drawn from |amp|^2 with a seeded stream.
void state_sample(hq_state_s* s, int shots, uint64_t seed, uint64_t* out);
size_t state_scratch_doubles(int n);  // FP64 reduction scratch a state carries

void apply_plain(hq_state_s* s, const std::vector<hq_gate>& gates);
void apply_oshm_group(hq_state_s* s, const std::vector<hq_gate>& gates, uint64_t tile_mask_logical);

CompileConfig config_from_options(const hq_compile_options& o, int n);
uint64_t oshm_tile_mask(const GroupPlan& gp, int n);
void circuit_compile(hq_circuit_s* c, const hq_compile_options& opt);
// the two halves of compile: the host plan (SWAP folding, fusion for the
// interpreter, partition) and the device lowering (phases, fused unitaries,
// uploads, generated kernels) of the plan already in `c`
void circuit_plan(hq_circuit_s* c, const hq_compile_options& opt);
void circuit_lower(hq_circuit_s* c);
// compiled-schedule bytes (schedule_io.cpp)
std::vector<uint8_t> schedule_serialize(const hq_circuit_s* c);
// parse and check `len` bytes into c's plan (gates, options, partition); no device work
void schedule_deserialize(const uint8_t* buf, size_t len, hq_circuit_s* c);
double circuit_run(hq_circuit_s* c, hq_state_s* s, bool sync);
double circuit_run_to_host(hq_circuit_s* c, hq_state_s* s, void* host);
void circuit_capture(hq_circuit_s* c, hq_state_s* s);
void circuit_profile(hq_circuit_s* c, hq_state_s* s, double* group_us);
// the cost model's device time per group (us) of a compiled circuit
void circuit_predict(const hq_circuit_s* c, double* group_us);
void circuit_release(hq_circuit_s* c);
// Generated kernels compiled on a host thread (specialize = 3): install them
// once ready (wait = true: wait for them).  Runs call this before launching.
void circuit_jit_install(hq_circuit_s* c, bool wait);
// Enqueue every group of a compiled circuit on `stream` (no layout handling).
void circuit_launch_groups(hq_circuit_s* c, void* state, cudaStream_t stream);

}  // namespace hq
