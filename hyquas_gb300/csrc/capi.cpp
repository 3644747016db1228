// C-ABI entry points (include/hyquas_gb300.h): state objects, the plain
// per-gate path, compiled circuits and their executor, FP64 readout.
#include <cuda_runtime.h>

#include <sys/mman.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "batch.h"
#include "common.h"
#include "compiler.h"
#include "device.h"
#include "executor.h"
#include "gates.h"
#include "server.h"

namespace hq {
const std::string& last_error();
void init_explicit(int device);
}  // namespace hq

using namespace hq;

#define HQ_API_BEGIN \
    try {            \
        clear_last_error();
#define HQ_API_END                              \
    return HQ_OK;                               \
    }                                           \
    catch (const Failure& f) {                  \
        set_last_error(f.what());               \
        return f.code;                          \
    }                                           \
    catch (const std::bad_alloc&) {             \
        set_last_error("host allocation failed"); \
        return HQ_ERR_NOMEM;                    \
    }                                           \
    catch (const std::exception& e) {           \
        set_last_error(e.what());               \
        return HQ_ERR_INVALID;                  \
    }

#define HQ_NONNULL(p) HQ_REQUIRE((p) != nullptr, HQ_ERR_INVALID, "%s must not be NULL", #p)

extern "C" {

const char* hq_last_error(void) { return hq::last_error().c_str(); }
const char* hq_version(void) { return "hyquas_gb300 0.1 (sm_103a)"; }

hq_status hq_init(int device) {
    HQ_API_BEGIN
    init_explicit(device);
    HQ_API_END
}

hq_status hq_device_info(int32_t* sm_count, uint64_t* hbm_bytes, int32_t* smem_per_block) {
    HQ_API_BEGIN
    Context& c = ctx();
    if (sm_count) *sm_count = c.sm_count;
    if (hbm_bytes) *hbm_bytes = c.hbm_bytes;
    if (smem_per_block) *smem_per_block = c.smem_optin;
    HQ_API_END
}

hq_status hq_set_hbm_budget(uint64_t bytes) {
    HQ_API_BEGIN
    ctx().budget = bytes;
    HQ_API_END
}

hq_status hq_hbm_in_use(uint64_t* bytes) {
    HQ_API_BEGIN
    HQ_NONNULL(bytes);
    *bytes = ctx().in_use;
    HQ_API_END
}

// Buffers of 64 MiB and more are mapped with transparent huge pages requested
// and then page-locked (cudaHostRegister): a multi-GiB buffer made of small
// pages, on a host whose memory is fragmented, was measured to read back at
// 27 GB/s against 193 GB/s for one made of huge pages on the same box.
namespace {
std::mutex g_host_mu;
std::map<void*, size_t> g_host_mapped;  // registered mmap buffers and their sizes
}  // namespace

hq_status hq_host_alloc(uint64_t bytes, void** out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    ensure_init();
    *out = nullptr;
    if (bytes >= (uint64_t(64) << 20)) {
        void* p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
        if (p != MAP_FAILED) {
            (void)madvise(p, bytes, MADV_HUGEPAGE);  // a hint: ignored where THP is off
            const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped);
            if (e == cudaSuccess) {
                // the device's first writes to the pages, made here rather than
                // in the first readback into the buffer
                void* dp = nullptr;
                if (cudaHostGetDevicePointer(&dp, p, 0) == cudaSuccess && dp) {
                    launch_touch_pages(dp, bytes, ctx().stream);
                    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
                } else {
                    (void)cudaGetLastError();
                }
                std::lock_guard<std::mutex> lk(g_host_mu);
                g_host_mapped[p] = bytes;
                *out = p;
                return HQ_OK;
            }
            (void)cudaGetLastError();
            munmap(p, bytes);
        }
    }
    HQ_CHECK_CUDA(cudaHostAlloc(out, bytes, cudaHostAllocDefault));
    HQ_API_END
}

hq_status hq_host_free(void* p) {
    HQ_API_BEGIN
    if (p) {
        size_t mapped = 0;
        {
            std::lock_guard<std::mutex> lk(g_host_mu);
            auto it = g_host_mapped.find(p);
            if (it != g_host_mapped.end()) {
                mapped = it->second;
                g_host_mapped.erase(it);
            }
        }
        if (mapped) {
            HQ_CHECK_CUDA(cudaHostUnregister(p));
            munmap(p, mapped);
        } else {
            HQ_CHECK_CUDA(cudaFreeHost(p));
        }
    }
    HQ_API_END
}

hq_status hq_gate_make(int32_t type, int32_t target, int32_t control, int32_t control2,
                       const double* params, hq_gate* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    *out = make_gate(type, target, control, control2, params);
    HQ_API_END
}

// ---- states ---------------------------------------------------------------------

hq_status hq_state_create(int32_t n, hq_state* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    *out = nullptr;
    *out = state_create(n);
    HQ_API_END
}

hq_status hq_state_destroy(hq_state s) {
    HQ_API_BEGIN
    state_destroy(s);
    HQ_API_END
}

hq_status hq_state_init_zero(hq_state s) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    state_wait_copy(s);
    launch_init_zero(s->d, s->n, ctx().stream);
    for (int q = 0; q < s->n; q++) s->pos[q] = q;
    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
    HQ_API_END
}

hq_status hq_state_load(hq_state s, const float* host) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(host);
    state_wait_copy(s);
    HQ_CHECK_CUDA(cudaMemcpyAsync(s->d, host, s->bytes, cudaMemcpyHostToDevice, ctx().stream));
    for (int q = 0; q < s->n; q++) s->pos[q] = q;
    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
    HQ_API_END
}

hq_status hq_state_store(hq_state s, float* host) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(host);
    state_canonicalize(s);
    HQ_CHECK_CUDA(cudaMemcpyAsync(host, s->d, s->bytes, cudaMemcpyDeviceToHost, ctx().stream));
    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
    HQ_API_END
}

hq_status hq_state_store_async(hq_state s, float* host) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(host);
    state_store_async(s, host);
    HQ_API_END
}

hq_status hq_state_wait(hq_state s) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    state_wait_host(s);
    HQ_API_END
}

hq_status hq_state_amps(hq_state s, const uint64_t* idx, int64_t count, float* out) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_REQUIRE(count >= 0, HQ_ERR_INVALID, "negative count");
    if (count == 0) return HQ_OK;
    HQ_NONNULL(idx);
    HQ_NONNULL(out);
    state_gather(s, idx, count, out);
    HQ_API_END
}

hq_status hq_state_layout(hq_state s, int32_t* pos) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(pos);
    for (int q = 0; q < s->n; q++) pos[q] = s->pos[q];
    HQ_API_END
}

hq_status hq_state_num_qubits(hq_state s, int32_t* n) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(n);
    *n = s->n;
    HQ_API_END
}

hq_status hq_state_device_ptr(hq_state s, void** p) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(p);
    *p = s->d;
    HQ_API_END
}

hq_status hq_state_marginals(hq_state s, double* p1) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(p1);
    double h[1 + 64];
    state_marginals(s, h);
    for (int q = 0; q < s->n; q++) p1[q] = h[1 + s->pos[q]];
    HQ_API_END
}

hq_status hq_state_sample(hq_state s, int32_t shots, uint64_t seed, uint64_t* out) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_REQUIRE(shots >= 0, HQ_ERR_INVALID, "negative shot count");
    if (shots > 0) HQ_NONNULL(out);
    state_sample(s, shots, seed, out);
    HQ_API_END
}

hq_status hq_state_norm(hq_state s, double* norm) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(norm);
    double h[1 + 64];
    state_marginals(s, h);
    *norm = h[0];
    HQ_API_END
}

hq_status hq_state_prob_zero(hq_state s, int32_t q, double* p0) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(p0);
    HQ_REQUIRE(q >= 0 && q < s->n, HQ_ERR_INVALID, "qubit %d out of range", q);
    double h[1 + 64];
    state_marginals(s, h);
    *p0 = h[0] - h[1 + s->pos[q]];
    HQ_API_END
}

hq_status hq_state_remap(hq_state s, const int32_t* new_pos) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    HQ_NONNULL(new_pos);
    std::vector<int> np(new_pos, new_pos + s->n);
    state_remap(s, np);
    HQ_API_END
}

// ---- plain path ------------------------------------------------------------------

hq_status hq_apply_gates(hq_state s, const hq_gate* gates, int32_t num_gates) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    state_wait_copy(s);
    HQ_REQUIRE(num_gates >= 0, HQ_ERR_INVALID, "negative gate count");
    if (num_gates == 0) return HQ_OK;
    HQ_NONNULL(gates);
    std::vector<hq_gate> v(gates, gates + num_gates);
    apply_plain(s, v);
    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
    HQ_API_END
}

hq_status hq_synchronize(void) {
    HQ_API_BEGIN
    HQ_CHECK_CUDA(cudaStreamSynchronize(ctx().stream));
    check_device_error();
    HQ_API_END
}

// ---- circuits --------------------------------------------------------------------

hq_status hq_compile_options_default(hq_compile_options* opt) {
    HQ_API_BEGIN
    HQ_NONNULL(opt);
    std::memset(opt, 0, sizeof(*opt));
    opt->backend = HQ_BACKEND_OSHM;
    opt->mm_precision = HQ_MM_BF16X3;
    opt->specialize = 2;
    HQ_API_END
}

hq_status hq_circuit_create(int32_t n, hq_circuit* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    HQ_REQUIRE(n >= 1 && n <= 36, HQ_ERR_INVALID, "num_qubits %d out of range [1,36]", n);
    auto c = new hq_circuit_s();
    c->n = n;
    *out = c;
    HQ_API_END
}

hq_status hq_circuit_destroy(hq_circuit c) {
    HQ_API_BEGIN
    if (c) {
        circuit_release(c);
        delete c;
    }
    HQ_API_END
}

hq_status hq_circuit_add_gates(hq_circuit c, const hq_gate* gates, int32_t num_gates) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_REQUIRE(num_gates >= 0, HQ_ERR_INVALID, "negative gate count");
    for (int i = 0; i < num_gates; i++) {
        validate_gate(gates[i], c->n);
        c->gates.push_back(gates[i]);
    }
    c->compiled = false;
    HQ_API_END
}

hq_status hq_circuit_num_gates(hq_circuit c, int32_t* num_gates) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(num_gates);
    *num_gates = (int32_t)c->gates.size();
    HQ_API_END
}

hq_status hq_circuit_compile(hq_circuit c, const hq_compile_options* opt) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    hq_compile_options o;
    if (opt)
        o = *opt;
    else
        hq_compile_options_default(&o);
    circuit_compile(c, o);
    HQ_API_END
}

hq_status hq_circuit_schedule(hq_circuit c, int32_t* num_groups, int32_t* backend,
                              int32_t* gates_per_group, int32_t* width, uint64_t* related) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    const auto& gs = c->part.groups;
    if (num_groups) *num_groups = (int32_t)gs.size();
    for (size_t i = 0; i < gs.size(); i++) {
        if (backend) backend[i] = gs[i].backend;
        if (gates_per_group) gates_per_group[i] = (int32_t)gs[i].gates.size();
        if (width) width[i] = gs[i].width;
        if (related) related[i] = gs[i].related;
    }
    HQ_API_END
}

hq_status hq_circuit_group_gates(hq_circuit c, int32_t g, int32_t* gate_idx, int32_t cap,
                                 int32_t* count) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    HQ_REQUIRE(g >= 0 && g < (int)c->part.groups.size(), HQ_ERR_INVALID, "group %d out of range", g);
    const auto& v = c->part.groups[g].gates;
    if (count) *count = (int32_t)v.size();
    if (gate_idx) {
        HQ_REQUIRE(cap >= (int)v.size(), HQ_ERR_INVALID, "gate_idx capacity %d < %zu", cap, v.size());
        for (size_t i = 0; i < v.size(); i++) gate_idx[i] = c->orig_index[v[i]];
    }
    HQ_API_END
}

hq_status hq_plan_groups(int32_t n, const hq_gate* gates, int32_t num_gates,
                         const hq_compile_options* opt, int32_t* num_groups, int32_t* backend,
                         int32_t* gates_per_group, int32_t* width, uint64_t* related,
                         int32_t* phases, int32_t* gate_order) {
    HQ_API_BEGIN
    HQ_REQUIRE(n >= 6 && n <= 36, HQ_ERR_INVALID, "num_qubits %d out of range [6,36]", n);
    HQ_REQUIRE(num_gates >= 0 && (num_gates == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    hq_compile_options o;
    if (opt)
        o = *opt;
    else
        hq_compile_options_default(&o);
    std::vector<hq_gate> v(gates, gates + num_gates);
    for (auto& g : v) validate_gate(g, n);
    std::vector<int> perm, orig;
    std::vector<hq_gate> folded = fold_swaps(v, n, perm);
    for (int i = 0; i < num_gates; i++)
        if (v[i].type != G_SWAP) orig.push_back(i);
    CompileConfig cfg = config_from_options(o, n);
    std::vector<int> id(n);
    for (int q = 0; q < n; q++) id[q] = q;
    Partition part = partition(n, folded, id, cfg);
    if (num_groups) *num_groups = (int32_t)part.groups.size();
    size_t k = 0;
    for (size_t i = 0; i < part.groups.size(); i++) {
        const GroupPlan& gp = part.groups[i];
        if (backend) backend[i] = gp.backend;
        if (gates_per_group) gates_per_group[i] = (int32_t)gp.gates.size();
        if (width) width[i] = gp.width;
        if (related) related[i] = gp.related;
        if (phases) {
            phases[i] = 0;
            if (gp.backend == HQ_BACKEND_OSHM && !cfg.reference) {
                std::vector<hq_gate> pg;
                for (int x : gp.gates) pg.push_back(folded[x]);
                phases[i] = (int32_t)plan_oshm(n, pg, oshm_tile_mask(gp, n)).phases.size();
            }
        }
        if (gate_order)
            for (int x : gp.gates) gate_order[k++] = orig[x];
    }
    HQ_API_END
}

namespace {
hq_status copy_out(const std::vector<uint8_t>& b, void* buf, uint64_t cap, uint64_t* len) {
    *len = b.size();
    if (!buf) return HQ_OK;  // size query
    HQ_REQUIRE(cap >= b.size(), HQ_ERR_INVALID, "buffer of %llu bytes, schedule needs %zu",
               (unsigned long long)cap, b.size());
    std::memcpy(buf, b.data(), b.size());
    return HQ_OK;
}
}  // namespace

hq_status hq_circuit_serialize(hq_circuit c, void* buf, uint64_t cap, uint64_t* len) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(len);
    copy_out(schedule_serialize(c), buf, cap, len);
    HQ_API_END
}

hq_status hq_plan_serialize(int32_t n, const hq_gate* gates, int32_t num_gates,
                            const hq_compile_options* opt, void* buf, uint64_t cap, uint64_t* len) {
    HQ_API_BEGIN
    HQ_NONNULL(len);
    HQ_REQUIRE(n >= 1 && n <= 36, HQ_ERR_INVALID, "num_qubits %d out of range [1,36]", n);
    HQ_REQUIRE(num_gates >= 0 && (num_gates == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    hq_compile_options o;
    if (opt)
        o = *opt;
    else
        hq_compile_options_default(&o);
    hq_circuit_s c;
    c.n = n;
    for (int32_t i = 0; i < num_gates; i++) {
        validate_gate(gates[i], n);
        c.gates.push_back(gates[i]);
    }
    circuit_plan(&c, o);
    c.compiled = true;  // the plan is all the bytes hold
    copy_out(schedule_serialize(&c), buf, cap, len);
    HQ_API_END
}

hq_status hq_schedule_inspect(const void* buf, uint64_t len, int32_t* num_qubits, int32_t* num_gates,
                              int32_t* num_groups, int32_t* backend, int32_t* gates_per_group,
                              int32_t* width, uint64_t* related) {
    HQ_API_BEGIN
    hq_circuit_s c;
    schedule_deserialize(static_cast<const uint8_t*>(buf), (size_t)len, &c);
    if (num_qubits) *num_qubits = c.n;
    if (num_gates) *num_gates = (int32_t)c.gates.size();
    if (num_groups) *num_groups = (int32_t)c.part.groups.size();
    for (size_t i = 0; i < c.part.groups.size(); i++) {
        const GroupPlan& gp = c.part.groups[i];
        if (backend) backend[i] = gp.backend;
        if (gates_per_group) gates_per_group[i] = (int32_t)gp.gates.size();
        if (width) width[i] = gp.width;
        if (related) related[i] = gp.related;
    }
    HQ_API_END
}

hq_status hq_circuit_deserialize(const void* buf, uint64_t len, hq_circuit* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    std::unique_ptr<hq_circuit_s> c(new hq_circuit_s());
    schedule_deserialize(static_cast<const uint8_t*>(buf), (size_t)len, c.get());
    ensure_init();
    try {
        circuit_lower(c.get());
    } catch (...) {
        circuit_release(c.get());
        throw;
    }
    *out = c.release();
    HQ_API_END
}

hq_status hq_circuit_program_bytes(hq_circuit c, uint64_t* bytes) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(bytes);
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    *bytes = c->phases_bytes + c->ops_bytes + c->umats_bytes + c->mm_scratch_bytes;
    HQ_API_END
}

hq_status hq_circuit_run(hq_circuit c, hq_state s, double* elapsed_us) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    const double us = circuit_run(c, s, true);
    if (elapsed_us) *elapsed_us = us;
    HQ_API_END
}

hq_status hq_circuit_run_to_host(hq_circuit c, hq_state s, float* host_amps, double* elapsed_us) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    HQ_NONNULL(host_amps);
    const double us = circuit_run_to_host(c, s, host_amps);
    if (elapsed_us) *elapsed_us = us;
    HQ_API_END
}

hq_status hq_circuit_profile(hq_circuit c, hq_state s, double* group_us) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    HQ_NONNULL(group_us);
    circuit_profile(c, s, group_us);
    HQ_API_END
}

hq_status hq_circuit_predict(hq_circuit c, double* group_us) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(group_us);
    circuit_predict(c, group_us);
    HQ_API_END
}

hq_status hq_circuit_enqueue(hq_circuit c, hq_state s) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    circuit_run(c, s, false);
    HQ_API_END
}

hq_status hq_circuit_capture_graph(hq_circuit c, hq_state s) {
    HQ_API_BEGIN
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    circuit_capture(c, s);
    HQ_API_END
}

// ---- OpenQASM front-end --------------------------------------------------------------

hq_status hq_qasm_parse(const char* text, int32_t* num_qubits, hq_gate* out, int32_t cap,
                        int32_t* count) {
    HQ_API_BEGIN
    HQ_NONNULL(text);
    int n = 0;
    std::vector<hq_gate> gates;
    parse_qasm(text, n, gates);
    if (num_qubits) *num_qubits = n;
    if (count) *count = (int32_t)gates.size();
    if (out) {
        HQ_REQUIRE(cap >= (int32_t)gates.size(), HQ_ERR_INVALID, "qasm: %zu gates, room for %d",
                   gates.size(), cap);
        std::copy(gates.begin(), gates.end(), out);
    }
    HQ_API_END
}

// ---- cost model ---------------------------------------------------------------------

hq_status hq_cost_params_get(hq_cost_params* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    *out = cost_params();
    HQ_API_END
}

hq_status hq_cost_params_set(const hq_cost_params* p) {
    HQ_API_BEGIN
    HQ_NONNULL(p);
    set_cost_params(*p);
    HQ_API_END
}

hq_status hq_autotune(int32_t num_qubits, hq_cost_params* out) {
    HQ_API_BEGIN
    const hq_cost_params p = autotune(num_qubits);
    if (out) *out = p;
    HQ_API_END
}

// ---- batches ------------------------------------------------------------------------

hq_status hq_batch_create(hq_batch* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    *out = new hq_batch_s();
    HQ_API_END
}

hq_status hq_batch_destroy(hq_batch b) {
    HQ_API_BEGIN
    if (b) {
        batch_release(b);
        if (b->ev0) cudaEventDestroy(b->ev0);
        if (b->ev1) cudaEventDestroy(b->ev1);
        delete b;
    }
    HQ_API_END
}

hq_status hq_batch_add(hq_batch b, hq_circuit c, hq_state s, int32_t* index) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    HQ_NONNULL(c);
    HQ_NONNULL(s);
    HQ_REQUIRE(c->n == s->n, HQ_ERR_INVALID, "state has %d qubits, circuit %d", s->n, c->n);
    for (const BatchEntry& e : b->entries)
        HQ_REQUIRE(e.s != s, HQ_ERR_INVALID, "state already in the batch");
    BatchEntry e;
    e.n = c->n;
    e.s = s;
    e.gates = c->gates;
    b->entries.push_back(std::move(e));
    batch_release(b);  // needs a new compile
    if (index) *index = (int32_t)b->entries.size() - 1;
    HQ_API_END
}

hq_status hq_batch_compile(hq_batch b, const hq_compile_options* opt) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    batch_compile(b, opt);
    HQ_API_END
}

hq_status hq_batch_run(hq_batch b, int32_t zero_init, double* elapsed_us) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    const double us = batch_run(b, zero_init != 0);
    if (elapsed_us) *elapsed_us = us;
    HQ_API_END
}

hq_status hq_batch_enqueue(hq_batch b, int32_t zero_init) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    batch_enqueue(b, zero_init != 0);
    HQ_API_END
}

hq_status hq_batch_inject_stall(hq_batch b) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    HQ_REQUIRE(b->compiled, HQ_ERR_STATE, "batch not compiled");
    b->stall_next = true;
    HQ_API_END
}

hq_status hq_batch_capture_graph(hq_batch b, int32_t zero_init) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    batch_capture(b, zero_init != 0);
    HQ_API_END
}

hq_status hq_batch_info(hq_batch b, int32_t* num_circuits, int64_t* num_groups,
                        int64_t* num_items, uint64_t* pass_bytes, int32_t* tile_qubits) {
    HQ_API_BEGIN
    HQ_NONNULL(b);
    if (num_circuits) *num_circuits = (int32_t)b->entries.size();
    if (num_groups) *num_groups = b->num_groups;
    if (num_items) *num_items = b->num_items;
    if (pass_bytes) *pass_bytes = b->pass_bytes;
    if (tile_qubits)
        for (size_t i = 0; i < b->entries.size(); i++) tile_qubits[i] = b->entries[i].k;
    HQ_API_END
}

// ---- serving ------------------------------------------------------------------------

hq_status hq_server_options_default(hq_server_options* opt) {
    HQ_API_BEGIN
    HQ_NONNULL(opt);
    std::memset(opt, 0, sizeof(*opt));
    opt->hbm_budget = 150ull * 1000 * 1000 * 1000;
    opt->step_budget_us = 2000.0;
    opt->planner_threads = 4;
    opt->tile_qubits = 0;
    opt->jit_min_qubits = 0;
    HQ_API_END
}

hq_status hq_server_check(const hq_server_options* opt, int32_t num_qubits, const hq_gate* gates,
                          int32_t num_gates) {
    HQ_API_BEGIN
    HQ_NONNULL(opt);
    server_check(*opt, num_qubits, gates, num_gates);
    HQ_API_END
}

hq_status hq_server_create(const hq_server_options* opt, hq_server* out) {
    HQ_API_BEGIN
    HQ_NONNULL(out);
    hq_server_options o;
    if (opt) {
        o = *opt;
    } else {
        hq_server_options_default(&o);
    }
    HQ_REQUIRE(o.tile_qubits == 0 || (o.tile_qubits >= kBatchMinTile && o.tile_qubits <= kBatchTile),
               HQ_ERR_INVALID, "tile_qubits %d outside [%d, %d]", o.tile_qubits, kBatchMinTile,
               kBatchTile);
    *out = server_create(o);
    HQ_API_END
}

hq_status hq_server_destroy(hq_server sv) {
    HQ_API_BEGIN
    if (sv) server_destroy(sv);
    HQ_API_END
}

hq_status hq_server_submit(hq_server sv, int32_t num_qubits, const hq_gate* gates,
                           int32_t num_gates, int64_t* id) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    const int64_t v = server_submit(sv, num_qubits, gates, num_gates);
    if (id) *id = v;
    HQ_API_END
}

hq_status hq_server_wait(hq_server sv, int64_t id, double timeout_s, int32_t* status) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    const int st = server_wait(sv, id, timeout_s);
    if (status) *status = st;
    HQ_API_END
}

hq_status hq_server_poll(hq_server sv, int64_t* ids, int32_t cap, int32_t* count) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    HQ_REQUIRE(cap >= 0 && (cap == 0 || ids), HQ_ERR_INVALID, "bad id buffer");
    const int k = server_poll(sv, ids, cap);
    if (count) *count = k;
    HQ_API_END
}

hq_status hq_server_state(hq_server sv, int64_t id, hq_state* out) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    HQ_NONNULL(out);
    std::lock_guard<std::mutex> lk(sv->mu);
    Request* r = server_find(sv, id);
    HQ_REQUIRE(r->status != HQ_REQ_FAILED, HQ_ERR_STATE, "request %lld failed: %s", (long long)id,
               r->error.c_str());
    HQ_REQUIRE(r->status == HQ_REQ_DONE, HQ_ERR_BUSY, "request %lld not finished", (long long)id);
    HQ_REQUIRE(!r->released && r->state, HQ_ERR_STATE, "request %lld released", (long long)id);
    *out = r->state;
    HQ_API_END
}

hq_status hq_server_times(hq_server sv, int64_t id, double* submit_us, double* admit_us,
                          double* done_us) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    std::lock_guard<std::mutex> lk(sv->mu);
    Request* r = server_find(sv, id);
    if (submit_us) *submit_us = r->t_submit;
    if (admit_us) *admit_us = r->t_admit;
    if (done_us) *done_us = r->t_done;
    HQ_API_END
}

hq_status hq_server_steps(hq_server sv, int64_t id, int64_t* first_step, int64_t* last_step) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    std::lock_guard<std::mutex> lk(sv->mu);
    Request* r = server_find(sv, id);
    if (first_step) *first_step = r->first_step;
    if (last_step) *last_step = r->last_step;
    HQ_API_END
}

hq_status hq_server_plan_cache(hq_server sv, int64_t* hits, int64_t* entries) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    std::lock_guard<std::mutex> lk(sv->cache_mu);
    if (hits) *hits = sv->cache_hits;
    if (entries) *entries = (int64_t)sv->plan_cache.size();
    HQ_API_END
}

hq_status hq_server_release(hq_server sv, int64_t id) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    server_release(sv, id);
    HQ_API_END
}

hq_status hq_server_stats(hq_server sv, int64_t* steps, int64_t* items, int64_t* finished,
                          uint64_t* resident_bytes, uint64_t* peak_resident_bytes) {
    HQ_API_BEGIN
    HQ_NONNULL(sv);
    std::lock_guard<std::mutex> lk(sv->mu);
    if (steps) *steps = sv->steps;
    if (items) *items = sv->items;
    if (finished) *finished = sv->ndone;
    if (resident_bytes) *resident_bytes = sv->resident;
    if (peak_resident_bytes) *peak_resident_bytes = sv->peak_resident;
    HQ_API_END
}

hq_status hq_apply_oshm_group(hq_state s, const hq_gate* gates, int32_t num_gates,
                              uint64_t tile_mask) {
    HQ_API_BEGIN
    HQ_NONNULL(s);
    state_wait_copy(s);
    HQ_REQUIRE(num_gates >= 0 && (num_gates == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    std::vector<hq_gate> v(gates, gates + num_gates);
    apply_oshm_group(s, v, tile_mask);
    HQ_API_END
}

}  // extern "C"
