#include "executor.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "common.h"
#include "transmm.h"

namespace hq {

// ---- states ---------------------------------------------------------------------

size_t state_scratch_doubles(int n) {
    const uint64_t nquads = (uint64_t(1) << n) / 2;
    const uint64_t nb1 = (nquads + 2047) / 2048;
    const uint64_t nb2 = (nb1 + 4095) / 4096;
    return size_t(nb1 * 13 + nb2 * 25);
}

hq_state_s* state_create(int n) {
    HQ_REQUIRE(n >= 1 && n <= 36, HQ_ERR_INVALID, "num_qubits %d out of range [1,36]", n);
    ensure_init();
    auto s = new hq_state_s();
    s->n = n;
    s->bytes = sizeof(float) * 2 * (size_t(1) << n);
    s->pos.resize(n);
    for (int q = 0; q < n; q++) s->pos[q] = q;
    try {
        s->d = dev_alloc(s->bytes);
        s->scratch_doubles = state_scratch_doubles(n);
        s->d_scratch = (double*)dev_alloc(sizeof(double) * s->scratch_doubles);
    } catch (...) {
        if (s->d) dev_free(s->d, s->bytes);
        delete s;
        throw;
    }
    return s;
}

void state_destroy(hq_state_s* s) {
    if (!s) return;
    if (s->copy_pending) cudaEventSynchronize(s->copy_done);
    if (s->ready) cudaEventDestroy(s->ready);
    if (s->copy_done) cudaEventDestroy(s->copy_done);
    if (s->d) dev_free(s->d, s->bytes);
    if (s->d_scratch) dev_free(s->d_scratch, sizeof(double) * s->scratch_doubles);
    delete s;
}

void state_remap(hq_state_s* s, const std::vector<int>& np) {
    state_wait_copy(s);
    const int n = s->n;
    HQ_REQUIRE((int)np.size() == n, HQ_ERR_INVALID, "remap: layout size");
    std::vector<char> seen(n, 0);
    for (int q = 0; q < n; q++) {
        HQ_REQUIRE(np[q] >= 0 && np[q] < n && !seen[np[q]], HQ_ERR_INVALID,
                   "remap: not a permutation");
        seen[np[q]] = 1;
    }
    cudaStream_t st = ctx().stream;
    // the exchanges that bring the layout to np, in order
    std::vector<std::pair<int, int>> swaps;
    {
        std::vector<int> pos = s->pos;
        for (int q = 0; q < n; q++) {
            if (pos[q] == np[q]) continue;
            int q2 = -1;
            for (int x = 0; x < n; x++)
                if (pos[x] == np[q]) q2 = x;
            swaps.push_back({pos[q], np[q]});
            pos[q2] = pos[q];
            pos[q] = np[q];
        }
    }
    // consecutive exchanges run together as one in-place pass while the bits
    // they move fit a tile (launch_permute_bits: one read and one write of the
    // state); a lone exchange runs as one (half the state read and written)
    size_t i = 0;
    while (i < swaps.size()) {
        std::vector<int> dest_of(n);
        for (int b = 0; b < n; b++) dest_of[b] = b;
        size_t j = i;
        while (j < swaps.size()) {
            std::vector<int> trial = dest_of;
            for (int b = 0; b < n; b++) {
                if (trial[b] == swaps[j].first) trial[b] = swaps[j].second;
                else if (trial[b] == swaps[j].second) trial[b] = swaps[j].first;
            }
            if (permute_tile_bits(n, trial.data()) > kPermuteMaxTileBits) break;
            dest_of.swap(trial);
            j++;
        }
        if (j == i) j = i + 1;  // cannot happen (one exchange moves two bits); kept safe
        if (j - i == 1)
            launch_bit_swap(s->d, n, swaps[i].first, swaps[i].second, st);
        else
            launch_permute_bits(s->d, n, dest_of.data(), st);
        i = j;
    }
    s->pos = np;
}

void state_wait_copy(hq_state_s* s) {
    if (s->copy_pending) HQ_CHECK_CUDA(cudaStreamWaitEvent(ctx().stream, s->copy_done, 0));
}

void state_store_async(hq_state_s* s, void* host) {
    state_canonicalize(s);
    Context& c = ctx();
    if (!c.copy_stream) HQ_CHECK_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    if (!s->ready) HQ_CHECK_CUDA(cudaEventCreateWithFlags(&s->ready, cudaEventDisableTiming));
    if (!s->copy_done) HQ_CHECK_CUDA(cudaEventCreateWithFlags(&s->copy_done, cudaEventDisableTiming));
    HQ_CHECK_CUDA(cudaEventRecord(s->ready, c.stream));
    HQ_CHECK_CUDA(cudaStreamWaitEvent(c.copy_stream, s->ready, 0));
    void* mapped = nullptr;
    {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost)
            mapped = a.devicePointer;
        else
            cudaGetLastError();
    }
    if (mapped && s->bytes >= (size_t(64) << 20) && s->bytes % 16 == 0) {
        // pinned and large: a copy kernel on a few SMs, so that the next
        // circuit's kernels run beside it on the others.  The host link sets
        // its rate: on GB300 4 blocks of 512 threads write 182 GB/s to pinned
        // memory, 8 190 GB/s, 12 or more 193 GB/s (the copy engine's rate);
        // 4 keep 148 SMs for the next circuit and an 8 GiB state still lands
        // within one 30-qubit circuit's run.
        const int ctas = std::min(c.sm_count, 4);
        launch_readback(s->d, mapped, s->bytes, ctas, c.copy_stream);
        HQ_CHECK_CUDA(cudaEventRecord(s->copy_done, c.copy_stream));
        if (!c.rb_done) HQ_CHECK_CUDA(cudaEventCreateWithFlags(&c.rb_done, cudaEventDisableTiming));
        HQ_CHECK_CUDA(cudaEventRecord(c.rb_done, c.copy_stream));
        c.rb_sms = ctas;
    } else {
        // 256 MiB per copy: large states go out as a queue of moderate copies
        // rather than one multi-GiB transfer
        constexpr size_t kChunk = size_t(256) << 20;
        for (size_t off = 0; off < s->bytes; off += kChunk) {
            const size_t len = s->bytes - off < kChunk ? s->bytes - off : kChunk;
            HQ_CHECK_CUDA(cudaMemcpyAsync((char*)host + off, (const char*)s->d + off, len,
                                          cudaMemcpyDeviceToHost, c.copy_stream));
        }
        HQ_CHECK_CUDA(cudaEventRecord(s->copy_done, c.copy_stream));
    }
    s->copy_pending = true;
}

void state_wait_host(hq_state_s* s) {
    if (!s->copy_pending) return;
    HQ_CHECK_CUDA(cudaEventSynchronize(s->copy_done));
    s->copy_pending = false;
}

void state_canonicalize(hq_state_s* s) {
    std::vector<int> id(s->n);
    for (int q = 0; q < s->n; q++) id[q] = q;
    state_remap(s, id);
}

void state_gather(hq_state_s* s, const uint64_t* idx, int64_t count, float* out) {
    const int n = s->n;
    std::vector<uint64_t> phys(count);
    for (int64_t i = 0; i < count; i++) {
        HQ_REQUIRE(n >= 64 || idx[i] < (uint64_t(1) << n), HQ_ERR_INVALID,
                   "amplitude index %llu out of range", (unsigned long long)idx[i]);
        uint64_t p = 0;
        for (int q = 0; q < n; q++)
            if ((idx[i] >> q) & 1) p |= uint64_t(1) << s->pos[q];
        phys[i] = p;
    }
    cudaStream_t st = ctx().stream;
    const size_t ib = sizeof(uint64_t) * count, ob = sizeof(float) * 2 * count;
    char* buf = (char*)dev_alloc_ordered(ib + ob);
    try {
        HQ_CHECK_CUDA(cudaMemcpyAsync(buf, phys.data(), ib, cudaMemcpyHostToDevice, st));
        launch_gather(s->d, (const uint64_t*)buf, count, buf + ib, st);
        HQ_CHECK_CUDA(cudaMemcpyAsync(out, buf + ib, ob, cudaMemcpyDeviceToHost, st));
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        dev_free_ordered(buf, ib + ob);
        throw;
    }
    dev_free_ordered(buf, ib + ob);
}

void state_marginals(hq_state_s* s, double* h) {
    launch_marginals(s->d, s->n, s->d_scratch, s->scratch_doubles, h, ctx().stream);
}

// ---- plain path ------------------------------------------------------------------

static PlainGate lower_plain(const hq_gate& g, const std::vector<int>& pos) {
    PlainGate p;
    std::memset(&p, 0, sizeof(p));
    p.target = pos[g.target];
    int ins[3], ni = 0;
    ins[ni++] = p.target;
    if (g.control >= 0) {
        ins[ni++] = pos[g.control];
        p.setmask |= uint64_t(1) << pos[g.control];
    }
    if (g.control2 >= 0) {
        ins[ni++] = pos[g.control2];
        p.setmask |= uint64_t(1) << pos[g.control2];
    }
    std::sort(ins, ins + ni);
    p.ninsert = ni;
    for (int i = 0; i < ni; i++) p.insert[i] = ins[i];
    for (int i = 0; i < 8; i++) p.m[i] = (float)g.mat[i];
    if (is_x_like(g))
        p.kind = PK_SWAP;
    else if (matrix_is_diagonal(g))
        p.kind = (g.mat[0] == 1.0 && g.mat[1] == 0.0) ? PK_DIAG_HI : PK_DIAG;
    else
        p.kind = PK_GENERAL;
    return p;
}

void state_sample(hq_state_s* s, int shots, uint64_t seed, uint64_t* out) {
    HQ_REQUIRE(shots >= 0, HQ_ERR_INVALID, "negative shot count");
    // the inverse CDF runs in logical index order, so draws do not depend on the layout
    state_canonicalize(s);
    const int n = s->n;
    const size_t nb = sample_scratch_doubles(n);
    const size_t bytes = sizeof(double) * nb + sizeof(uint64_t) * size_t(std::max(shots, 1));
    char* buf = (char*)dev_alloc_ordered(bytes);
    cudaStream_t st = ctx().stream;
    std::vector<uint64_t> phys(size_t(std::max(shots, 1)));
    double total = 0.0;
    try {
        double* cdf = (double*)buf;
        uint64_t* d_out = (uint64_t*)(buf + sizeof(double) * nb);
        launch_sample(s->d, n, shots, seed, cdf, d_out, st);
        HQ_CHECK_CUDA(cudaMemcpyAsync(&total, cdf + nb - 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (shots > 0)
            HQ_CHECK_CUDA(cudaMemcpyAsync(phys.data(), d_out, sizeof(uint64_t) * shots,
                                          cudaMemcpyDeviceToHost, st));
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        dev_free_ordered(buf, bytes);
        throw;
    }
    dev_free_ordered(buf, bytes);
    HQ_REQUIRE(total > 0.0, HQ_ERR_STATE, "sample: the state has zero norm");
    for (int i = 0; i < shots; i++) {
        uint64_t l = 0;
        for (int q = 0; q < n; q++)
            if ((phys[i] >> s->pos[q]) & 1) l |= uint64_t(1) << q;
        out[i] = l;
    }
}

void apply_plain(hq_state_s* s, const std::vector<hq_gate>& gates) {
    cudaStream_t st = ctx().stream;
    for (const hq_gate& g : gates) {
        validate_gate(g, s->n);
        if (g.type == G_SWAP) {
            // exchange the two qubits' physical positions in the layout (no data pass)
            std::swap(s->pos[g.target], s->pos[g.control]);
            continue;
        }
        launch_plain_gate(s->d, s->n, lower_plain(g, s->pos), st);
    }
}

void apply_oshm_group(hq_state_s* s, const std::vector<hq_gate>& gates, uint64_t tile_logical) {
    const int n = s->n;
    std::vector<hq_gate> phys;
    for (const hq_gate& g0 : gates) {
        validate_gate(g0, n);
        HQ_REQUIRE(g0.type != G_SWAP, HQ_ERR_INVALID, "oshm group: SWAP not allowed");
        hq_gate g = g0;
        g.target = s->pos[g0.target];
        if (g0.control >= 0) g.control = s->pos[g0.control];
        if (g0.control2 >= 0) g.control2 = s->pos[g0.control2];
        phys.push_back(g);
    }
    uint64_t tile = 0;
    for (int q = 0; q < n; q++)
        if ((tile_logical >> q) & 1) tile |= uint64_t(1) << s->pos[q];
    OshmProgram prog = plan_oshm(n, phys, tile);
    // ops start on a 256-byte boundary: OshmOp holds 64-bit fields
    const size_t pb = (sizeof(OshmPhase) * std::max<size_t>(1, prog.phases.size()) + 255) & ~size_t(255);
    const size_t ob = sizeof(OshmOp) * std::max<size_t>(1, prog.ops.size());
    char* buf = (char*)dev_alloc_ordered(pb + ob);
    cudaStream_t st = ctx().stream;
    try {
        HQ_CHECK_CUDA(cudaMemcpyAsync(buf, prog.phases.data(), sizeof(OshmPhase) * prog.phases.size(),
                                      cudaMemcpyHostToDevice, st));
        HQ_CHECK_CUDA(cudaMemcpyAsync(buf + pb, prog.ops.data(), sizeof(OshmOp) * prog.ops.size(),
                                      cudaMemcpyHostToDevice, st));
        OshmLaunch p = make_oshm_launch(prog, s->d, (const OshmPhase*)buf, (const OshmOp*)(buf + pb),
                                        ctx().d_error);
        launch_oshm(p, st);
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        dev_free_ordered(buf, pb + ob);
        throw;
    }
    dev_free_ordered(buf, pb + ob);
    check_device_error();
}

// ---- circuits ---------------------------------------------------------------------

// Every background compile is registered here.  A released circuit does not
// wait for its kernels (they still land in the process-wide cache); finished
// jobs are dropped at the next registration or release, and the ones still
// running are joined by an exit hook registered with atexit when the first
// job starts -- after the CUDA runtime's own registration, so it runs before
// the runtime tears down.
struct JobRegistry {
    std::mutex mu;
    std::vector<std::shared_ptr<JitJob>> jobs;
    void prune() {
        std::lock_guard<std::mutex> lk(mu);
        for (size_t i = 0; i < jobs.size();) {
            bool done;
            {
                std::lock_guard<std::mutex> jl(jobs[i]->mu);
                done = jobs[i]->done;
            }
            if (done) {
                jobs[i]->join();
                jobs.erase(jobs.begin() + i);
            } else {
                i++;
            }
        }
    }
};
JobRegistry g_jobs;

void join_background_compiles() {
    std::vector<std::shared_ptr<JitJob>> jobs;
    {
        std::lock_guard<std::mutex> lk(g_jobs.mu);
        jobs.swap(g_jobs.jobs);
    }
    for (auto& j : jobs) j->join();
}

void circuit_release(hq_circuit_s* c) {
    c->jit_job.reset();  // the registry keeps it until it is done
    g_jobs.prune();
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_state = nullptr;
    if (c->d_phases) dev_free_ordered(c->d_phases, c->phases_bytes);
    if (c->d_ops) dev_free_ordered(c->d_ops, c->ops_bytes);
    if (c->d_umats) dev_free_ordered(c->d_umats, c->umats_bytes);
    if (c->d_mm_scratch) dev_free_ordered(c->d_mm_scratch, c->mm_scratch_bytes);
    c->d_phases = nullptr;
    c->d_ops = nullptr;
    c->d_umats = nullptr;
    c->d_mm_scratch = nullptr;
    c->phases_bytes = c->ops_bytes = c->umats_bytes = c->mm_scratch_bytes = 0;
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    c->ev0 = c->ev1 = nullptr;
    c->dgroups.clear();
    c->compiled = false;
}

CompileConfig config_from_options(const hq_compile_options& o, int n) {
    CompileConfig cfg;
    cfg.backend = o.backend;
    cfg.reference = o.reference_grouping != 0;
    cfg.tile = o.tile_qubits > 0 ? o.tile_qubits : 13;
    cfg.tile_auto = o.tile_qubits == 0;
    cfg.coalesce = o.coalesce > 0 ? o.coalesce : 3;
    // tensor-core passes cost the same at 6 and 7 qubits (measured), so the
    // wider group is the default there; FP32 SIMT doubles its cost per qubit
    cfg.mm_qubits = o.mm_qubits > 0 ? o.mm_qubits : (o.mm_precision == HQ_MM_FP32 ? 6 : 7);
    cfg.mm_precision = o.mm_precision;
    HQ_REQUIRE(o.backend == HQ_BACKEND_PLAIN || o.backend == HQ_BACKEND_OSHM ||
                   o.backend == HQ_BACKEND_TRANSMM || o.backend == HQ_BACKEND_HYBRID,
               HQ_ERR_INVALID, "unknown backend %d", o.backend);
    HQ_REQUIRE(cfg.tile >= 6 && cfg.tile <= OSHM_MAX_K, HQ_ERR_INVALID,
               "tile_qubits %d out of range [6,%d]", cfg.tile, OSHM_MAX_K);
    HQ_REQUIRE(cfg.mm_qubits >= 1 && cfg.mm_qubits <= 8, HQ_ERR_INVALID,
               "mm_qubits %d out of range [1,8]", cfg.mm_qubits);
    HQ_REQUIRE(o.mm_precision >= HQ_MM_BF16X3 && o.mm_precision <= HQ_MM_FP32, HQ_ERR_INVALID,
               "unknown TransMM precision %d", o.mm_precision);
    HQ_REQUIRE(cfg.coalesce >= 1, HQ_ERR_INVALID, "coalesce must be >= 1");
    HQ_REQUIRE(o.specialize >= 0 && o.specialize <= 3, HQ_ERR_INVALID, "specialize %d outside [0,3]",
               o.specialize);
    cfg.tile = std::min(cfg.tile, n);
    return cfg;
}

uint64_t oshm_tile_mask(const GroupPlan& gp, int n) {
    // the group's related qubits (they include the coalesced low qubits, so
    // physical qubit 0) padded with the lowest free qubits to the tile width
    uint64_t tile = pad_tile(gp.related | 1, gp.width, n);
    HQ_REQUIRE(__builtin_popcountll(tile) == gp.width, HQ_ERR_INVALID,
               "oshm: related set wider than the tile (%d > %d)", __builtin_popcountll(tile),
               gp.width);
    return tile;
}

void circuit_plan(hq_circuit_s* c, const hq_compile_options& o) {
    const int n = c->n;
    c->opt = o;
    // SWAP folding: drop swaps, relabel the gates after them
    std::vector<int> perm;
    c->folded = fold_swaps(c->gates, n, perm);
    c->swap_perm = perm;
    c->orig_index.clear();
    for (size_t i = 0; i < c->gates.size(); i++)
        if (c->gates[i].type != G_SWAP) c->orig_index.push_back((int)i);
    if (o.specialize == 0 && o.backend != HQ_BACKEND_PLAIN && !o.reference_grouping) {
        // interpreted kernels pay per op: fuse runs of single-qubit gates (a
        // fused gate is listed in its group by its first gate)
        std::vector<int> origin;
        c->folded = fuse_single_qubit_runs(c->folded, n, &origin);
        std::vector<int> idx;
        for (int x : origin) idx.push_back(c->orig_index[x]);
        c->orig_index.swap(idx);
    }

    CompileConfig cfg = config_from_options(o, n);
    if (o.backend == HQ_BACKEND_PLAIN || n < 6) {
        // one launch per gate; small registers always take this path
        c->part = Partition();
        c->part.final_pos.resize(n);
        for (int q = 0; q < n; q++) c->part.final_pos[q] = q;
        return;
    }
    std::vector<int> id(n);
    for (int q = 0; q < n; q++) id[q] = q;
    c->part = partition(n, c->folded, id, cfg);
}

void circuit_lower(hq_circuit_s* c) {
    const int n = c->n;
    const hq_compile_options& o = c->opt;
    if (o.backend == HQ_BACKEND_PLAIN || n < 6) {
        c->compiled = true;
        return;
    }
    CompileConfig cfg = config_from_options(o, n);
    std::vector<OshmPhase> phases;
    std::vector<OshmOp> ops;
    std::vector<double> umats;
    for (const GroupPlan& gp : c->part.groups) {
        DeviceGroup dg;
        dg.backend = gp.backend;
        // execution keeps the identity layout: a group's gates act on their
        // qubits in place (TransMM gathers its rows, no transpose pass)
        for (int x : gp.gates) dg.phys_gates.push_back(c->folded[x]);
        if (gp.backend == HQ_BACKEND_OSHM) {
            dg.prog = plan_oshm(n, dg.phys_gates, oshm_tile_mask(gp, n));
            dg.phase_off = phases.size();
            dg.op_off = ops.size();
            for (auto ph : dg.prog.phases) {
                ph.op_begin += (uint32_t)dg.op_off;
                ph.op_end += (uint32_t)dg.op_off;
                phases.push_back(ph);
            }
            ops.insert(ops.end(), dg.prog.ops.begin(), dg.prog.ops.end());
        } else {
            transmm_prepare(n, gp, dg, cfg, umats);
        }
        c->dgroups.push_back(std::move(dg));
    }
    cudaStream_t st = ctx().stream;
    if (!phases.empty()) {
        c->phases_bytes = sizeof(OshmPhase) * phases.size();
        c->d_phases = (OshmPhase*)dev_alloc_ordered(c->phases_bytes);
        HQ_CHECK_CUDA(cudaMemcpyAsync(c->d_phases, phases.data(), c->phases_bytes,
                                      cudaMemcpyHostToDevice, st));
    }
    if (!ops.empty()) {
        c->ops_bytes = sizeof(OshmOp) * ops.size();
        c->d_ops = (OshmOp*)dev_alloc_ordered(c->ops_bytes);
        HQ_CHECK_CUDA(cudaMemcpyAsync(c->d_ops, ops.data(), c->ops_bytes, cudaMemcpyHostToDevice, st));
    }
    if (!umats.empty()) {
        c->umats_bytes = sizeof(double) * umats.size();
        c->d_umats = (double*)dev_alloc_ordered(c->umats_bytes);
        HQ_CHECK_CUDA(cudaMemcpyAsync(c->d_umats, umats.data(), c->umats_bytes,
                                      cudaMemcpyHostToDevice, st));
    }
    transmm_finalize(c);
    HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    c->specialized = false;
    c->specialize_note.clear();
    if (o.specialize != 0) {
        std::vector<const OshmProgram*> progs;
        std::vector<size_t> idx;
        for (size_t i = 0; i < c->dgroups.size(); i++)
            if (c->dgroups[i].backend == HQ_BACKEND_OSHM) {
                progs.push_back(&c->dgroups[i].prog);
                idx.push_back(i);
            }
        if (!progs.empty()) {
            std::vector<JitKernel> ks;
            try {
                HQ_REQUIRE(jit_available(), HQ_ERR_UNSUPPORTED, "NVRTC not available");
                if (o.specialize != 3 || jit_lookup_cached(progs, ks)) {
                    if (ks.empty()) ks = jit_compile_groups(progs);
                    for (size_t i = 0; i < idx.size(); i++) {
                        c->dgroups[idx[i]].jit = ks[i];
                        c->dgroups[idx[i]].has_jit = true;
                    }
                    c->specialized = true;
                } else {
                    // background mode, kernels not compiled yet: compile them on a
                    // host thread; until they are in, the interpreter runs the groups
                    static std::once_flag exit_hook;
                    std::call_once(exit_hook, [] { std::atexit(join_background_compiles); });
                    auto job = std::make_shared<JitJob>();
                    for (const OshmProgram* pr : progs) job->progs.push_back(*pr);
                    job->groups = idx;
                    std::shared_ptr<JitJob> keep = job;
                    job->th = std::thread([keep] {
                        JitJob* jp = keep.get();
                        std::vector<const OshmProgram*> ps;
                        for (const OshmProgram& pr : jp->progs) ps.push_back(&pr);
                        std::vector<JitKernel> out;
                        std::string err;
                        try {
                            out = jit_compile_groups(ps);
                        } catch (const std::exception& e) {
                            err = e.what();
                        }
                        std::lock_guard<std::mutex> lk(jp->mu);
                        jp->kernels = out;
                        jp->err = err;
                        jp->done = true;
                    });
                    g_jobs.prune();
                    {
                        std::lock_guard<std::mutex> lk(g_jobs.mu);
                        g_jobs.jobs.push_back(job);
                    }
                    c->jit_job = job;
                }
            } catch (const Failure& f) {
                if (o.specialize == 1) throw;
                c->specialize_note = f.what();  // auto mode: the interpreter runs these groups
            }
        }
    }
    c->compiled = true;
}

void circuit_jit_install(hq_circuit_s* c, bool wait) {
    std::shared_ptr<JitJob> job = c->jit_job;
    if (!job) return;
    {
        std::lock_guard<std::mutex> lk(job->mu);
        if (!job->done && !wait) return;
    }
    job->join();
    c->jit_job.reset();
    if (!job->err.empty() || job->kernels.size() != job->groups.size()) {
        c->specialize_note = job->err.empty() ? "specialisation failed" : job->err;
        return;
    }
    for (size_t i = 0; i < job->groups.size(); i++) {
        c->dgroups[job->groups[i]].jit = job->kernels[i];
        c->dgroups[job->groups[i]].has_jit = true;
    }
    c->specialized = true;
    // a graph captured meanwhile holds interpreter launches: capture again later
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
        c->graph_state = nullptr;
    }
}

void circuit_compile(hq_circuit_s* c, const hq_compile_options& o) {
    circuit_release(c);
    ensure_init();
    circuit_plan(c, o);
    circuit_lower(c);
}

void circuit_launch_groups(hq_circuit_s* c, void* state, cudaStream_t st) {
    for (const DeviceGroup& dg : c->dgroups) {
        if (dg.backend == HQ_BACKEND_OSHM && dg.has_jit) {
            jit_launch(dg.jit, state, uint64_t(1) << (c->n - dg.prog.k), ctx().d_error, st);
        } else if (dg.backend == HQ_BACKEND_OSHM) {
            OshmLaunch p = make_oshm_launch(dg.prog, state, c->d_phases + dg.phase_off,
                                            c->d_ops, ctx().d_error);
            launch_oshm(p, st);
        } else {
            transmm_launch(c, dg, state, st);
        }
    }
}

double circuit_run(hq_circuit_s* c, hq_state_s* s, bool sync) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    HQ_REQUIRE(s->n == c->n, HQ_ERR_INVALID, "state has %d qubits, circuit %d", s->n, c->n);
    cudaStream_t st = ctx().stream;
    state_canonicalize(s);
    if (!c->ev0) {
        HQ_CHECK_CUDA(cudaEventCreate(&c->ev0));
        HQ_CHECK_CUDA(cudaEventCreate(&c->ev1));
    }
    circuit_jit_install(c, false);
    HQ_CHECK_CUDA(cudaEventRecord(c->ev0, st));
    if (c->graph && c->graph_state == s) {
        HQ_CHECK_CUDA(cudaGraphLaunch(c->graph, st));
    } else if (c->opt.backend == HQ_BACKEND_PLAIN || c->n < 6) {
        apply_plain(s, c->folded);
    } else {
        circuit_launch_groups(c, s->d, st);
    }
    HQ_CHECK_CUDA(cudaEventRecord(c->ev1, st));
    for (int q = 0; q < c->n; q++) s->pos[q] = c->swap_perm[q];
    if (!sync) return 0.0;
    HQ_CHECK_CUDA(cudaEventSynchronize(c->ev1));
    check_device_error();
    float ms = 0.f;
    HQ_CHECK_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    return double(ms) * 1000.0;
}

// A run that also leaves the final state, in logical order, at `host` (the
// reference's run followed by its full-state readback, src/circuit.cpp:46-62).
// When the last group is a generated kernel, the run ends in the canonical
// layout and `host` is pinned, that group writes every finished amplitude to
// HBM and to `host` (one pass, no separate copy); otherwise the run is
// followed by a copy.  Returns the device time of the run including the
// readback, in microseconds.
double circuit_run_to_host(hq_circuit_s* c, hq_state_s* s, void* host) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    HQ_REQUIRE(s->n == c->n, HQ_ERR_INVALID, "state has %d qubits, circuit %d", s->n, c->n);
    circuit_jit_install(c, false);
    bool fused = c->opt.backend != HQ_BACKEND_PLAIN && c->n >= 6 && !c->dgroups.empty() &&
                 c->dgroups.back().backend == HQ_BACKEND_OSHM && c->dgroups.back().has_jit;
    for (int q = 0; fused && q < c->n; q++) fused = c->swap_perm[q] == q;
    void* dhost = nullptr;
    if (fused) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer != nullptr)
            dhost = a.devicePointer;
        else
            cudaGetLastError();  // not pinned: the copy path below
        fused = dhost != nullptr;
    }
    cudaStream_t st = ctx().stream;
    if (!fused) {
        circuit_run(c, s, false);
        state_canonicalize(s);
        HQ_CHECK_CUDA(cudaMemcpyAsync(host, s->d, s->bytes, cudaMemcpyDeviceToHost, st));
        HQ_CHECK_CUDA(cudaEventRecord(c->ev1, st));
        HQ_CHECK_CUDA(cudaEventSynchronize(c->ev1));
        check_device_error();
        float ms = 0.f;
        HQ_CHECK_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        return double(ms) * 1000.0;
    }
    state_canonicalize(s);
    if (!c->ev0) {
        HQ_CHECK_CUDA(cudaEventCreate(&c->ev0));
        HQ_CHECK_CUDA(cudaEventCreate(&c->ev1));
    }
    HQ_CHECK_CUDA(cudaEventRecord(c->ev0, st));
    const size_t ng = c->dgroups.size();
    for (size_t g = 0; g < ng; g++) {
        const DeviceGroup& dg = c->dgroups[g];
        if (g + 1 == ng) {
            jit_launch(dg.jit, s->d, uint64_t(1) << (c->n - dg.prog.k), ctx().d_error, st, dhost);
        } else if (dg.backend == HQ_BACKEND_OSHM && dg.has_jit) {
            jit_launch(dg.jit, s->d, uint64_t(1) << (c->n - dg.prog.k), ctx().d_error, st);
        } else if (dg.backend == HQ_BACKEND_OSHM) {
            OshmLaunch p = make_oshm_launch(dg.prog, s->d, c->d_phases + dg.phase_off, c->d_ops,
                                            ctx().d_error);
            launch_oshm(p, st);
        } else {
            transmm_launch(c, dg, s->d, st);
        }
    }
    HQ_CHECK_CUDA(cudaEventRecord(c->ev1, st));
    for (int q = 0; q < c->n; q++) s->pos[q] = c->swap_perm[q];
    HQ_CHECK_CUDA(cudaEventSynchronize(c->ev1));
    check_device_error();
    float ms = 0.f;
    HQ_CHECK_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    return double(ms) * 1000.0;
}

void circuit_predict(const hq_circuit_s* c, double* group_us) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    for (size_t g = 0; g < c->dgroups.size(); g++) {
        const DeviceGroup& dg = c->dgroups[g];
        if (dg.backend == HQ_BACKEND_OSHM)
            group_us[g] = cost_oshm(c->n, (int)dg.prog.phases.size(), dg.phys_gates, dg.prog.k) * 1e6;
        else
            group_us[g] = cost_transmm(c->n, dg.mm_m, dg.mm_precision) * 1e6;
    }
}

void circuit_profile(hq_circuit_s* c, hq_state_s* s, double* group_us) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    circuit_jit_install(c, false);
    HQ_REQUIRE(s->n == c->n, HQ_ERR_INVALID, "state/circuit size mismatch");
    HQ_REQUIRE(c->opt.backend != HQ_BACKEND_PLAIN && c->n >= 6, HQ_ERR_STATE,
               "plain-path circuits have no groups to profile");
    cudaStream_t st = ctx().stream;
    state_canonicalize(s);
    const size_t ng = c->dgroups.size();
    std::vector<cudaEvent_t> ev(ng + 1);
    for (auto& e : ev) HQ_CHECK_CUDA(cudaEventCreate(&e));
    HQ_CHECK_CUDA(cudaEventRecord(ev[0], st));
    for (size_t g = 0; g < ng; g++) {
        const DeviceGroup& dg = c->dgroups[g];
        if (dg.backend == HQ_BACKEND_OSHM && dg.has_jit) {
            jit_launch(dg.jit, s->d, uint64_t(1) << (c->n - dg.prog.k), ctx().d_error, st);
        } else if (dg.backend == HQ_BACKEND_OSHM) {
            OshmLaunch p = make_oshm_launch(dg.prog, s->d, c->d_phases + dg.phase_off, c->d_ops,
                                            ctx().d_error);
            launch_oshm(p, st);
        } else {
            transmm_launch(c, dg, s->d, st);
        }
        HQ_CHECK_CUDA(cudaEventRecord(ev[g + 1], st));
    }
    HQ_CHECK_CUDA(cudaEventSynchronize(ev[ng]));
    for (size_t g = 0; g < ng; g++) {
        float ms = 0.f;
        HQ_CHECK_CUDA(cudaEventElapsedTime(&ms, ev[g], ev[g + 1]));
        group_us[g] = double(ms) * 1000.0;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int q = 0; q < c->n; q++) s->pos[q] = c->swap_perm[q];
    check_device_error();
}

void circuit_capture(hq_circuit_s* c, hq_state_s* s) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    HQ_REQUIRE(s->n == c->n, HQ_ERR_INVALID, "state/circuit size mismatch");
    const bool plain = c->opt.backend == HQ_BACKEND_PLAIN || c->n < 6;
    cudaStream_t st = ctx().stream;
    circuit_jit_install(c, true);  // a graph holds the generated kernels
    // runs start from the canonical layout, so the captured launches (plain
    // gates are lowered through the layout) are the ones every run makes
    state_canonicalize(s);
    HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    HQ_CHECK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        if (plain)
            apply_plain(s, c->folded);  // one kernel node per gate
        else
            circuit_launch_groups(c, s->d, st);
    } catch (...) {
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    HQ_CHECK_CUDA(cudaStreamEndCapture(st, &g));
    cudaError_t e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    HQ_REQUIRE(e == cudaSuccess, HQ_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    c->graph_state = s;
}

}  // namespace hq
