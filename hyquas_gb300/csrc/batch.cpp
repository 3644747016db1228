// Batched execution: many circuits, one persistent launch (k_oshm_batch).
//
// The reference simulates one circuit per process (src/circuit.cpp:16-71,
// src/main.cpp:12-230); it has no batching.  Here every circuit of a batch is
// partitioned into OShareMem groups with the same grouping and lowering as a
// single compiled circuit (compiler.cpp), the group programs of all circuits
// are concatenated into one device program, and a work queue of
// (circuit, group, tile range) items is built group level by group level.
// Persistent blocks take items in queue order; an item of group g waits
// (bounded) until every tile of groups < g of its circuit is written.
#include <algorithm>
#include <queue>
#include <cstring>

#include "batch.h"
#include "common.h"
#include "gates.h"

namespace hq {

namespace {

// Estimated device seconds of one circuit planned with tile width k: the
// refitted per-pass cost of every group plus a per-item dispatch overhead
// spread over the resident blocks.
double batch_cost(const Partition& part, const std::vector<hq_gate>& gates, int n, int k,
                  int slots) {
    const double kItemSec = 1.5e-6;
    double t = 0;
    for (const GroupPlan& gp : part.groups) {
        std::vector<hq_gate> gs;
        for (int x : gp.gates) gs.push_back(gates[x]);
        t += cost_oshm(n, 0, gs, k) - 4e-6;  // no launch per group
    }
    const double items = double(part.groups.size()) * double(uint64_t(1) << (n - k));
    return t + items * kItemSec / std::max(1, slots);
}

}  // namespace

// Tiles per work item: an eighth of a circuit's tiles, at most 16 (1 MiB of
// amplitudes).  The items of every circuit of a level interleave, so even the
// largest circuits need not be split per block; fewer, larger items spend
// less on the item queue and the dependency counters (512 RY/RZ+CZ circuits:
// 48,089 items in 133.9 ms against 514,785 one-tile items in 148.7 ms).
uint32_t batch_chunk_tiles(uint64_t tiles, int slots) {
    (void)slots;
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(tiles / 8, 1), 16);
}

void batch_release(hq_batch_s* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    dev_free(b->d_program, b->program_bytes);
    b->d_program = nullptr;
    b->program_bytes = 0;
    b->compiled = false;
}

void batch_compile(hq_batch_s* b, const hq_compile_options* opt) {
    ensure_init();
    batch_release(b);
    const int fixed_k = opt ? opt->tile_qubits : 0;
    HQ_REQUIRE(fixed_k == 0 || (fixed_k >= kBatchMinTile && fixed_k <= kBatchTile), HQ_ERR_INVALID,
               "batch: tile width %d outside [%d, %d]", fixed_k, kBatchMinTile, kBatchTile);
    const int slots = oshm_batch_slots();
    b->slots = slots;

    std::vector<OshmProgram> progs;
    std::vector<uint32_t> prog_circuit;
    b->num_groups = 0;
    b->pass_bytes = 0;
    for (BatchEntry& e : b->entries) {
        const int n = e.n;
        std::vector<int> perm;
        // the batched kernel interprets its ops: fewer, fused ops run faster
        e.folded = fuse_single_qubit_runs(fold_swaps(e.gates, n, perm), n);
        e.swap_perm = perm;
        e.group0 = (uint32_t)progs.size();
        e.ngroups = 0;
        e.k = 0;
        if (n < kBatchMinTile || e.folded.empty()) continue;  // gate by gate / init only
        std::vector<int> id(n);
        for (int q = 0; q < n; q++) id[q] = q;
        CompileConfig cfg;
        cfg.backend = HQ_BACKEND_OSHM;
        cfg.coalesce = opt && opt->coalesce > 0 ? opt->coalesce : 3;
        Partition best;
        double best_cost = 1e300;
        const int kmax = std::min(n, kBatchTile);
        const int kmin = fixed_k ? std::min(fixed_k, kmax) : kBatchMinTile;
        for (int k = fixed_k ? kmin : kmax; k >= kmin; k--) {
            cfg.tile = k;
            cfg.coalesce = std::min(cfg.coalesce, k);
            Partition part = partition(n, e.folded, id, cfg);
            const double c = batch_cost(part, e.folded, n, k, slots);
            if (c < best_cost) {
                best_cost = c;
                best = std::move(part);
                e.k = k;
            }
        }
        for (const GroupPlan& gp : best.groups) {
            std::vector<hq_gate> phys;
            for (int x : gp.gates) phys.push_back(e.folded[x]);
            OshmProgram prog = plan_oshm(n, phys, oshm_tile_mask(gp, n));
            HQ_REQUIRE(prog.k == e.k && prog.r == 5, HQ_ERR_UNSUPPORTED,
                       "batch: group planned with tile %d/%d registers", prog.k, prog.r);
            progs.push_back(std::move(prog));
            prog_circuit.push_back(uint32_t(&e - b->entries.data()));
            e.ngroups++;
        }
        b->num_groups += e.ngroups;
        b->pass_bytes += uint64_t(e.ngroups) * 16ull * (uint64_t(1) << n);
    }

    // one device program: groups | items | phases | ops | counters
    std::vector<OshmPhase> phases;
    std::vector<OshmOp> ops;
    std::vector<size_t> phase_off(progs.size());
    for (size_t i = 0; i < progs.size(); i++) {
        phase_off[i] = phases.size();
        const uint32_t o = (uint32_t)ops.size();
        for (OshmPhase ph : progs[i].phases) {
            ph.op_begin += o;
            ph.op_end += o;
            phases.push_back(ph);
        }
        ops.insert(ops.end(), progs[i].ops.begin(), progs[i].ops.end());
    }
    // Item order: a list schedule of the launch simulated on the host.  The
    // device hands items out in queue order, and an item whose circuit's
    // previous group is not finished makes its block wait; so the queue is the
    // order in which `slots` workers would start the items if each item ran
    // for its estimated time (tiles x the group's ops and phases), an item
    // becoming ready when every item of its circuit's previous group has
    // finished, and a free worker taking the ready item of the circuit with
    // the most estimated work left (its critical path).  An item is queued
    // only after all its predecessors (they finished first in the
    // simulation), so the bounded waits always end.
    std::vector<BatchItem> items;
    {
        struct Level {
            uint32_t circuit, group;
            uint64_t tiles;
            uint32_t chunk;
            double item_t;  // estimated time of one item (arbitrary units)
        };
        std::vector<std::vector<Level>> lv(b->entries.size());
        std::vector<double> left(b->entries.size(), 0.0);
        for (uint32_t ci = 0; ci < b->entries.size(); ci++) {
            const BatchEntry& e = b->entries[ci];
            const uint64_t tiles = e.ngroups ? uint64_t(1) << (e.n - e.k) : 0;
            HQ_REQUIRE(tiles * e.ngroups < (uint64_t(1) << 32), HQ_ERR_UNSUPPORTED,
                       "batch: circuit %u has too many tiles for the 32-bit item counters", ci);
            for (uint32_t g = 0; g < e.ngroups; g++) {
                const OshmProgram& pr = progs[e.group0 + g];
                const uint32_t ch = batch_chunk_tiles(tiles, slots);
                const double per_tile = 8.0 + double(pr.ops.size()) + 4.0 * double(pr.phases.size());
                lv[ci].push_back({ci, g, tiles, ch, per_tile * double(ch) * double(1u << e.k) / 8192.0});
                left[ci] += per_tile * double(tiles) * double(1u << e.k) / 8192.0 / double(slots);
            }
        }
        // ready queue: (priority = estimated work left, circuit, next item of its level)
        using Ready = std::pair<double, uint32_t>;
        std::priority_queue<Ready> ready;
        std::vector<uint32_t> level_of(b->entries.size(), 0);
        std::vector<uint64_t> next_tile(b->entries.size(), 0), done_items(b->entries.size(), 0);
        for (uint32_t ci = 0; ci < b->entries.size(); ci++)
            if (!lv[ci].empty()) ready.push({left[ci], ci});
        // workers: (time free, worker); running items finish events
        using Fin = std::pair<double, uint32_t>;  // (finish time, circuit)
        std::priority_queue<Fin, std::vector<Fin>, std::greater<Fin>> running;
        double now = 0.0;
        int busy = 0;
        auto level_items = [&](uint32_t ci) {
            const Level& L = lv[ci][level_of[ci]];
            return (L.tiles + L.chunk - 1) / L.chunk;
        };
        while (!ready.empty() || !running.empty()) {
            while (busy < slots && !ready.empty()) {
                const uint32_t ci = ready.top().second;
                ready.pop();
                const Level& L = lv[ci][level_of[ci]];
                const uint64_t u = next_tile[ci];
                BatchItem it;
                it.group = b->entries[ci].group0 + L.group;
                it.circuit = ci;
                it.tile0 = (uint32_t)u;
                it.count = (uint32_t)std::min<uint64_t>(L.chunk, L.tiles - u);
                it.need = (uint32_t)(L.group * L.tiles);
                it.flags = L.group == 0 ? ITEM_FIRST : 0;
                items.push_back(it);
                next_tile[ci] = u + it.count;
                running.push({now + L.item_t, ci});
                busy++;
                if (next_tile[ci] < L.tiles) ready.push({left[ci], ci});  // more of this level
            }
            if (running.empty()) break;
            const Fin f = running.top();
            running.pop();
            now = f.first;
            busy--;
            const uint32_t ci = f.second;
            left[ci] = std::max(0.0, left[ci] - lv[ci][level_of[ci]].item_t / double(slots));
            if (++done_items[ci] == level_items(ci)) {  // the level is complete: the next one is ready
                done_items[ci] = 0;
                next_tile[ci] = 0;
                if (++level_of[ci] < lv[ci].size()) ready.push({left[ci], ci});
            }
        }
    }
    b->num_items = items.size();
    b->h_need.clear();
    for (const BatchItem& it : items) b->h_need.push_back(it.need);
    HQ_REQUIRE(items.size() < (uint64_t(1) << 32) - 1, HQ_ERR_UNSUPPORTED, "batch: too many items");

    auto up16 = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t groups_b = up16(sizeof(OshmLaunch) * std::max<size_t>(progs.size(), 1));
    const size_t items_b = up16(sizeof(BatchItem) * std::max<size_t>(items.size(), 1));
    const size_t phases_b = up16(sizeof(OshmPhase) * std::max<size_t>(phases.size(), 1));
    const size_t ops_b = up16(sizeof(OshmOp) * std::max<size_t>(ops.size(), 1));
    const size_t ctr_b = up16(sizeof(uint32_t) * (1 + b->entries.size()));
    b->program_bytes = groups_b + items_b + phases_b + ops_b + ctr_b;
    b->d_program = (char*)dev_alloc(b->program_bytes);
    char* base = b->d_program;
    OshmLaunch* d_groups = (OshmLaunch*)base;
    BatchItem* d_items = (BatchItem*)(base + groups_b);
    OshmPhase* d_phases = (OshmPhase*)(base + groups_b + items_b);
    OshmOp* d_ops = (OshmOp*)(base + groups_b + items_b + phases_b);
    b->d_counters = (uint32_t*)(base + groups_b + items_b + phases_b + ops_b);
    b->counters_bytes = sizeof(uint32_t) * (1 + b->entries.size());

    std::vector<OshmLaunch> launches;
    for (size_t i = 0; i < progs.size(); i++) {
        const BatchEntry& e = b->entries[prog_circuit[i]];
        launches.push_back(make_oshm_launch(progs[i], e.s->d, d_phases + phase_off[i], d_ops,
                                            ctx().d_error));
    }
    cudaStream_t st = ctx().stream;
    auto put = [&](void* dst, const void* src, size_t bytes) {
        if (bytes) HQ_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    };
    put(d_groups, launches.data(), sizeof(OshmLaunch) * launches.size());
    put(d_items, items.data(), sizeof(BatchItem) * items.size());
    put(d_phases, phases.data(), sizeof(OshmPhase) * phases.size());
    put(d_ops, ops.data(), sizeof(OshmOp) * ops.size());
    HQ_CHECK_CUDA(cudaStreamSynchronize(st));

    b->launch = BatchLaunch{};
    b->launch.groups = d_groups;
    b->launch.items = d_items;
    b->launch.nitems = (uint32_t)items.size();
    b->launch.head = b->d_counters;
    b->launch.done = b->d_counters + 1;
    b->launch.err = ctx().d_error;
    b->grid = (int)std::min<uint64_t>(uint64_t(slots), std::max<uint64_t>(items.size(), 1));
    b->compiled = true;
}

// Everything one run enqueues: layouts, gate-by-gate circuits, counter reset,
// the persistent launch.
static void batch_enqueue_work(hq_batch_s* b, bool zero_init, cudaStream_t st) {
    for (BatchEntry& e : b->entries) {
        state_wait_copy(e.s);
        if (zero_init) {
            for (int q = 0; q < e.n; q++) e.s->pos[q] = q;  // contents are rewritten
            if (e.ngroups == 0) launch_init_zero(e.s->d, e.n, st);
        } else {
            state_canonicalize(e.s);
        }
        if (e.ngroups == 0 && !e.folded.empty()) apply_plain(e.s, e.folded);
    }
    if (b->num_items) {
        HQ_CHECK_CUDA(cudaMemsetAsync(b->d_counters, 0, b->counters_bytes, st));
        BatchLaunch l = b->launch;
        l.zero_init = zero_init ? 1u : 0u;
        l.stall_item = ~0u;
        if (b->stall_next) {
            // the first item that waits on a predecessor (else item 0) waits forever;
            // its bounded wait gives up and the run reports HQ_ERR_TIMEOUT
            l.stall_item = 0;
            for (uint32_t i = 0; i < b->h_need.size(); i++)
                if (b->h_need[i]) {
                    l.stall_item = i;
                    break;
                }
            b->stall_next = false;
        }
        launch_oshm_batch(l, b->grid, b->cooperative, st);
    }
    for (BatchEntry& e : b->entries)
        for (int q = 0; q < e.n; q++) e.s->pos[q] = e.swap_perm[q];
}

void batch_enqueue(hq_batch_s* b, bool zero_init) {
    HQ_REQUIRE(b->compiled, HQ_ERR_STATE, "batch not compiled");
    cudaStream_t st = ctx().stream;
    if (b->graph && b->graph_zero == zero_init && !b->stall_next) {
        for (BatchEntry& e : b->entries) {
            state_wait_copy(e.s);
            if (!zero_init) state_canonicalize(e.s);
        }
        HQ_CHECK_CUDA(cudaGraphLaunch(b->graph, st));
        for (BatchEntry& e : b->entries)
            for (int q = 0; q < e.n; q++) e.s->pos[q] = e.swap_perm[q];
        return;
    }
    batch_enqueue_work(b, zero_init, st);
}

double batch_run(hq_batch_s* b, bool zero_init) {
    cudaStream_t st = ctx().stream;
    if (!b->ev0) {
        HQ_CHECK_CUDA(cudaEventCreate(&b->ev0));
        HQ_CHECK_CUDA(cudaEventCreate(&b->ev1));
    }
    HQ_CHECK_CUDA(cudaEventRecord(b->ev0, st));
    batch_enqueue(b, zero_init);
    HQ_CHECK_CUDA(cudaEventRecord(b->ev1, st));
    HQ_CHECK_CUDA(cudaEventSynchronize(b->ev1));
    check_device_error();
    float ms = 0.f;
    HQ_CHECK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    return double(ms) * 1000.0;
}

void batch_capture(hq_batch_s* b, bool zero_init) {
    HQ_REQUIRE(b->compiled, HQ_ERR_STATE, "batch not compiled");
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    // the graph replays on canonical layouts; bring states there first, and
    // keep the layouts as they are now (capturing runs nothing)
    if (!zero_init)
        for (BatchEntry& e : b->entries) state_canonicalize(e.s);
    std::vector<std::vector<int>> saved;
    for (const BatchEntry& e : b->entries) saved.push_back(e.s->pos);
    struct Restore {
        hq_batch_s* b;
        std::vector<std::vector<int>>& saved;
        ~Restore() {
            for (size_t i = 0; i < b->entries.size(); i++) b->entries[i].s->pos = saved[i];
        }
    } restore{b, saved};
    cudaStream_t cs;
    HQ_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    try {
        HQ_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        try {
            batch_enqueue_work(b, zero_init, cs);
        } catch (...) {
            cudaStreamEndCapture(cs, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        HQ_CHECK_CUDA(cudaStreamEndCapture(cs, &g));
        HQ_CHECK_CUDA(cudaGraphInstantiate(&b->graph, g, 0));
        cudaGraphDestroy(g);
    } catch (...) {
        cudaStreamDestroy(cs);
        throw;
    }
    cudaStreamDestroy(cs);
    b->graph_zero = zero_init;
}

}  // namespace hq
