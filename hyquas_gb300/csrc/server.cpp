// Serving: a request loop with HBM-budget admission and continuous batching.
//
// The reference runs one circuit per process (src/main.cpp:12-230); it has no
// request loop.  Here requests (an n-qubit gate list) are submitted from any
// host thread.  Planner threads partition and lower them (the same OShareMem
// grouping as compiled circuits, compiler.cpp).  One engine thread admits
// planned requests in arrival order while their state bytes (2^n x 8 B) fit
// the budget, and runs STEPS: a step is one persistent batched launch
// (k_oshm_batch) over the next few gate groups of every admitted request, so
// requests that arrive while others run join at the next step and their work
// overlaps on the device.  A step holds about `step_budget_us` of estimated
// device time split evenly between the admitted requests; a request whose
// next group is larger than its share runs a slice of that group's tiles, so
// a 32-qubit request never holds newly arrived small ones back for longer
// than a step.  Small circuits finish within one step.  The engine builds and
// enqueues step s+1 before it waits for step s.  States stay resident until
// the caller releases them.
#include <algorithm>
#include <chrono>
#include <cstring>

#include "batch.h"
#include "common.h"
#include "gates.h"
#include "server.h"

namespace hq {

namespace {

double now_us(const hq_server_s* sv) {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - sv->t0)
        .count();
}

// Host-side request checks shared with hq_server_check (no GPU needed).
void check_request(const hq_server_options& o, int n, const hq_gate* gates, int count) {
    HQ_REQUIRE(n >= kBatchMinTile && n <= 34, HQ_ERR_INVALID,
               "served circuits have %d to 34 qubits, got %d", kBatchMinTile, n);
    HQ_REQUIRE(count >= 0 && (count == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    for (int i = 0; i < count; i++) validate_gate(gates[i], n);
    const uint64_t bytes = uint64_t(8) << n;
    HQ_REQUIRE(o.hbm_budget == 0 || bytes <= o.hbm_budget, HQ_ERR_NOMEM,
               "a %d-qubit state (%llu bytes) exceeds the serving budget (%llu bytes)", n,
               (unsigned long long)bytes, (unsigned long long)o.hbm_budget);
}

// Plans are cached by circuit (qubit count, gate records, tile option): a
// request whose circuit was planned before reuses that plan.
uint64_t plan_key(const Request* r, int fixed_k) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* b = (const unsigned char*)p;
        for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    };
    mix(&r->n, sizeof(r->n));
    mix(&fixed_k, sizeof(fixed_k));
    if (!r->gates.empty()) mix(r->gates.data(), sizeof(hq_gate) * r->gates.size());
    return h;
}

bool same_gates(const std::vector<hq_gate>& a, const std::vector<hq_gate>& b) {
    return a.size() == b.size() &&
           (a.empty() || std::memcmp(a.data(), b.data(), sizeof(hq_gate) * a.size()) == 0);
}

// fuse: runs of single-qubit gates as one gate (for the interpreted batch
// kernel; generated kernels run the gates unfused more cheaply)
void plan_request(Request* r, int fixed_k, bool fuse) {
    std::vector<int> perm;
    std::vector<hq_gate> folded = fold_swaps(r->gates, r->n, perm);
    if (fuse) folded = fuse_single_qubit_runs(folded, r->n);
    r->swap_perm = perm;
    const int n = r->n;
    if (folded.empty()) return;
    std::vector<int> id(n);
    for (int q = 0; q < n; q++) id[q] = q;
    CompileConfig cfg;
    cfg.backend = HQ_BACKEND_OSHM;
    cfg.tile = fixed_k ? std::min(fixed_k, n) : std::min(n, kBatchTile);
    cfg.coalesce = std::min(3, cfg.tile);
    Partition part = partition(n, folded, id, cfg);
    r->k = cfg.tile;
    for (const GroupPlan& gp : part.groups) {
        std::vector<hq_gate> phys;
        for (int x : gp.gates) phys.push_back(folded[x]);
        r->progs.push_back(plan_oshm(n, phys, oshm_tile_mask(gp, n)));
        r->group_cost.push_back(cost_oshm(n, 0, phys, cfg.tile) * 1e6);
    }
}

void planner_main(hq_server_s* sv) {
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_plan.wait(lk, [&] { return sv->stop || !sv->to_plan.empty(); });
            if (sv->stop) return;
            r = sv->to_plan.front();
            sv->to_plan.pop_front();
        }
        std::string err;
        try {
            const uint64_t key = plan_key(r, sv->opt.tile_qubits);
            std::shared_ptr<const PlanEntry> hit;
            {
                std::lock_guard<std::mutex> lk(sv->cache_mu);
                auto it = sv->plan_cache.find(key);
                if (it != sv->plan_cache.end() && it->second->n == r->n &&
                    same_gates(it->second->gates, r->gates))
                    hit = it->second;
            }
            if (hit) {
                r->progs = hit->progs;
                r->group_cost = hit->group_cost;
                r->swap_perm = hit->swap_perm;
                r->k = hit->k;
                r->jit = hit->jit;
                std::lock_guard<std::mutex> lk(sv->cache_mu);
                sv->cache_hits++;
            } else {
                const int jit_min = sv->opt.jit_min_qubits;
                const bool use_jit = jit_min > 0 && r->n >= jit_min && jit_available();
                plan_request(r, sv->opt.tile_qubits, !use_jit);
                if (use_jit && !r->progs.empty()) {
                    std::vector<const OshmProgram*> ps;
                    for (const OshmProgram& pg : r->progs) ps.push_back(&pg);
                    try {
                        r->jit = jit_compile_groups(ps);
                    } catch (const Failure&) {
                        r->jit.clear();  // the batched interpreter runs it instead
                    }
                }
                auto e = std::make_shared<PlanEntry>();
                e->n = r->n;
                e->gates = r->gates;
                e->progs = r->progs;
                e->group_cost = r->group_cost;
                e->swap_perm = r->swap_perm;
                e->k = r->k;
                e->jit = r->jit;
                std::lock_guard<std::mutex> lk(sv->cache_mu);
                if (!sv->plan_cache.count(key)) {
                    sv->plan_cache[key] = e;
                    sv->cache_order.push_back(key);
                    while (sv->cache_order.size() > kPlanCacheEntries) {
                        sv->plan_cache.erase(sv->cache_order.front());
                        sv->cache_order.pop_front();
                    }
                }
            }
        } catch (const std::exception& e) {
            err = e.what();
        }
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            if (!err.empty()) {
                r->status = HQ_REQ_FAILED;
                r->error = err;
                r->t_done = now_us(sv);
                sv->completed.push_back(r->id);
                sv->cv_done.notify_all();
            } else {
                r->status = HQ_REQ_QUEUED;
                sv->planned.push_back(r);
                sv->cv_engine.notify_all();
            }
        }
    }
}

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Grow a pinned host buffer (only ever called for a buffer no copy is using).
void grow_host(char*& p, size_t& cap, size_t need) {
    if (need <= cap) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t c = std::max<size_t>(need, 1 << 20);
    c = c + c / 2;
    HQ_CHECK_CUDA(cudaHostAlloc((void**)&p, c, cudaHostAllocDefault));
    cap = c;
}

void grow_dev(char*& p, size_t& cap, size_t need, cudaStream_t st) {
    if (need <= cap) return;
    if (p) HQ_CHECK_CUDA(cudaFreeAsync(p, st));
    p = nullptr;
    cap = 0;
    size_t c = std::max<size_t>(need, 1 << 20);
    c = c + c / 2;
    HQ_CHECK_CUDA(cudaMallocAsync((void**)&p, c, st));
    cap = c;
}

void free_request_memory(hq_server_s* sv, Request* r) {
    cudaStream_t st = sv->stream;
    if (r->state) {
        // a caller's asynchronous readback of the borrowed state finishes first
        if (r->state->copy_pending) HQ_CHECK_CUDA(cudaStreamWaitEvent(st, r->state->copy_done, 0));
        if (r->state->ready) cudaEventDestroy(r->state->ready);
        if (r->state->copy_done) cudaEventDestroy(r->state->copy_done);
        if (r->state->d) cudaFreeAsync(r->state->d, st);
        if (r->state->d_scratch) cudaFreeAsync(r->state->d_scratch, st);
        delete r->state;
        r->state = nullptr;
    }
    if (r->d_prog) cudaFreeAsync(r->d_prog, st);
    r->d_prog = nullptr;
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->resident -= std::min(sv->resident, r->resident_bytes);
    r->resident_bytes = 0;
}

// Admission (engine thread, lock held): planned requests in arrival order while
// they fit; a request that does not fit blocks the ones behind it unless those
// are small (at most 1/64 of the budget), so large requests are not starved.
std::vector<Request*> pick_admissions(hq_server_s* sv) {
    std::vector<Request*> out;
    const uint64_t budget = sv->opt.hbm_budget ? sv->opt.hbm_budget : ~uint64_t(0);
    uint64_t used = sv->resident;
    bool blocked = false;
    for (auto it = sv->planned.begin(); it != sv->planned.end();) {
        Request* r = *it;
        const uint64_t need = r->state_bytes;
        const bool small = need <= budget / 64;
        if ((!blocked || small) && used + need <= budget) {
            used += need;
            out.push_back(r);
            it = sv->planned.erase(it);
        } else {
            blocked = true;
            ++it;
        }
    }
    return out;
}

// Allocate a request's state and program and queue the program upload from
// the step's pinned staging area (engine thread).
void admit(hq_server_s* sv, Request* r, StepBuf& sb, size_t& host_off) {
    cudaStream_t st = sv->stream;
    const int n = r->n;
    auto s = new hq_state_s();
    s->n = n;
    s->bytes = size_t(8) << n;
    s->pos.resize(n);
    for (int q = 0; q < n; q++) s->pos[q] = q;
    s->scratch_doubles = state_scratch_doubles(n);
    r->state = s;
    HQ_CHECK_CUDA(cudaMallocAsync(&s->d, s->bytes, st));
    HQ_CHECK_CUDA(cudaMallocAsync((void**)&s->d_scratch, sizeof(double) * s->scratch_doubles, st));
    size_t nph = 0, nop = 0;
    for (const OshmProgram& p : r->progs) {
        nph += p.phases.size();
        nop += p.ops.size();
    }
    const size_t ph_b = round256(sizeof(OshmPhase) * std::max<size_t>(nph, 1));
    const size_t op_b = round256(sizeof(OshmOp) * std::max<size_t>(nop, 1));
    r->prog_bytes = ph_b + op_b;
    HQ_CHECK_CUDA(cudaMallocAsync((void**)&r->d_prog, r->prog_bytes, st));
    r->d_phases = (OshmPhase*)r->d_prog;
    r->d_ops = (OshmOp*)(r->d_prog + ph_b);
    // stage phases (op indices made absolute) and ops
    char* h = sb.h + host_off;
    OshmPhase* hp = (OshmPhase*)h;
    OshmOp* ho = (OshmOp*)(h + ph_b);
    size_t pi = 0, oi = 0;
    r->phase_off.clear();
    for (const OshmProgram& p : r->progs) {
        r->phase_off.push_back(pi);
        for (OshmPhase ph : p.phases) {
            ph.op_begin += (uint32_t)oi;
            ph.op_end += (uint32_t)oi;
            hp[pi++] = ph;
        }
        for (const OshmOp& op : p.ops) ho[oi++] = op;
    }
    HQ_CHECK_CUDA(cudaMemcpyAsync(r->d_prog, h, r->prog_bytes, cudaMemcpyHostToDevice, st));
    host_off += r->prog_bytes;
    r->next = 0;
}

size_t program_stage_bytes(const Request* r) {
    size_t nph = 0, nop = 0;
    for (const OshmProgram& p : r->progs) {
        nph += p.phases.size();
        nop += p.ops.size();
    }
    return round256(sizeof(OshmPhase) * std::max<size_t>(nph, 1)) +
           round256(sizeof(OshmOp) * std::max<size_t>(nop, 1));
}

// Build and enqueue one step over `members` into buffer sb.
void enqueue_step(hq_server_s* sv, StepBuf& sb, std::vector<Request*>& newly,
                  std::vector<Request*>& members) {
    cudaStream_t st = sv->stream;
    const int slots = sv->slots;
    // What each member runs in this step: whole groups [g0, g1), or, when its
    // next group alone is over its share of the step, a tile range
    // [ta, tb) of group g0 (g1 = g0 + 1, partial = true).  Shares split the
    // step budget evenly between the members.
    const size_t nm = members.size();
    std::vector<uint32_t> g0(nm), g1(nm);
    std::vector<uint64_t> ta(nm), tb(nm);
    std::vector<char> partial(nm, 0);
    size_t working = 0;
    for (Request* r : members)
        if (r->next < r->progs.size()) working++;
    const double share = sv->opt.step_budget_us / double(std::max<size_t>(working, 1));
    // requests with generated kernels: whole groups, launched on their own
    std::vector<std::pair<Request*, uint32_t>> jit_runs;  // (request, groups to run)
    for (size_t i = 0; i < nm; i++) {
        Request* r = members[i];
        const uint32_t total = (uint32_t)r->progs.size();
        g0[i] = g1[i] = r->next;
        if (r->next >= total) continue;
        if (!r->jit.empty()) {
            uint32_t e = r->next;
            double acc = 0;
            while (e < total && (e == r->next || acc + r->group_cost[e] <= share)) {
                acc += r->group_cost[e];
                e++;
            }
            jit_runs.push_back({r, e});
            g1[i] = g0[i];  // no batched items
            continue;
        }
        const uint64_t tiles = uint64_t(1) << (r->n - r->k);
        const uint32_t ch = batch_chunk_tiles(tiles, slots);
        const double group_us = r->group_cost[r->next];
        if (r->next_tile > 0 || group_us > share) {
            // a slice of one group, whole items, at least one
            const double per_tile = group_us / double(tiles);
            uint64_t want = uint64_t(share / std::max(per_tile, 1e-12));
            want = std::max<uint64_t>((want / ch) * ch, ch);
            ta[i] = r->next_tile;
            tb[i] = std::min<uint64_t>(tiles, ta[i] + want);
            g1[i] = r->next + 1;
            partial[i] = 1;
            continue;
        }
        uint32_t e = r->next;
        double acc = 0;
        while (e < total && (e == r->next || acc + r->group_cost[e] <= share)) {
            acc += r->group_cost[e];
            e++;
        }
        g1[i] = e;
        ta[i] = 0;
        tb[i] = tiles;
    }
    // items, level-major; members sorted by remaining depth so long chains start first
    std::vector<size_t> order(nm);
    for (size_t i = 0; i < nm; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
        return members[x]->progs.size() - g0[x] > members[y]->progs.size() - g0[y];
    });
    std::vector<size_t> launch_base(nm);
    size_t nl = 0;
    uint32_t levels = 0;
    size_t nitems = 0;
    for (size_t i = 0; i < nm; i++) {
        launch_base[i] = nl;
        nl += g1[i] - g0[i];
        levels = std::max(levels, g1[i] - g0[i]);
        if (g1[i] == g0[i]) continue;
        const uint64_t tiles = uint64_t(1) << (members[i]->n - members[i]->k);
        const uint32_t ch = batch_chunk_tiles(tiles, slots);
        nitems += size_t(g1[i] - g0[i]) * ((tb[i] - ta[i] + ch - 1) / ch);
    }
    const size_t launches_b = round256(sizeof(OshmLaunch) * std::max<size_t>(nl, 1));
    const size_t items_b = round256(sizeof(BatchItem) * std::max<size_t>(nitems, 1));
    const size_t ctr_b = round256(sizeof(uint32_t) * (1 + nm));
    size_t prog_b = 0;
    for (Request* r : newly) prog_b += program_stage_bytes(r);
    grow_host(sb.h, sb.hcap, launches_b + items_b + prog_b);
    grow_dev(sb.d, sb.dcap, launches_b + items_b + ctr_b, st);

    // admissions: states and programs (their copies precede the launch)
    size_t host_off = launches_b + items_b;
    for (Request* r : newly) admit(sv, r, sb, host_off);

    OshmLaunch* hl = (OshmLaunch*)sb.h;
    BatchItem* hi = (BatchItem*)(sb.h + launches_b);
    OshmLaunch* dl = (OshmLaunch*)sb.d;
    for (size_t i = 0; i < nm; i++) {
        Request* r = members[i];
        for (uint32_t g = g0[i]; g < g1[i]; g++)
            hl[launch_base[i] + (g - g0[i])] = make_oshm_launch(
                r->progs[g], r->state->d, r->d_phases + r->phase_off[g], r->d_ops, sv->d_err);
    }
    size_t ii = 0;
    for (uint32_t L = 0; L < levels; L++) {
        for (size_t oi : order) {
            Request* r = members[oi];
            if (L >= g1[oi] - g0[oi]) continue;
            const uint64_t tiles = uint64_t(1) << (r->n - r->k);
            const uint32_t ch = batch_chunk_tiles(tiles, slots);
            for (uint64_t u = ta[oi]; u < tb[oi]; u += ch) {
                BatchItem& it = hi[ii++];
                it.group = (uint32_t)(launch_base[oi] + L);
                it.circuit = (uint32_t)oi;
                it.tile0 = (uint32_t)u;
                it.count = (uint32_t)std::min<uint64_t>(ch, tb[oi] - u);
                it.need = (uint32_t)(uint64_t(L) * tiles);  // every tile of the levels before
                it.flags = (g0[oi] + L == 0) ? ITEM_FIRST : 0;
            }
        }
    }
    // gate-less requests: |0...0> only
    for (Request* r : members)
        if (r->progs.empty() && r->next == 0) launch_init_zero(r->state->d, r->n, st);
    // generated kernels: |0...0> before the first group, then whole groups
    for (auto& jr : jit_runs) {
        Request* r = jr.first;
        if (r->next == 0) launch_init_zero(r->state->d, r->n, st);
        for (uint32_t g = r->next; g < jr.second; g++)
            jit_launch(r->jit[g], r->state->d, uint64_t(1) << (r->n - r->progs[g].k), sv->d_err, st);
    }
    if (nl) {
        HQ_CHECK_CUDA(cudaMemcpyAsync(sb.d, sb.h, launches_b + items_b, cudaMemcpyHostToDevice, st));
        uint32_t* ctr = (uint32_t*)(sb.d + launches_b + items_b);
        HQ_CHECK_CUDA(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * (1 + members.size()), st));
        BatchLaunch bl{};
        bl.groups = dl;
        bl.items = (const BatchItem*)(sb.d + launches_b);
        bl.nitems = (uint32_t)nitems;
        bl.zero_init = 1;
        bl.head = ctr;
        bl.done = ctr + 1;
        bl.err = sv->d_err;
        bl.stall_item = ~0u;
        const int grid = (int)std::min<size_t>(size_t(slots), std::max<size_t>(nitems, 1));
        launch_oshm_batch(bl, grid, true, st);
        HQ_CHECK_CUDA(cudaMemcpyAsync(sb.h_err, sv->d_err, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
    }
    HQ_CHECK_CUDA(cudaEventRecord(sb.ev, st));
    sb.members = members;
    sb.finishing.clear();
    for (auto& jr : jit_runs) jr.first->next = jr.second;
    for (size_t i = 0; i < nm; i++) {
        Request* r = members[i];
        if (r->first_step < 0) r->first_step = sv->steps;
        r->last_step = sv->steps;
        if (!r->jit.empty()) {
            if (r->next == r->progs.size()) sb.finishing.push_back(r);
            continue;
        }
        if (partial[i]) {
            const uint64_t tiles = uint64_t(1) << (r->n - r->k);
            r->next_tile = tb[i] < tiles ? tb[i] : 0;
            if (r->next_tile == 0) r->next = g1[i];
        } else {
            r->next = g1[i];
        }
        if (r->next == r->progs.size()) sb.finishing.push_back(r);
    }
    sb.had_launch = nl > 0;
    sb.inflight = true;
    sv->steps++;
    sv->items += (int64_t)nitems;
}

// Wait for a step; mark its finishing requests done (or every member failed).
void finish_step(hq_server_s* sv, StepBuf& sb) {
    if (!sb.inflight) return;
    HQ_CHECK_CUDA(cudaEventSynchronize(sb.ev));
    sb.inflight = false;
    const double t = now_us(sv);
    std::string err;
    if (sb.had_launch && sb.h_err[0] != 0) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "device error %d at site %d (item %d) in a serving step",
                      sb.h_err[0], sb.h_err[1], sb.h_err[2]);
        err = msg;
        HQ_CHECK_CUDA(cudaMemsetAsync(sv->d_err, 0, sizeof(int) * 4, sv->stream));
        HQ_CHECK_CUDA(cudaStreamSynchronize(sv->stream));
    }
    std::lock_guard<std::mutex> lk(sv->mu);
    auto settle = [&](Request* r, int status) {
        r->status = status;
        r->t_done = t;
        if (status == HQ_REQ_FAILED) r->error = err;
        if (r->state)
            for (int q = 0; q < r->n; q++) r->state->pos[q] = r->swap_perm[q];
        sv->completed.push_back(r->id);
        sv->running.erase(std::remove(sv->running.begin(), sv->running.end(), r), sv->running.end());
        sv->ndone++;
    };
    if (!err.empty()) {
        for (Request* r : sb.members)
            if (r->status == HQ_REQ_RUNNING) settle(r, HQ_REQ_FAILED);
    } else {
        for (Request* r : sb.finishing) settle(r, HQ_REQ_DONE);
    }
    sv->cv_done.notify_all();
}

void engine_main(hq_server_s* sv) {
    cudaSetDevice(ctx().device);
    uint64_t s = 0;
    try {
        for (;;) {
            std::vector<Request*> newly, members;
            std::vector<Request*> frees;
            {
                std::unique_lock<std::mutex> lk(sv->mu);
                const bool inflight = sv->buf[0].inflight || sv->buf[1].inflight;
                if (!inflight && sv->running.empty() && sv->planned.empty() && sv->to_free.empty()) {
                    if (sv->stop) break;
                    sv->cv_engine.wait_for(lk, std::chrono::milliseconds(2));
                    continue;
                }
                if (sv->stop && !inflight) break;
                frees.swap(sv->to_free);
                if (!sv->stop) {
                    newly = pick_admissions(sv);
                    for (Request* r : newly) {
                        r->status = HQ_REQ_RUNNING;
                        r->t_admit = now_us(sv);
                        sv->resident += r->state_bytes;  // admission counts state bytes
                        r->resident_bytes = r->state_bytes;
                        sv->running.push_back(r);
                    }
                    sv->peak_resident = std::max(sv->peak_resident, sv->resident);
                    for (Request* r : sv->running)
                        if (r->next < r->progs.size() || (r->progs.empty() && r->next == 0 &&
                                                           r->state == nullptr))
                            members.push_back(r);
                }
            }
            for (Request* r : frees) {
                // the record (status, times) stays; memory and plan go
                free_request_memory(sv, r);
                std::vector<OshmProgram>().swap(r->progs);
                std::vector<hq_gate>().swap(r->gates);
            }
            const bool busy = sv->buf[0].inflight || sv->buf[1].inflight;
            if (members.empty() && newly.empty() && frees.empty() && !busy) {
                // planned requests wait for memory held by unreleased results
                std::unique_lock<std::mutex> lk(sv->mu);
                sv->cv_engine.wait_for(lk, std::chrono::milliseconds(1));
                continue;
            }
            StepBuf& cur = sv->buf[s & 1];
            StepBuf& prev = sv->buf[(s + 1) & 1];
            bool launched = false;
            // gate-less requests are members once (their state gets |0...0>)
            if (!members.empty() || !newly.empty()) {
                for (Request* r : newly)
                    if (r->progs.empty() &&
                        std::find(members.begin(), members.end(), r) == members.end())
                        members.push_back(r);
                finish_step(sv, cur);  // the buffer's previous step (s-2) is long done
                enqueue_step(sv, cur, newly, members);
                launched = true;
                s++;
            }
            finish_step(sv, prev);
            if (!launched) finish_step(sv, cur);
        }
        finish_step(sv, sv->buf[0]);
        finish_step(sv, sv->buf[1]);
    } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->engine_error = e.what();
        for (Request* r : sv->running) {
            r->status = HQ_REQ_FAILED;
            r->error = e.what();
            sv->completed.push_back(r->id);
        }
        sv->running.clear();
        for (Request* r : sv->planned) {
            r->status = HQ_REQ_FAILED;
            r->error = e.what();
            sv->completed.push_back(r->id);
        }
        sv->planned.clear();
        sv->cv_done.notify_all();
    }
}

}  // namespace

void server_check(const hq_server_options& o, int n, const hq_gate* gates, int count) {
    check_request(o, n, gates, count);
}

hq_server_s* server_create(const hq_server_options& o) {
    ensure_init();
    auto sv = new hq_server_s();
    sv->opt = o;
    if (sv->opt.step_budget_us <= 0) sv->opt.step_budget_us = 2000.0;
    if (sv->opt.planner_threads <= 0) sv->opt.planner_threads = 4;
    sv->t0 = std::chrono::steady_clock::now();
    try {
        HQ_CHECK_CUDA(cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking));
        // keep freed pool memory for reuse instead of returning it after each sync
        cudaMemPool_t pool;
        HQ_CHECK_CUDA(cudaDeviceGetDefaultMemPool(&pool, ctx().device));
        uint64_t keep = ~uint64_t(0);
        HQ_CHECK_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        HQ_CHECK_CUDA(cudaMalloc(&sv->d_err, sizeof(int) * 4));
        HQ_CHECK_CUDA(cudaMemset(sv->d_err, 0, sizeof(int) * 4));
        for (StepBuf& b : sv->buf) {
            HQ_CHECK_CUDA(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming));
            HQ_CHECK_CUDA(cudaHostAlloc((void**)&b.h_err, sizeof(int) * 4, cudaHostAllocDefault));
            std::memset(b.h_err, 0, sizeof(int) * 4);
        }
        sv->slots = oshm_batch_slots();
    } catch (...) {
        server_destroy(sv);
        throw;
    }
    sv->engine = std::thread(engine_main, sv);
    for (int i = 0; i < sv->opt.planner_threads; i++) sv->planners.emplace_back(planner_main, sv);
    return sv;
}

void server_destroy(hq_server_s* sv) {
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_plan.notify_all();
    sv->cv_engine.notify_all();
    if (sv->engine.joinable()) sv->engine.join();
    for (auto& t : sv->planners)
        if (t.joinable()) t.join();
    for (auto& kv : sv->reqs) free_request_memory(sv, kv.second.get());
    for (StepBuf& b : sv->buf) {
        if (b.d) cudaFreeAsync(b.d, sv->stream);
        if (b.h) cudaFreeHost(b.h);
        if (b.h_err) cudaFreeHost(b.h_err);
        if (b.ev) cudaEventDestroy(b.ev);
    }
    if (sv->stream) {
        cudaStreamSynchronize(sv->stream);
        cudaStreamDestroy(sv->stream);
    }
    if (sv->d_err) cudaFree(sv->d_err);
    delete sv;
}

int64_t server_submit(hq_server_s* sv, int n, const hq_gate* gates, int count) {
    check_request(sv->opt, n, gates, count);
    auto r = std::make_unique<Request>();
    r->n = n;
    r->gates.assign(gates, gates + count);
    r->state_bytes = uint64_t(8) << n;
    std::lock_guard<std::mutex> lk(sv->mu);
    HQ_REQUIRE(sv->engine_error.empty(), HQ_ERR_STATE, "server stopped: %s", sv->engine_error.c_str());
    r->id = sv->next_id++;
    r->t_submit = now_us(sv);
    r->status = HQ_REQ_PLANNING;
    Request* p = r.get();
    sv->reqs[r->id] = std::move(r);
    sv->to_plan.push_back(p);
    sv->cv_plan.notify_one();
    return p->id;
}

Request* server_find(hq_server_s* sv, int64_t id) {
    auto it = sv->reqs.find(id);
    HQ_REQUIRE(it != sv->reqs.end(), HQ_ERR_INVALID, "no request %lld", (long long)id);
    return it->second.get();
}

int server_wait(hq_server_s* sv, int64_t id, double timeout_s) {
    std::unique_lock<std::mutex> lk(sv->mu);
    Request* r = server_find(sv, id);
    const auto until = std::chrono::steady_clock::now() +
                       std::chrono::microseconds(int64_t(std::max(0.0, timeout_s) * 1e6));
    sv->cv_done.wait_until(lk, until, [&] {
        return r->status == HQ_REQ_DONE || r->status == HQ_REQ_FAILED;
    });
    return r->status;
}

int server_poll(hq_server_s* sv, int64_t* ids, int cap) {
    std::lock_guard<std::mutex> lk(sv->mu);
    const int k = std::min<int>(cap, (int)sv->completed.size());
    for (int i = 0; i < k; i++) ids[i] = sv->completed[i];
    sv->completed.erase(sv->completed.begin(), sv->completed.begin() + k);
    return k;
}

void server_release(hq_server_s* sv, int64_t id) {
    std::lock_guard<std::mutex> lk(sv->mu);
    Request* r = server_find(sv, id);
    HQ_REQUIRE(r->status == HQ_REQ_DONE || r->status == HQ_REQ_FAILED, HQ_ERR_BUSY,
               "request %lld is still queued or running", (long long)id);
    HQ_REQUIRE(!r->released, HQ_ERR_INVALID, "request %lld already released", (long long)id);
    r->released = true;
    sv->to_free.push_back(r);
    sv->cv_engine.notify_all();
}

}  // namespace hq
