// Request loop with HBM-budget admission and continuous batching (server.cpp).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"
#include "compiler.h"
#include "device.h"
#include "executor.h"
#include "jit.h"

namespace hq {

struct Request {
    int64_t id = 0;
    int n = 0;
    std::vector<hq_gate> gates;
    // plan (planner thread)
    std::vector<OshmProgram> progs;
    std::vector<double> group_cost;  // estimated device microseconds per group
    std::vector<int> swap_perm;
    int k = 0;
    std::vector<JitKernel> jit;      // generated group kernels (large requests), else empty
    // device (engine thread)
    hq_state_s* state = nullptr;
    char* d_prog = nullptr;
    size_t prog_bytes = 0;
    OshmPhase* d_phases = nullptr;
    OshmOp* d_ops = nullptr;
    std::vector<size_t> phase_off;   // first phase of each group
    uint32_t next = 0;               // next group to put in a step
    uint64_t next_tile = 0;          // first tile of `next` not yet in a step
    int status = HQ_REQ_PLANNING;
    bool released = false;
    std::string error;
    double t_submit = 0, t_admit = 0, t_done = 0;  // microseconds since the server started
    int64_t first_step = -1, last_step = -1;       // steps the request's work ran in
    uint64_t state_bytes = 0, resident_bytes = 0;
};

// A cached plan: the circuit it is for and its lowered groups.
struct PlanEntry {
    int n = 0;
    std::vector<hq_gate> gates;
    std::vector<OshmProgram> progs;
    std::vector<double> group_cost;
    std::vector<int> swap_perm;
    int k = 0;
    std::vector<JitKernel> jit;
};
constexpr size_t kPlanCacheEntries = 256;

// One step's staging: pinned host copy of launches, items and new programs,
// their device copy, and the completion event.
struct StepBuf {
    char* h = nullptr;
    size_t hcap = 0;
    char* d = nullptr;
    size_t dcap = 0;
    int* h_err = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<Request*> members, finishing;
    bool inflight = false, had_launch = false;
};

}  // namespace hq

struct hq_server_s {
    hq_server_options opt{};
    std::mutex mu;
    std::condition_variable cv_plan, cv_engine, cv_done;
    std::deque<hq::Request*> to_plan, planned;
    std::vector<hq::Request*> running, to_free;
    std::unordered_map<int64_t, std::unique_ptr<hq::Request>> reqs;
    std::vector<int64_t> completed;  // finished since the last poll
    int64_t next_id = 1;
    uint64_t resident = 0, peak_resident = 0;
    int64_t steps = 0, items = 0, ndone = 0;
    bool stop = false;
    std::string engine_error;
    std::thread engine;
    std::vector<std::thread> planners;
    cudaStream_t stream = nullptr;
    int* d_err = nullptr;
    int slots = 0;
    hq::StepBuf buf[2];
    std::mutex cache_mu;  // plan cache (planner threads)
    std::unordered_map<uint64_t, std::shared_ptr<const hq::PlanEntry>> plan_cache;
    std::deque<uint64_t> cache_order;
    int64_t cache_hits = 0;
    std::chrono::steady_clock::time_point t0;
};

namespace hq {

void server_check(const hq_server_options& o, int n, const hq_gate* gates, int count);
hq_server_s* server_create(const hq_server_options& o);
void server_destroy(hq_server_s* sv);
int64_t server_submit(hq_server_s* sv, int n, const hq_gate* gates, int count);
Request* server_find(hq_server_s* sv, int64_t id);  // caller holds sv->mu
int server_wait(hq_server_s* sv, int64_t id, double timeout_s);
int server_poll(hq_server_s* sv, int64_t* ids, int cap);
void server_release(hq_server_s* sv, int64_t id);

}  // namespace hq
