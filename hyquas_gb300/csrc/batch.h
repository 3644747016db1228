// Batched execution of many circuits in one persistent launch (batch.cpp).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "compiler.h"
#include "device.h"
#include "executor.h"

namespace hq {

struct BatchEntry {
    int n = 0;
    hq_state_s* s = nullptr;
    std::vector<hq_gate> gates;     // as added
    std::vector<hq_gate> folded;    // SWAPs folded away
    std::vector<int> swap_perm;     // layout after the run
    int k = 0;                      // tile width (0: gate by gate)
    uint32_t group0 = 0, ngroups = 0;
};

}  // namespace hq

struct hq_batch_s {
    std::vector<hq::BatchEntry> entries;
    bool compiled = false;
    char* d_program = nullptr;      // groups | items | phases | ops | counters
    size_t program_bytes = 0;
    uint32_t* d_counters = nullptr; // head, then one per circuit
    size_t counters_bytes = 0;
    hq::BatchLaunch launch{};
    int grid = 0, slots = 0;
    bool cooperative = true;
    bool stall_next = false;        // test hook: the next run's bounded wait expires
    int64_t num_groups = 0, num_items = 0;
    std::vector<uint32_t> h_need;   // each item's dependency count (host copy)
    uint64_t pass_bytes = 0;
    cudaGraphExec_t graph = nullptr;
    bool graph_zero = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace hq {

uint32_t batch_chunk_tiles(uint64_t tiles, int slots);
void batch_compile(hq_batch_s* b, const hq_compile_options* opt);
void batch_release(hq_batch_s* b);
void batch_enqueue(hq_batch_s* b, bool zero_init);
double batch_run(hq_batch_s* b, bool zero_init);
void batch_capture(hq_batch_s* b, bool zero_init);

}  // namespace hq
