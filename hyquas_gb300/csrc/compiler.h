// Hybrid partitioner (gate grouping), cost model and OShareMem lowering.
//
// Grouping follows the reference's greedy OneLayerCompiler::getGroupOpt
// (src/compiler.cpp:322-452) driven the way AdvanceCompiler::run drives it
// (src/compiler.cpp:220-319).  With `reference_grouping` the widths are the
// reference's (tile 10 qubits, 3 coalesced qubits, MAT 6) and the partition is
// gate-for-gate the reference's; otherwise the GB300 widths and the GB300 cost
// model are used.
#pragma once

#include <cstdint>
#include <vector>

#include "device.h"
#include "gates.h"

namespace hq {

struct CompileConfig {
    int backend = HQ_BACKEND_OSHM;
    int tile = 13;       // OShareMem tile width k
    int coalesce = 3;    // low physical qubits always in a tile
    int mm_qubits = 6;   // TransMM width
    int mm_precision = HQ_MM_BF16X3;
    bool reference = false;
    bool tile_auto = false;  // choose the tile width (11..13) by predicted time
};

struct GroupPlan {
    int backend = HQ_BACKEND_OSHM;
    std::vector<int> gates;       // indices into the swap-folded gate list
    uint64_t related = 0;         // logical qubits the group's tile/matrix spans
    int width = 0;                // tile width (OShareMem) or matrix qubits (TransMM)
    std::vector<int> pos;         // logical -> physical layout while the group runs
    std::vector<int> pos_after;   // layout after the group
};

struct Partition {
    std::vector<GroupPlan> groups;
    std::vector<int> final_pos;   // logical -> physical after the last group
};

// Group `gates` (logical qubits, no SWAP) for an n-qubit register whose
// initial layout is `pos0` (logical -> physical).
Partition partition(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                    const CompileConfig& cfg);

// The cost model's device time (seconds) of a partition of `gates`.
double predicted_time(int n, const std::vector<hq_gate>& gates, const Partition& part,
                      const CompileConfig& cfg);

// GB300 cost model (seconds) used by the hybrid backend; the constants are
// fitted to kernel timings on GB300 (compiler.cpp).
hq_cost_params cost_params();
void set_cost_params(const hq_cost_params& p);
hq_cost_params autotune(int n);  // autotune.cpp: measure and install the parameters
double cost_oshm(int n, int nphases, const std::vector<hq_gate>& gates, int k);
double oshm_gate_units(const hq_gate& g);  // arithmetic weight of a non-diagonal gate
double cost_transmm(int n, int m, int precision);

// ---- OShareMem lowering ------------------------------------------------------
struct OshmProgram {
    int n = 0, k = 0, r = 0;
    uint64_t tile_mask = 0;          // physical tile bits
    std::vector<OshmPhase> phases;
    std::vector<OshmOp> ops;
};

// Lower gates (PHYSICAL qubits) into phases over the tile `tile_mask`
// (physical, popcount = k, must contain bit 0).  Every non-diagonal target
// must be a tile bit.
OshmProgram plan_oshm(int n, const std::vector<hq_gate>& phys_gates, uint64_t tile_mask);

// Fill the launch parameters (tile-base runs, piece offsets) for a program.
OshmLaunch make_oshm_launch(const OshmProgram& prog, void* state, const OshmPhase* d_phases,
                            const OshmOp* d_ops, int* d_err);

// Pad `mask` (physical) to exactly k bits with the lowest free physical bits.
uint64_t pad_tile(uint64_t mask, int k, int n);

}  // namespace hq
