// TransMM: a gate group fused into a 2^m x 2^m unitary and applied as a
// contraction over tiles gathered in place (replaces GateGroup::initMatrix,
// cuttExecute and cublasGEMM, src/executor.cpp:533-551, src/schedule.cpp:578-721).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "executor.h"

namespace hq {

// Local gate record for the FP64 composition kernel (qubits are row bits).
struct ComposeGate {
    int32_t target, control, control2, pad;
    double m[8];
};

struct TransmmLaunch {
    void* state;
    const void* umat;         // operand prepared for the precision (see transmm.cu)
    int* err;
    int32_t n, m, k;          // register, rows (group qubits), tile bits
    int32_t precision;
    uint64_t ntiles;
    int32_t nruns;
    uint8_t run_src[32], run_dst[32], run_len[32];
    uint8_t tile_phys[16];    // physical bit of local tile bit j (ascending)
    uint8_t row_local[8];     // local tile bit of row bit r
    uint8_t col_local[16];    // local tile bit of column bit c
    uint64_t piece_off[32];       // 512-thread piece tables (SIMT kernel)
    uint32_t piece_slot[32];
    // 6-qubit tensor-core kernel: the tile runs as 2 sub-tiles of 64 x 64 with
    // its top column bit fixed, pipelined through three staging buffers
    uint8_t sub_phys[12];         // physical bit of sub-tile local bit j
    uint8_t row_sub[8];           // sub-tile local bit of row bit r
    uint8_t col_sub[8];           // sub-tile local bit of column bit c
    uint64_t split_off[2];        // physical offsets of the fixed top column bits
    uint64_t sub_piece_off[8];    // 256-thread piece tables of a sub-tile
    uint32_t sub_piece_slot[8];
};

void transmm_prepare(int n, const GroupPlan& gp, DeviceGroup& dg, const CompileConfig& cfg,
                     std::vector<double>& umats);
void transmm_finalize(hq_circuit_s* c);
void transmm_launch(hq_circuit_s* c, const DeviceGroup& dg, void* state, cudaStream_t st);

// Compose the FP64 unitary of `gates` (row-bit indices) on the GPU into
// d_u (column-major complex128, 2^m x 2^m).
void compose_unitary(int m, const std::vector<ComposeGate>& gates, double* d_u, cudaStream_t st);
// Apply a device-resident FP64 unitary to a state over the given physical row bits.
void apply_unitary_device(hq_state_s* s, const double* d_u, int m, uint64_t rows_phys,
                          int precision);

// launchers (transmm.cu)
void launch_compose(int m, const ComposeGate* d_gates, int ngates, double* d_u, cudaStream_t st);
void launch_u_to_f32(int m, const double* d_u, void* d_out, cudaStream_t st);
void launch_transmm_simt(const TransmmLaunch& p, cudaStream_t st);
int transmm_tile_bits(int m);

}  // namespace hq
