// Structures shared by host lowering code and the CUDA kernels, and the
// launchers each .cu file exports.  Plain C++ (no CUDA-only types) so that
// g++-compiled host code can include it.
#pragma once

#include <cstdint>

#include "../../include/hyquas_gb300.h"

namespace hq {

// ---- plain path ---------------------------------------------------------
enum PlainKind : int32_t { PK_GENERAL = 0, PK_SWAP = 1, PK_DIAG = 2, PK_DIAG_HI = 3 };

struct PlainGate {
    int32_t kind;
    int32_t target;       // physical bit
    int32_t ninsert;      // number of zero bits inserted (target + controls)
    int32_t insert[3];    // ascending physical positions
    uint64_t setmask;     // control bits forced to 1
    float m[8];           // matrix (re00 im00 re01 im01 re10 im10 re11 im11)
};

// ---- OShareMem tile program ------------------------------------------------
// Op kinds applied to the amplitudes a thread holds in registers.
enum OshmOpKind : uint8_t {
    OP_U = 0,       // general 2x2 on register bit `tbit`
    OP_X = 1,       // exchange lo/hi on register bit `tbit`
    OP_DREG = 2,    // diag(d0,d1) with register target bit `tbit` (d0 = m[0..1], d1 = m[6..7])
    OP_DOUT = 3,    // diag(d0,d1) whose target is outside the register set (physical `tout`)
    OP_RY = 4,      // real 2x2 [[a,-b],[b,a]] on `tbit` (RY, H-like real rotations use OP_REAL)
    OP_REAL = 5     // real 2x2 (m00r m01r m10r m11r in m[0],m[2],m[4],m[6])
};

struct OshmOp {
    uint8_t kind;
    uint8_t tbit;
    uint8_t d0_is_one;  // OP_DREG/OP_DOUT: d0 == 1, lo untouched
    uint8_t pad;
    uint32_t creg;      // register-index control mask
    uint64_t cout;      // physical control mask outside the register set
    uint64_t tout;      // OP_DOUT: physical target bit
    float m[8];
};
static_assert(sizeof(OshmOp) == 56, "OshmOp layout");

constexpr int OSHM_MAX_R = 5;      // register bits per thread (32 amplitudes)
constexpr int OSHM_MAX_K = 13;     // tile bits
constexpr int OSHM_MAX_G = OSHM_MAX_K;  // thread-index bits

struct alignas(16) OshmPhase {
    uint32_t op_begin, op_end;
    uint8_t r_local[OSHM_MAX_R];  // local tile bit of register bit j
    uint8_t g_local[OSHM_MAX_G];  // local tile bit of thread-index bit j
    uint8_t g_phys[OSHM_MAX_G];   // physical bit of thread-index bit j
    uint8_t pair0;                // local bit 0 is register bit 0 (16-byte smem accesses)
};
static_assert(sizeof(OshmPhase) == 48, "OshmPhase layout");

struct OshmProgramHeader {
    int32_t k;            // tile bits
    int32_t r;            // register bits
    int32_t nphases;
    int32_t nops;
    uint64_t tile_mask;   // physical tile bits (bit 0 set)
};

// Launch parameters passed by value.
struct OshmLaunch {
    void* state;                // float2*
    const OshmPhase* phases;    // device
    const OshmOp* ops;          // device
    int* err;
    int32_t n, k, nphases;
    int32_t nruns;              // runs of block (non-tile) bits
    uint8_t run_src[32], run_dst[32], run_len[32];
    uint8_t tile_phys[16];      // physical bit of local tile bit j
    uint64_t piece_off[32];     // per-thread piece m: physical offset of (m * threads) piece
    uint32_t piece_slot[32];    // matching smem slot offsets
    uint64_t ntiles;
};

// ---- launchers (implemented in the .cu files) -------------------------------
void launch_plain_gate(void* state, int n, const PlainGate& g, void* stream);
void launch_init_zero(void* state, int n, void* stream);
// FP64 reductions: writes norm and p1[q] (physical bits) into host memory.
void launch_marginals(const void* state, int n, double* d_partials, size_t cap, double* h_out,
                      void* stream);
void launch_gather(const void* state, const uint64_t* d_phys_idx, int64_t count, void* d_out,
                   void* stream);
// In-place exchange of two physical bits.
void launch_bit_swap(void* state, int n, int a, int b, void* stream);
void launch_oshm(const OshmLaunch& p, void* stream);
int oshm_threads(int k, int r);
int oshm_reg_bits(int k);
uint32_t oshm_swizzle(uint32_t local_index);

}  // namespace hq
