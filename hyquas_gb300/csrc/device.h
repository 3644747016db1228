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
// In a phase every thread holds 32 amplitudes over 5 "register qubits".
// Register index i: bit 0 = the tile's local qubit 0 (physical qubit 0),
// always a register qubit and the lane of the packed f32x2 vectors; bits 1..4
// = four more tile qubits chosen per phase.  Amplitudes are kept as
// structure-of-arrays vectors: re[j] = (re(2j), re(2j+1)), im[j] likewise.
enum OshmOpKind : uint8_t {
    OP_U = 0,      // general complex 2x2 (m = re00 im00 re01 im01 re10 im10 re11 im11)
    OP_REAL = 1,   // real 2x2 (m0, m2, m4, m6)
    OP_IMOFF = 2,  // [[a, i b], [i c, d]], a, b, c, d real (m0, m3, m5, m6)
    OP_H = 3,      // (1/sqrt2) [[1, 1], [1, -1]], scale deferred
    OP_SY = 4,     // (1/sqrt2) [[1, -1], [1, 1]], scale deferred (RY(pi/2))
    OP_SX = 5,     // (1/sqrt2) [[1, -i], [-i, 1]], scale deferred (RX(pi/2))
    OP_X = 6,      // exchange lo/hi
    OP_DREG = 7,   // diag(d0, d1) on a register qubit (d0 = m0 m1, d1 = m6 m7)
    OP_NEGHI = 8,  // diag(1, -1) on a register qubit (Z, CZ)
    OP_DOUT = 9,   // diag(d0, d1) whose target is outside the register set
    OP_DROT = 11,  // diag(1, e^{i phi}) on a register qubit: the high amplitude's
                   // (re, im) rotated by phi in place with three shears
                   // x += a y; y += b x; x += a y (a = -tan(phi/2) = m0, b = sin(phi) = m1),
                   // then negated when OPF_NEG (phi was reduced by pi)
    OP_RROT = 12   // [[c, -s], [s, c]] (RY and the like) on a register qubit J >= 1:
                   // (lo, hi) rotated by phi = atan2(s, c) with the same three shears
                   // in the real and in the imaginary plane (m0, m1, OPF_NEG as DROT)
};
enum OshmOpFlags : uint8_t {
    OPF_D0_ONE = 1,   // diagonal op: d0 == 1
    OPF_COUT = 2,     // has controls outside the register set (`cout`)
    OPF_CREG = 4,     // has controls on register qubits (`creg`)
    OPF_NEG = 8       // OP_DROT, OP_RROT: negate the result
};

struct alignas(16) OshmOp {
    uint8_t kind;
    uint8_t tbit;       // register-index bit of the target (0..4)
    uint8_t flags;
    uint8_t pad0;
    uint32_t creg;      // register-index control mask
    uint64_t cout;      // physical control mask outside the register set
    uint64_t tout;      // OP_DOUT: physical target bit
    uint64_t pad1;
    float m[8];
};
static_assert(sizeof(OshmOp) == 64, "OshmOp layout");

constexpr int OSHM_MAX_R = 5;      // register bits per thread (32 amplitudes)
constexpr int OSHM_MAX_K = 13;     // tile bits
constexpr int OSHM_MAX_G = OSHM_MAX_K;  // thread-index bits

enum OshmPhaseFlags : uint8_t {
    PHF_ACC = 1     // apply the per-thread phase accumulated by OP_DOUT ops
};

struct alignas(16) OshmPhase {
    uint32_t op_begin, op_end;
    uint8_t r_local[OSHM_MAX_R];  // local tile bit of register bit j (r_local[0] == 0)
    uint8_t g_local[OSHM_MAX_G];  // local tile bit of thread-index bit j
    uint8_t g_phys[OSHM_MAX_G];   // physical bit of thread-index bit j
    uint8_t flags;
    float scale;                  // real factor applied at the end of the phase (deferred 1/sqrt2's)
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
struct alignas(16) OshmLaunch {
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

static_assert(sizeof(OshmLaunch) % 16 == 0, "OshmLaunch is copied as 16-byte words");

// ---- batched OShareMem engine -----------------------------------------------------
// One persistent launch serves many circuits.  Work items (circuit, group,
// range of tiles) are handed out in queue order by an atomic counter; an item
// of group g starts when its circuit's completion counter shows every tile of
// groups 0..g-1 written.  Items are queued group level by group level, so an
// item's predecessors were always handed out before it.
enum : uint32_t {
    ITEM_FIRST = 1,  // first group of its circuit: may synthesise |0...0> instead of loading
};
struct BatchItem {
    uint32_t group;    // index of the group's OshmLaunch
    uint32_t circuit;  // completion counter of the circuit
    uint32_t tile0;    // first tile
    uint32_t count;    // tiles
    uint32_t need;     // counter value that must be reached before the item starts
    uint32_t flags;
};
struct BatchLaunch {
    const OshmLaunch* groups;
    const BatchItem* items;
    uint32_t nitems;
    uint32_t zero_init;  // ITEM_FIRST items start from |0...0> (the state is not read)
    uint32_t* head;      // next item to hand out
    uint32_t* done;      // per circuit: tiles finished
    int* err;
    uint32_t stall_item; // test hook: this item waits for a count never reached (~0u: none)
};
constexpr int kBatchTile = 13;  // widest tile of the batched kernel (2^13 amplitudes)
constexpr int kBatchMinTile = 10;  // narrowest: one warp per tile
void launch_oshm_batch(const BatchLaunch& b, int grid, bool cooperative, void* stream);
int oshm_batch_slots();  // resident blocks of the batched kernel on this GPU

// ---- sampling (k_sample.cu) ----------------------------------------------------------
constexpr int kSampleBlockBits = 12;  // amplitudes per block of the cumulative distribution
size_t sample_scratch_doubles(int n);
uint64_t sample_mix64(uint64_t z);   // SplitMix64 output function
// Block CDF into d_cdf, then `shots` physical indices into d_out.
void launch_sample(const void* state, int n, int shots, uint64_t seed, double* d_cdf,
                   uint64_t* d_out, void* stream);

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
// In-place permutation of the physical bits in one pass: the amplitude at index
// x goes to the index whose bit dest_of[b] is bit b of x.  The moved bits and
// the five lowest must number at most kPermuteMaxTileBits.
constexpr int kPermuteMaxTileBits = 13;
int permute_tile_bits(int n, const int* dest_of);
void launch_permute_bits(void* state, int n, const int* dest_of, void* stream);
// bytes from device memory d to a device-mapped pinned host buffer, by `ctas`
// blocks (a few SMs); stream-ordered
void launch_readback(const void* d, void* host_mapped, uint64_t bytes, int ctas, void* stream);
// a zero word in every 4 KB page of a device-mapped host buffer (its first
// device writes), stream-ordered
void launch_touch_pages(void* host_mapped, uint64_t bytes, void* stream);
// the 4-int device error word to a device-mapped host copy, stream-ordered
void launch_error_readout(const int* d_error, int* h_mapped, void* stream);
void launch_oshm(const OshmLaunch& p, void* stream);
int oshm_threads(int k, int r);
int oshm_reg_bits(int k);
uint32_t oshm_swizzle(uint32_t local_index);

}  // namespace hq
