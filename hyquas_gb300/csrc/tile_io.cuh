// Tile staging shared by the OShareMem and TransMM kernels.
//
// A tile is the set of 2^K amplitudes whose indices agree on every non-tile
// ("block") bit.  Local tile index bit j <-> the j-th lowest physical tile bit.
// Physical bit 0 is always a tile bit, so local amplitudes (2q, 2q+1) are
// adjacent in HBM and are moved as one 16-byte piece.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace hq {

// Linear, involutive shared-memory swizzle on local tile indices (K <= 14):
// bits 1..3 are XORed with a fold of bits >= 4 (bit b >= 4 lands on bit
// 1 + (b-4) % 3).  Bit 0 is never touched, so pieces stay 16-byte aligned.
__host__ __device__ __forceinline__ uint32_t tile_swz(uint32_t x) {
    const uint32_t f = ((x >> 4) ^ (x >> 7) ^ (x >> 10) ^ (x >> 13)) & 7u;
    return x ^ (f << 1);
}

// Physical index of the tile's local amplitude 0: deposit of the tile number
// into the block bits, given as runs (src bit in the tile number, dst bit, length).
__device__ __forceinline__ uint64_t tile_base(uint64_t u, int nruns, const uint8_t* src,
                                              const uint8_t* dst, const uint8_t* len) {
    uint64_t base = 0;
    for (int i = 0; i < nruns; i++)
        base |= ((u >> src[i]) & ((uint64_t(1) << len[i]) - 1)) << dst[i];
    return base;
}

// Physical offset of a local tile index.
__device__ __forceinline__ uint64_t local_to_phys(uint32_t x, int K, const uint8_t* tile_phys) {
    uint64_t off = 0;
    for (int j = 0; j < K; j++)
        if ((x >> j) & 1) off |= uint64_t(1) << tile_phys[j];
    return off;
}

__device__ __forceinline__ void cp_async16(uint32_t smem_addr, const void* gptr) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr), "l"(gptr) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

}  // namespace hq
