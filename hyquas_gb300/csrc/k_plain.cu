// Plain-path kernels: one launch per gate (the reference's BACKEND=serial,
// src/kernelSimple.cu:335-446), |0..0> initialisation (src/kernelSimple.cu:9-37),
// FP64 probability reductions (src/kernelSimple.cu:467-516), amplitude gather
// (src/kernelSimple.cu:518-522) and the in-HBM qubit remaps (one bit exchange,
// or a permutation of up to 13 tile bits per pass, in place).
//
// All indices are 64-bit (the reference's `int nVec` overflows at n >= 32,
// src/kernelSimple.cu:338).  Every kernel is HBM-bound.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "common.h"
#include "device.h"

namespace hq {

namespace {

constexpr int kPlainThreads = 256;

__device__ __forceinline__ uint64_t insert_zeros(uint64_t x, const PlainGate& g) {
#pragma unroll
    for (int s = 0; s < 3; s++) {
        if (s < g.ninsert) {
            const int p = g.insert[s];
            x = ((x >> p) << (p + 1)) | (x & ((uint64_t(1) << p) - 1));
        }
    }
    return x;
}

// One gate over the 2^(n - ninsert) (lo, hi) pairs whose control bits are 1.
template <int KIND>
__global__ void __launch_bounds__(kPlainThreads) k_plain_gate(float2* __restrict__ a, uint64_t npairs,
                                                              PlainGate g) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t tbit = uint64_t(1) << g.target;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < npairs; j += stride) {
        const uint64_t lo = insert_zeros(j, g) | g.setmask;
        const uint64_t hi = lo | tbit;
        if (KIND == PK_SWAP) {
            const float2 x = a[lo], y = a[hi];
            a[lo] = y;
            a[hi] = x;
        } else if (KIND == PK_DIAG_HI) {
            const float2 y = a[hi];
            a[hi] = make_float2(y.x * g.m[6] - y.y * g.m[7], y.x * g.m[7] + y.y * g.m[6]);
        } else if (KIND == PK_DIAG) {
            const float2 x = a[lo], y = a[hi];
            a[lo] = make_float2(x.x * g.m[0] - x.y * g.m[1], x.x * g.m[1] + x.y * g.m[0]);
            a[hi] = make_float2(y.x * g.m[6] - y.y * g.m[7], y.x * g.m[7] + y.y * g.m[6]);
        } else {
            const float2 x = a[lo], y = a[hi];
            a[lo] = make_float2(x.x * g.m[0] - x.y * g.m[1] + y.x * g.m[2] - y.y * g.m[3],
                                x.x * g.m[1] + x.y * g.m[0] + y.x * g.m[3] + y.y * g.m[2]);
            a[hi] = make_float2(x.x * g.m[4] - x.y * g.m[5] + y.x * g.m[6] - y.y * g.m[7],
                                x.x * g.m[5] + x.y * g.m[4] + y.x * g.m[7] + y.y * g.m[6]);
        }
    }
}

__global__ void k_set_one(float2* a) { a[0] = make_float2(1.f, 0.f); }

// ---- FP64 marginals ---------------------------------------------------------
// Level 1: each block covers 4096 amplitudes (2048 float4 = 256 threads x 8).
// Output row (13 doubles): [total, p1(bit0), p1(bit1..8) from the thread bits,
// p1(bit9..11) from the iteration bits].  |a|^2 is formed in FP32 per
// amplitude and summed over at most 16 amplitudes in FP32; everything above
// that is FP64.
constexpr int kMargRow1 = 13;
constexpr int kMargRow2 = 25;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* out) {
    __shared__ double red[8][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) v[i] = warp_sum(v[i]);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) red[warp][i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
        out[threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) k_marg_l1(const float4* __restrict__ a, uint64_t nquads,
                                                 double* __restrict__ rows) {
    const int t = threadIdx.x;
    const uint64_t base = uint64_t(blockIdx.x) * 2048;
    float w[8], u[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t q = base + t + 256 * i;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (q < nquads) v = __ldcs(a + q);
        const float w0 = v.x * v.x + v.y * v.y, w1 = v.z * v.z + v.w * v.w;
        w[i] = w0 + w1;
        u[i] = w1;
    }
    float W = 0.f, U = 0.f, I0 = 0.f, I1 = 0.f, I2 = 0.f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        W += w[i];
        U += u[i];
        if (i & 1) I0 += w[i];
        if (i & 2) I1 += w[i];
        if (i & 4) I2 += w[i];
    }
    double v[kMargRow1];
    v[0] = W;
    v[1] = U;
#pragma unroll
    for (int j = 0; j < 8; j++) v[2 + j] = ((t >> j) & 1) ? (double)W : 0.0;
    v[10] = I0;
    v[11] = I1;
    v[12] = I2;
    block_sum<kMargRow1>(v, rows + uint64_t(blockIdx.x) * kMargRow1);
}

// Level 2: each block covers 4096 level-1 rows.  Output row (25 doubles):
// [total, sums of level-1 columns 1..12 (amplitude bits 0..11), marginals of
// the row-index bits 0..11 (amplitude bits 12..23)].
__global__ void __launch_bounds__(256) k_marg_l2(const double* __restrict__ rows1, uint64_t nrows,
                                                 double* __restrict__ rows2) {
    const int t = threadIdx.x;
    const uint64_t base = uint64_t(blockIdx.x) * 4096;
    double C[12], W = 0, I[4] = {0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 12; c++) C[c] = 0;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
        const uint64_t r = base + t + 256 * i;
        if (r >= nrows) continue;
        const double* row = rows1 + r * kMargRow1;
        const double tot = row[0];
        W += tot;
#pragma unroll
        for (int c = 0; c < 12; c++) C[c] += row[1 + c];
#pragma unroll
        for (int b = 0; b < 4; b++)
            if ((i >> b) & 1) I[b] += tot;
    }
    double v[kMargRow2];
    v[0] = W;
#pragma unroll
    for (int c = 0; c < 12; c++) v[1 + c] = C[c];
#pragma unroll
    for (int j = 0; j < 8; j++) v[13 + j] = ((t >> j) & 1) ? W : 0.0;
#pragma unroll
    for (int b = 0; b < 4; b++) v[21 + b] = I[b];
    block_sum<kMargRow2>(v, rows2 + uint64_t(blockIdx.x) * kMargRow2);
}

__global__ void k_gather(const float2* __restrict__ a, const uint64_t* __restrict__ idx, int64_t count,
                         float2* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count) out[i] = a[idx[i]];
}

// Exchange physical bits lo_bit < hi_bit in place: swap a[x | 1<<lo_bit] with
// a[x | 1<<hi_bit] for every x with both bits clear.
__global__ void __launch_bounds__(256) k_bit_swap(float2* __restrict__ a, uint64_t count, int lo_bit,
                                                  int hi_bit) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t lm = (uint64_t(1) << lo_bit) - 1;
    const uint64_t hm = (uint64_t(1) << hi_bit) - 1;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < count; j += stride) {
        uint64_t x = ((j >> lo_bit) << (lo_bit + 1)) | (j & lm);
        x = ((x >> hi_bit) << (hi_bit + 1)) | (x & hm);
        const uint64_t p = x | (uint64_t(1) << lo_bit), q = x | (uint64_t(1) << hi_bit);
        const float2 u = a[p], v = a[q];
        a[p] = v;
        a[q] = u;
    }
}

unsigned grid_for(uint64_t work, int threads) {
    const uint64_t blocks = (work + threads - 1) / threads;
    const uint64_t cap = uint64_t(ctx().sm_count) * 16;
    return (unsigned)(blocks < cap ? (blocks ? blocks : 1) : cap);
}

// Allocation-free variant: the final reduction of the level-2 rows runs on
// the device too, so the whole reduction is stream-ordered and needs no host
// buffer.  Row order and FP64 addition order match launch_marginals.
__global__ void k_marg_final(const double* __restrict__ rows2, uint64_t nb2, int n,
                             double* __restrict__ out) {
    const int b = threadIdx.x;  // b < n: P(bit b = 1); b == n: total
    if (b > n) return;
    double acc = 0.0;
    for (uint64_t r = 0; r < nb2; r++) {
        const double* row = rows2 + r * kMargRow2;
        if (b == n)
            acc += row[0];
        else if (b < 12)
            acc += row[1 + b];
        else if (b < 24)
            acc += row[13 + (b - 12)];
        else if ((r >> (b - 24)) & 1)
            acc += row[0];
    }
    if (b == n)
        out[0] = acc;
    else
        out[1 + b] = acc;
}

}  // namespace

void launch_plain_gate(void* state, int n, const PlainGate& g, void* stream) {
    const uint64_t npairs = uint64_t(1) << (n - g.ninsert);
    const unsigned grid = grid_for(npairs, kPlainThreads);
    cudaStream_t s = (cudaStream_t)stream;
    float2* a = (float2*)state;
    switch (g.kind) {
        case PK_SWAP: k_plain_gate<PK_SWAP><<<grid, kPlainThreads, 0, s>>>(a, npairs, g); break;
        case PK_DIAG: k_plain_gate<PK_DIAG><<<grid, kPlainThreads, 0, s>>>(a, npairs, g); break;
        case PK_DIAG_HI: k_plain_gate<PK_DIAG_HI><<<grid, kPlainThreads, 0, s>>>(a, npairs, g); break;
        default: k_plain_gate<PK_GENERAL><<<grid, kPlainThreads, 0, s>>>(a, npairs, g); break;
    }
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_init_zero(void* state, int n, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    HQ_CHECK_CUDA(cudaMemsetAsync(state, 0, sizeof(float2) << n, s));
    k_set_one<<<1, 1, 0, s>>>((float2*)state);
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_marginals(const void* state, int n, double* d_partials, size_t cap, double* h_out,
                      void* stream) {
    // h_out: [0] = total, [1 + b] = P(bit b = 1) for physical bits b < n.
    HQ_REQUIRE(n >= 1 && n <= 36, HQ_ERR_INVALID, "marginals: n=%d unsupported", n);
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t nquads = (uint64_t(1) << n) / 2;
    const uint64_t nb1 = (nquads + 2047) / 2048;
    const uint64_t nb2 = (nb1 + 4095) / 4096;
    HQ_REQUIRE(nb1 * kMargRow1 + nb2 * kMargRow2 <= cap, HQ_ERR_INVALID,
               "marginals: scratch too small");
    double* rows1 = d_partials;
    double* rows2 = d_partials + nb1 * kMargRow1;
    k_marg_l1<<<(unsigned)nb1, 256, 0, s>>>((const float4*)state, nquads, rows1);
    HQ_CHECK_CUDA(cudaGetLastError());
    k_marg_l2<<<(unsigned)nb2, 256, 0, s>>>(rows1, nb1, rows2);
    HQ_CHECK_CUDA(cudaGetLastError());
    double* h = ctx().h_pinned;
    HQ_REQUIRE(nb2 * kMargRow2 <= ctx().pinned_cap, HQ_ERR_INVALID, "marginals: pinned too small");
    HQ_CHECK_CUDA(cudaMemcpyAsync(h, rows2, sizeof(double) * nb2 * kMargRow2,
                                  cudaMemcpyDeviceToHost, s));
    HQ_CHECK_CUDA(cudaStreamSynchronize(s));
    double out[1 + 64] = {0};
    for (uint64_t r = 0; r < nb2; r++) {
        const double* row = h + r * kMargRow2;
        out[0] += row[0];
        for (int b = 0; b < 12; b++) out[1 + b] += row[1 + b];
        for (int b = 0; b < 12; b++) out[1 + 12 + b] += row[13 + b];
        for (int b = 24; b < n; b++)
            if ((r >> (b - 24)) & 1) out[1 + b] += row[0];
    }
    for (int b = 0; b <= n; b++) h_out[b] = out[b];
}

void launch_gather(const void* state, const uint64_t* d_idx, int64_t count, void* d_out,
                   void* stream) {
    if (count <= 0) return;
    const unsigned grid = (unsigned)((count + 255) / 256);
    k_gather<<<grid, 256, 0, (cudaStream_t)stream>>>((const float2*)state, d_idx, count,
                                                     (float2*)d_out);
    HQ_CHECK_CUDA(cudaGetLastError());
}

// ---- in-place qubit remap, many bits per pass ---------------------------------------
//
// The single-GPU form of the reference's layout change (src/executor.cpp:59-179,
// a local transpose plus an all-to-all).  One pass applies a permutation of the
// physical bits that moves at most a tile's worth of them: every amplitude goes
// from index x to the index whose bit dest_of[b] is bit b of x.  A CTA owns a
// tile of up to 2^13 amplitudes over the moved bits and the five lowest bits
// (padded with the next lowest); every other bit stays where it is, so a tile
// maps onto itself and the pass runs in place.  The tile is read in source
// order (the five lowest bits contiguous: whole 256-byte runs) into shared
// memory and written back in destination order (again 256-byte runs); slots
// are XOR-swizzled so the destination-order reads spread over the banks.
// One read and one write of each amplitude in the tiles the pass touches.
struct PermuteParams {
    // offsets of the local index bits 0-4 / 5-9 / 10-12 in the source and the
    // destination; write-order index -> local index; slot swizzle of bits 5-12
    uint64_t src_lo[32], src_mid[32], src_hi[8];
    uint64_t dst_lo[32], dst_mid[32], dst_hi[8];
    uint16_t wr_lo[32], wr_mid[32], wr_hi[8];
    uint16_t swz_mid[32], swz_hi[8];
    // write-order index w -> destination offset / smem read slot, composed
    // (the destination of local index wr(w), the slot of wr(w)); both are
    // bit-linear in w, so three tables per map
    uint64_t wdst_lo[32], wdst_mid[32], wdst_hi[8];
    uint16_t wslot_lo[32], wslot_mid[32], wslot_hi[8];
    uint8_t rest[64];   // tile-index bit r -> its (unmoved) physical bit
    int nrest;
    // the tile index's bits as runs: (u >> run_src) & (2^run_len - 1) lands at run_dst
    uint8_t run_src[32], run_dst[32], run_len[32];
    int nruns;
    int pair_read;      // write-order bit 0 is local bit 0: index pairs are slot pairs
    int tile_bits;
    uint64_t ntiles;
};

// Any tile size (used below 2^10 amplitudes): one amplitude per access.
__global__ void __launch_bounds__(256) k_permute_bits(float2* __restrict__ a,
                                                      const __grid_constant__ PermuteParams p) {
    extern __shared__ float2 tile[];
    const int len = 1 << p.tile_bits;
    for (uint64_t u = blockIdx.x; u < p.ntiles; u += gridDim.x) {
        uint64_t base = 0;
        for (int r = 0; r < p.nrest; r++) base |= ((u >> r) & 1) << p.rest[r];
        for (int e = threadIdx.x; e < len; e += 256) {
            const float2 v = a[base + p.src_lo[e & 31] + p.src_mid[(e >> 5) & 31] + p.src_hi[e >> 10]];
            tile[e ^ p.swz_mid[(e >> 5) & 31] ^ p.swz_hi[e >> 10]] = v;
        }
        __syncthreads();
        for (int w = threadIdx.x; w < len; w += 256) {
            const int j = p.wr_lo[w & 31] | p.wr_mid[(w >> 5) & 31] | p.wr_hi[w >> 10];
            a[base + p.dst_lo[j & 31] + p.dst_mid[(j >> 5) & 31] + p.dst_hi[j >> 10]] =
                tile[j ^ p.swz_mid[(j >> 5) & 31] ^ p.swz_hi[j >> 10]];
        }
        __syncthreads();
    }
}

// Tiles of 2^K amplitudes, K = 10..13: 16-byte accesses (local index bit 0 is
// source bit 0 and write-order bit 0 lands on destination bit 0, so index
// pairs 2i, 2i+1 are neighbours on both sides), and every load of a tile is
// issued before the first shared-memory store so that 2^K / 512 loads per
// thread can be in flight at once.
template <int K>
__global__ void __launch_bounds__(256) k_permute_tile(float2* __restrict__ a,
                                                      const __grid_constant__ PermuteParams p) {
    constexpr int PP = (1 << K) / 512;  // index pairs per thread
    extern __shared__ float2 tile[];
    const int t = threadIdx.x;
    // Thread t moves index pairs e = 2t + 512m (m < PP) on both sides.  The
    // maps are bit-linear, so their per-thread parts (index bits 0-9, the
    // same for every tile) are looked up once here; bits 10-12 come from m
    // and read the same table entry in every lane.
    const int lo = (2 * t) & 31, mid = (2 * t) >> 5;
    const uint64_t src0 = p.src_lo[lo] + p.src_mid[mid], src1 = p.src_lo[lo] + p.src_mid[mid + 16];
    const uint64_t dst0 = p.wdst_lo[lo] + p.wdst_mid[mid], dst1 = p.wdst_lo[lo] + p.wdst_mid[mid + 16];
    const unsigned st0 = (2 * t) ^ p.swz_mid[mid], st1 = (2 * t) ^ p.swz_mid[mid + 16];
    const unsigned rd0 = p.wslot_lo[lo] ^ p.wslot_mid[mid], rd1 = p.wslot_lo[lo] ^ p.wslot_mid[mid + 16];
    const unsigned rd_pair = p.wslot_lo[1];  // slot of write index w + 1 relative to w
    for (uint64_t u = blockIdx.x; u < p.ntiles; u += gridDim.x) {
        uint64_t base = 0;
        for (int r = 0; r < p.nruns; r++)
            base |= ((u >> p.run_src[r]) & ((uint64_t(1) << p.run_len[r]) - 1)) << p.run_dst[r];
        float4 v[PP];
#pragma unroll
        for (int m = 0; m < PP; m++)
            v[m] = __ldcs(reinterpret_cast<const float4*>(a + base + ((m & 1) ? src1 : src0) + p.src_hi[m >> 1]));
        // the swizzle leaves slot bit 0 alone: index pair (e, e + 1) is slot pair
        // (slot(e), slot(e) + 1), one 16-byte store
#pragma unroll
        for (int m = 0; m < PP; m++)
            *reinterpret_cast<float4*>(tile + (((m & 1) ? st1 : st0) ^ (512u * m) ^ p.swz_hi[m >> 1])) = v[m];
        __syncthreads();
#pragma unroll
        for (int m = 0; m < PP; m++) {
            const unsigned r0 = ((m & 1) ? rd1 : rd0) ^ p.wslot_hi[m >> 1];
            float4 x;
            if (p.pair_read) {
                x = *reinterpret_cast<const float4*>(tile + r0);
            } else {
                const float2 x0 = tile[r0], x1 = tile[r0 ^ rd_pair];
                x = make_float4(x0.x, x0.y, x1.x, x1.y);
            }
            __stcs(reinterpret_cast<float4*>(a + base + ((m & 1) ? dst1 : dst0) + p.wdst_hi[m >> 1]), x);
        }
        __syncthreads();
    }
}

// One word per 4 KB page of a freshly registered host buffer, written through
// its device mapping: the first device writes to each page are slow (on GB300
// the first 8 GiB readback into a new buffer took about 0.57 s, later ones
// 45 ms), so they happen when the buffer is made.
__global__ void k_touch_pages(unsigned int* __restrict__ p, uint64_t words, uint64_t step) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i * step < words; i += stride)
        p[i * step] = 0u;
}

void launch_touch_pages(void* host_mapped, uint64_t bytes, void* stream) {
    const uint64_t words = bytes / 4;
    if (words == 0) return;
    k_touch_pages<<<256, 256, 0, (cudaStream_t)stream>>>((unsigned int*)host_mapped, words, 1024);
    HQ_CHECK_CUDA(cudaGetLastError());
}

__global__ void k_error_readout(const int* __restrict__ d, int* __restrict__ h) {
    if (threadIdx.x < 4) h[threadIdx.x] = d[threadIdx.x];
}

void launch_error_readout(const int* d_error, int* h_mapped, void* stream) {
    k_error_readout<<<1, 32, 0, (cudaStream_t)stream>>>(d_error, h_mapped);
    HQ_CHECK_CUDA(cudaGetLastError());
}

// Device -> pinned host copy run by a few SMs: 16-byte streaming loads from
// HBM and plain stores through the host mapping, four per thread in flight.
__global__ void __launch_bounds__(512) k_readback(const float4* __restrict__ src,
                                                  float4* __restrict__ dst, uint64_t n4) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        const float4 a = __ldcs(src + i), b = __ldcs(src + i + stride), c = __ldcs(src + i + 2 * stride),
                     d = __ldcs(src + i + 3 * stride);
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n4; i += stride) dst[i] = __ldcs(src + i);
}

void launch_readback(const void* d, void* host_mapped, uint64_t bytes, int ctas, void* stream) {
    HQ_REQUIRE(bytes % 16 == 0 && ((uintptr_t)d % 16) == 0 && ((uintptr_t)host_mapped % 16) == 0,
               HQ_ERR_INVALID, "readback: 16-byte aligned buffers and size");
    k_readback<<<ctas, 512, 0, (cudaStream_t)stream>>>((const float4*)d, (float4*)host_mapped, bytes / 16);
    HQ_CHECK_CUDA(cudaGetLastError());
}

int permute_tile_bits(int n, const int* dest_of) {
    uint64_t t = 0;
    for (int b = 0; b < n && b < 5; b++) t |= uint64_t(1) << b;
    for (int b = 0; b < n; b++)
        if (dest_of[b] != b) t |= uint64_t(1) << b;
    const int need = popcount64(t), floor_bits = n < 10 ? n : 10;
    return need > floor_bits ? need : floor_bits;
}

PermuteParams make_permute_params(int n, const int* dest_of) {
    PermuteParams p;
    std::memset(&p, 0, sizeof(p));
    const int K = permute_tile_bits(n, dest_of), c = n < 5 ? n : 5;
    HQ_REQUIRE(K <= kPermuteMaxTileBits, HQ_ERR_INVALID, "remap pass moves too many bits");
    int src_of[64];
    for (int b = 0; b < n; b++) src_of[dest_of[b]] = b;
    // local bits: source bits 0..c-1, the moved bits, then the lowest others
    int loc_src[kPermuteMaxTileBits], nl = 0;
    uint64_t used = 0;
    auto take = [&](int b) {
        if (nl < K && !((used >> b) & 1)) {
            loc_src[nl++] = b;
            used |= uint64_t(1) << b;
        }
    };
    for (int b = 0; b < c; b++) take(b);
    for (int b = 0; b < n; b++)
        if (dest_of[b] != b) take(b);
    for (int b = 0; b < n && nl < K; b++) take(b);
    // every bit outside the tile stays put: the tile maps onto itself
    for (int b = 0; b < n; b++)
        HQ_REQUIRE(((used >> b) & 1) || dest_of[b] == b, HQ_ERR_INVALID, "remap tile not closed");
    auto fill = [&](uint64_t* t, int nent, int first, bool dst) {
        for (int j = 0; j < nent; j++)
            for (int b = 0; (1 << b) <= j; b++)
                if (((j >> b) & 1) && first + b < K)
                    t[j] |= uint64_t(1) << (dst ? dest_of[loc_src[first + b]] : loc_src[first + b]);
    };
    fill(p.src_lo, 32, 0, false);
    fill(p.src_mid, 32, 5, false);
    fill(p.src_hi, 8, 10, false);
    fill(p.dst_lo, 32, 0, true);
    fill(p.dst_mid, 32, 5, true);
    fill(p.dst_hi, 8, 10, true);
    // write order: the local bits that land on destination bits 0..c-1 first
    int wbit[kPermuteMaxTileBits], nw = 0;
    uint32_t wused = 0;
    for (int d = 0; d < c; d++)
        for (int j = 0; j < K; j++)
            if (loc_src[j] == src_of[d]) {
                wbit[nw++] = j;
                wused |= 1u << j;
            }
    for (int j = 0; j < K; j++)
        if (!((wused >> j) & 1)) wbit[nw++] = j;
    auto fillw = [&](uint16_t* t, int nent, int first) {
        for (int w = 0; w < nent; w++)
            for (int b = 0; (1 << b) <= w; b++)
                if (((w >> b) & 1) && first + b < K) t[w] |= uint16_t(1) << wbit[first + b];
    };
    fillw(p.wr_lo, 32, 0);
    fillw(p.wr_mid, 32, 5);
    fillw(p.wr_hi, 8, 10);
    // swizzle: local bits >= 5 that vary across a destination-order warp fold
    // onto slot bits 1-4 that do not vary there; the other high bits fold onto
    // slot bits 1-4 in turn.  Slot bit 0 is never folded, so index pairs
    // (2i, 2i + 1) stay slot pairs.
    int target[kPermuteMaxTileBits];
    for (int j = 0; j < K; j++) target[j] = -1;
    uint32_t taken = 1u;
    for (int b = 0; b < c && b < nw; b++)
        if (wbit[b] < 5) taken |= 1u << wbit[b];
    for (int b = 0; b < c && b < nw; b++)
        if (wbit[b] >= 5)
            for (int f = 1; f < 5; f++)
                if (!((taken >> f) & 1)) {
                    target[wbit[b]] = f;
                    taken |= 1u << f;
                    break;
                }
    for (int j = 5; j < K; j++)
        if (target[j] < 0) target[j] = 1 + (j - 5) % 4;
    p.pair_read = (nw > 0 && wbit[0] == 0) ? 1 : 0;
    for (int m = 0; m < 32; m++)
        for (int b = 0; b < 5; b++)
            if (((m >> b) & 1) && 5 + b < K) p.swz_mid[m] ^= uint16_t(1) << target[5 + b];
    for (int m = 0; m < 8; m++)
        for (int b = 0; b < 3; b++)
            if (((m >> b) & 1) && 10 + b < K) p.swz_hi[m] ^= uint16_t(1) << target[10 + b];
    // composed write-side maps, one entry per write-order bit
    uint64_t wd[kPermuteMaxTileBits];
    uint16_t ws[kPermuteMaxTileBits];
    for (int b = 0; b < K; b++) {
        const int j = wbit[b];  // local bit written at write-order bit b
        wd[b] = uint64_t(1) << dest_of[loc_src[j]];
        uint16_t sl = uint16_t(1u << j);
        if (j >= 5 && j < 10) sl ^= p.swz_mid[1 << (j - 5)];
        if (j >= 10) sl ^= p.swz_hi[1 << (j - 10)];
        ws[b] = sl;
    }
    auto fillc = [&](uint64_t* d, uint16_t* sl, int nent, int first) {
        for (int w = 0; w < nent; w++)
            for (int b = 0; (1 << b) <= w; b++)
                if (((w >> b) & 1) && first + b < K) {
                    d[w] += wd[first + b];
                    sl[w] ^= ws[first + b];
                }
    };
    fillc(p.wdst_lo, p.wslot_lo, 32, 0);
    fillc(p.wdst_mid, p.wslot_mid, 32, 5);
    fillc(p.wdst_hi, p.wslot_hi, 8, 10);
    p.tile_bits = K;
    p.nrest = 0;
    for (int b = 0; b < n; b++)
        if (!((used >> b) & 1)) p.rest[p.nrest++] = (uint8_t)b;
    p.nruns = 0;
    for (int r = 0; r < p.nrest;) {
        int len = 1;
        while (r + len < p.nrest && p.rest[r + len] == p.rest[r] + len) len++;
        p.run_src[p.nruns] = (uint8_t)r;
        p.run_dst[p.nruns] = p.rest[r];
        p.run_len[p.nruns] = (uint8_t)len;
        p.nruns++;
        r += len;
    }
    p.ntiles = uint64_t(1) << (n - K);
    return p;
}

template <int K>
void launch_permute_tile(void* state, const PermuteParams& p, cudaStream_t st) {
    const int smem = int(sizeof(float2) << K);
    static std::once_flag once;
    static int per_sm = 1;
    std::call_once(once, [&] {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_permute_tile<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        HQ_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_permute_tile<K>, 256, smem));
        if (per_sm < 1) per_sm = 1;
    });
    const uint64_t cap = uint64_t(ctx().sm_count) * per_sm;
    const unsigned grid = (unsigned)(p.ntiles < cap ? p.ntiles : cap);
    k_permute_tile<K><<<grid, 256, smem, st>>>((float2*)state, p);
}

void launch_permute_bits(void* state, int n, const int* dest_of, void* stream) {
    const PermuteParams p = make_permute_params(n, dest_of);
    cudaStream_t st = (cudaStream_t)stream;
    switch (p.tile_bits) {
        case 10: launch_permute_tile<10>(state, p, st); break;
        case 11: launch_permute_tile<11>(state, p, st); break;
        case 12: launch_permute_tile<12>(state, p, st); break;
        case 13: launch_permute_tile<13>(state, p, st); break;
        default: {
            const size_t smem = sizeof(float2) << p.tile_bits;  // at most 8 KiB here
            const uint64_t cap = uint64_t(ctx().sm_count) * 4;
            const unsigned grid = (unsigned)(p.ntiles < cap ? p.ntiles : cap);
            k_permute_bits<<<grid, 256, smem, st>>>((float2*)state, p);
        }
    }
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_bit_swap(void* state, int n, int a, int b, void* stream) {
    if (a == b) return;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const uint64_t count = uint64_t(1) << (n - 2);
    k_bit_swap<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>((float2*)state, count, lo, hi);
    HQ_CHECK_CUDA(cudaGetLastError());
}

// ---- allocation-free marginals ------------------------------------------------
//
// For callers that cannot call cudaMalloc: code whose device memory is owned
// by another allocator (a framework's caching pool or an admission budget
// that has already handed out every byte of HBM), and latency-critical
// paths where cudaMalloc's implicit device synchronisation is not allowed.
// They pass the state and a device output buffer; the reduction partials
// live in the static array below, which every GPU that loads this library
// holds until the process exits.

constexpr int kNoAllocMaxQubits = 26;
constexpr uint64_t kNoAllocRows1 = (uint64_t(1) << (kNoAllocMaxQubits - 1)) / 2048;  // 16384
constexpr uint64_t kNoAllocRows2 = (kNoAllocRows1 + 4095) / 4096;                    // 4
constexpr uint64_t kNoAllocDoubles = kNoAllocRows1 * kMargRow1 + kNoAllocRows2 * kMargRow2;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];  // 1.6 MiB

// Host-side address of g_noalloc_scratch on each device: the array's name in
// host code is only a stand-in, so the address is looked up once per device,
// with that device current, by the first call made on it.
static std::mutex g_noalloc_mu;
static double* g_noalloc_dev_ptr[128];

static double* noalloc_scratch_current_device() {
    int dev = -1;
    HQ_CHECK_CUDA(cudaGetDevice(&dev));
    HQ_REQUIRE(dev >= 0 && dev < 128, HQ_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_dev_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        HQ_REQUIRE(e == cudaSuccess, HQ_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s",
                   cudaGetErrorString(e));
        g_noalloc_dev_ptr[dev] = (double*)p;
    }
    return g_noalloc_dev_ptr[dev];
}

}  // namespace hq

extern "C" hq_status hq_marginals_noalloc(const void* d_state, int32_t num_qubits, double* d_out,
                                          void* stream) {
    using namespace hq;
    try {
        clear_last_error();
        HQ_REQUIRE(d_state != nullptr && d_out != nullptr, HQ_ERR_INVALID,
                   "d_state and d_out must not be NULL");
        HQ_REQUIRE(num_qubits >= 1 && num_qubits <= kNoAllocMaxQubits, HQ_ERR_INVALID,
                   "num_qubits %d outside the allocation-free range [1,%d] (static scratch of %llu "
                   "doubles)",
                   num_qubits, kNoAllocMaxQubits, (unsigned long long)kNoAllocDoubles);
        HQ_REQUIRE(((uintptr_t)d_state & 15) == 0 && ((uintptr_t)d_out & 7) == 0, HQ_ERR_INVALID,
                   "d_state must be 16-byte and d_out 8-byte aligned");
        {
            // The scratch address is per device: a state on another device
            // (or in another context) would pair with the wrong array.
            int dev = -1;
            HQ_CHECK_CUDA(cudaGetDevice(&dev));
            cudaPointerAttributes attr{};
            HQ_CHECK_CUDA(cudaPointerGetAttributes(&attr, d_state));
            HQ_REQUIRE(attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged,
                       HQ_ERR_INVALID, "d_state is not device memory");
            HQ_REQUIRE(attr.device == dev, HQ_ERR_INVALID,
                       "d_state lives on device %d but device %d is current", attr.device, dev);
        }
        double* scratch = noalloc_scratch_current_device();
        cudaStream_t st = (cudaStream_t)stream;
        const int n = num_qubits;
        const uint64_t nquads = (uint64_t(1) << n) / 2;
        const uint64_t nb1 = (nquads + 2047) / 2048;
        const uint64_t nb2 = (nb1 + 4095) / 4096;
        double* rows1 = scratch;                    // every row read below is written first
        double* rows2 = scratch + nb1 * kMargRow1;  // by this call: nothing needs clearing
        k_marg_l1<<<(unsigned)nb1, 256, 0, st>>>((const float4*)d_state, nquads, rows1);
        k_marg_l2<<<(unsigned)nb2, 256, 0, st>>>(rows1, nb1, rows2);
        k_marg_final<<<1, 64, 0, st>>>(rows2, nb2, n, d_out);
        HQ_CHECK_CUDA(cudaGetLastError());
    } catch (const Failure& f) {
        set_last_error(f.what());
        return f.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HQ_ERR_INVALID;
    }
    return HQ_OK;
}
