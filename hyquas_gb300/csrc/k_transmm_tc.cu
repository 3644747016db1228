// Tensor-core TransMM contraction for sm_103a (tcgen05 + TMEM).
//
// A group of m = 6 qubits fused into a 64x64 complex unitary U is applied to
// every tile of 2^13 amplitudes gathered in place (rows = the group's qubits,
// columns = 128 other qubits), each half of 64 columns as the real-form GEMM
//
//     [Cr; Ci] (128 x 64) = [[Ur, -Ui], [Ui, Ur]] (128 x 128) . [Br; Bi] (128 x 64)
//
// on the 5th-generation tensor cores: operands in shared memory (K-major,
// canonical 8x16-byte core matrices, no swizzle), the FP32 accumulator in
// tensor memory, MMAs issued by one thread and completed through an mbarrier.
//   HQ_MM_BF16X3: U and B split into hi + lo BF16; D = Uhi.Bhi + Uhi.Blo +
//                 Ulo.Bhi (the lo.lo product, ~2^-16 relative, is dropped).
//   HQ_MM_TF32:   one product with TF32-rounded operands.
// Replaces the reference's cuTT transpose + cublasZgemm/Cgemm
// (src/executor.cpp:533-551): the transpose is folded into the tile gather.
//
// Every wait is bounded: on expiry the kernel records an error word (read by
// the host as HQ_ERR_TIMEOUT), frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "common.h"
#include "tile_io.cuh"
#include "transmm.h"

namespace hq {

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_TILE_BITS = 13;
constexpr int TC_ROWS = 64;       // 2^m, m = 6
constexpr int TC_NSUB = 64;       // columns of a sub-tile (half of the tile's 128)
constexpr uint32_t SUB_BYTES = 32768;  // a sub-tile, float2[4096]
constexpr uint32_t SM_A = 0;           // A operand, 64 KB
constexpr uint32_t SM_B = 65536;       // B operand, two buffers of 32 KB
constexpr uint32_t SM_R = 131072;      // sub-tile staging, three buffers of 32 KB
constexpr uint32_t SM_MISC = 229376;   // mbarriers, TMEM slot, row/column slot tables
constexpr uint32_t SM_TOTAL = SM_MISC + 1024;
constexpr uint32_t TMEM_COLS = 128;    // two accumulators of 64 columns
constexpr uint32_t kWaitLimit = 1u << 22;  // bounded mbarrier polls (with nanosleep)
static_assert(SM_TOTAL <= 232448, "shared memory per block");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets >> 4, version 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
           ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor: F32 accumulator, A/B format, K-major A and B, N, M.
__host__ __device__ constexpr uint32_t make_idesc(uint32_t ab_format, uint32_t M, uint32_t N) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_test(uint32_t addr, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        if (mbar_test(addr, parity)) return true;
        __nanosleep(32);
    }
    return false;
}

// The group's A operand (contiguous, a multiple of 16 KB) copied to shared
// memory by the TMA engine: one thread arms the mbarrier at s_bar with the
// byte count and issues bulk copies that complete on it.
__device__ __forceinline__ void bulk_load(uint32_t sdst, const void* gsrc, uint32_t bytes,
                                          uint32_t s_bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(s_bar), "r"(bytes)
                 : "memory");
    for (uint32_t off = 0; off < bytes; off += 16384u)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                sdst + off),
            "l"(reinterpret_cast<const char*>(gsrc) + off), "r"(16384u), "r"(s_bar)
            : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
          "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
          "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
          "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Byte offset of element (row, k) in a K-major no-swizzle operand with
// `kdim` K-elements of `esize` bytes per row.
__host__ __device__ __forceinline__ uint32_t kmajor_off(uint32_t row, uint32_t k, uint32_t kdim,
                                                        uint32_t esize) {
    const uint32_t per_core = 16 / esize;  // K-elements per 16-byte core row
    const uint32_t sbo = (kdim / per_core) * 128;
    return (row / 8) * sbo + (k / per_core) * 128 + (row % 8) * 16 + (k % per_core) * esize;
}

// One CTA per SM runs a pipeline over its sub-tiles j (64 rows x 64 columns):
//   load j+2 (cp.async) | convert j -> B[j&1], MMA j -> TMEM acc[j&1] | epilogue j-1
// Sub-tile j is staged in R[j%3]; its results are written back over it (the
// raw amplitudes are dead once converted) and stored to HBM from there.
template <int PREC>
__global__ void __launch_bounds__(TC_THREADS, 1) k_transmm_tc(const TransmmLaunch p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(smem + SM_MISC + 64);
    uint32_t* colslot = rowslot + TC_ROWS;
    const uint32_t sb = smem_u32(smem);
    const uint32_t s_mbar = sb + SM_MISC;         // two mbarriers, 8 bytes each
    const uint32_t s_tslot = sb + SM_MISC + 16;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_tslot),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar + 8));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar + 24));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    // the group's A operand (prepared once per circuit), 64 KB, by the TMA engine
    if (t == 0) bulk_load(sb + SM_A, p.umat, 65536u, s_mbar + 24);
    for (int r = t; r < TC_ROWS; r += TC_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 6; b++)
            if ((r >> b) & 1) x |= 1u << p.row_sub[b];
        rowslot[r] = tile_swz(x);
    }
    for (int c = t; c < TC_NSUB; c += TC_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 6; b++)
            if ((c >> b) & 1) x |= 1u << p.col_sub[b];
        colslot[c] = tile_swz(x);
    }
    const bool a_ok = mbar_wait(s_mbar + 24, 0);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    const bool a_failed = __syncthreads_or(!a_ok);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (a_failed && t == 0 && p.err) {
        atomicCAS(p.err, 0, 1);
        p.err[1] = 9;  // site: TransMM operand load
    }
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + SM_MISC + 16);

    const uint64_t toff = local_to_phys(uint32_t(t) << 1, TC_TILE_BITS - 1, p.sub_phys);
    const uint32_t tsl = tile_swz(uint32_t(t) << 1);
    constexpr uint32_t esize = PREC == HQ_MM_TF32 ? 4 : 2;
    constexpr uint32_t kstep_bytes = 256;  // 16 bf16 or 8 tf32 K-elements = two core matrices
    constexpr uint32_t sbo = (128 / (16 / esize)) * 128;
    constexpr uint32_t b_lo = 16384;       // B lo half (BF16x3): 64 rows x 128 K bf16
    constexpr uint32_t idesc = make_idesc(PREC == HQ_MM_TF32 ? 2u : 1u, 128, TC_NSUB);
    constexpr int nsteps = PREC == HQ_MM_TF32 ? 16 : 8;

    const uint64_t nsub = p.ntiles * 2;
    const uint64_t G = gridDim.x;
    const uint64_t J = blockIdx.x < nsub ? (nsub - blockIdx.x + G - 1) / G : 0;
    auto sub_base = [&](uint64_t j) {
        const uint64_t v = blockIdx.x + j * G;
        return tile_base(v >> 1, p.nruns, p.run_src, p.run_dst, p.run_len) + (v & 1) * p.split_off[0];
    };
    auto load = [&](uint64_t j) {
        if (j < J) {
            const float2* gsrc = state + sub_base(j) + toff;
            const uint32_t rb = sb + SM_R + uint32_t(j % 3) * SUB_BYTES;
#pragma unroll
            for (int m = 0; m < 8; m++)
                cp_async16(rb + (tsl ^ p.sub_piece_slot[m]) * 8u, gsrc + p.sub_piece_off[m]);
        }
        cp_async_commit();
    };
    // results of sub-tile j: TMEM acc[j&1] -> over its staging buffer -> HBM
    bool failed = a_failed;
    auto epilogue = [&](uint64_t j) {
        const uint32_t b = uint32_t(j & 1);
        const bool ok = mbar_wait(s_mbar + 8 * b, uint32_t((j >> 1) & 1));
        if (__syncthreads_or(!ok)) {
            if (t == 0 && p.err) {
                atomicCAS(p.err, 0, 1);
                p.err[1] = 7;  // site: TransMM accumulator wait
                p.err[2] = (int)(j & 0x7fffffff);
            }
            failed = true;
            return;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // D row i = TMEM lane i: i < 64 the real part of row i, else the imaginary part of row i-64
        float* Rf = reinterpret_cast<float*>(smem + SM_R + uint32_t(j % 3) * SUB_BYTES);
        {
            const int q = warp & 3, half = warp >> 2;
            const int i = 32 * q + lane;
            const uint32_t rs = rowslot[i & 63], comp = uint32_t(i >> 6);
            uint32_t v[32];
            tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + b * TC_NSUB + 32 * half, v);
#pragma unroll
            for (int c = 0; c < 32; c++) Rf[2 * (rs ^ colslot[32 * half + c]) + comp] = __uint_as_float(v[c]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        float2* gdst = state + sub_base(j) + toff;
        const float4* R4 = reinterpret_cast<const float4*>(Rf);
#pragma unroll
        for (int m = 0; m < 8; m++)
            *reinterpret_cast<float4*>(gdst + p.sub_piece_off[m]) = R4[(tsl ^ p.sub_piece_slot[m]) >> 1];
        __syncthreads();
    };

    if (!failed) {
        load(0);
        load(1);
    }
    for (uint64_t j = 0; j < J && !failed; j++) {
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        // B operand of sub-tile j: column n; K index k = component * 64 + row
        {
            const float2* Rj = reinterpret_cast<const float2*>(smem + SM_R + uint32_t(j % 3) * SUB_BYTES);
            unsigned char* B = smem + SM_B + uint32_t(j & 1) * 32768u;
            const int n = t & 63;
            const uint32_t cs = colslot[n];
            for (int rb = 2 * (t >> 6); rb < 2 * (t >> 6) + 2; rb++) {
                float re[8], im[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const float2 a = Rj[rowslot[rb * 8 + q] ^ cs];
                    re[q] = a.x;
                    im[q] = a.y;
                }
                if (PREC == HQ_MM_TF32) {
#pragma unroll
                    for (int half = 0; half < 2; half++) {
                        const uint32_t ore = kmajor_off(n, rb * 8 + half * 4, 128, 4);
                        const uint32_t oim = kmajor_off(n, 64 + rb * 8 + half * 4, 128, 4);
                        *reinterpret_cast<float4*>(B + ore) =
                            make_float4(to_tf32(re[4 * half]), to_tf32(re[4 * half + 1]),
                                        to_tf32(re[4 * half + 2]), to_tf32(re[4 * half + 3]));
                        *reinterpret_cast<float4*>(B + oim) =
                            make_float4(to_tf32(im[4 * half]), to_tf32(im[4 * half + 1]),
                                        to_tf32(im[4 * half + 2]), to_tf32(im[4 * half + 3]));
                    }
                } else {
                    uint32_t hre[4], lre[4], him[4], lim[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const __nv_bfloat16 h0 = __float2bfloat16_rn(re[2 * q]);
                        const __nv_bfloat16 h1 = __float2bfloat16_rn(re[2 * q + 1]);
                        const __nv_bfloat16 l0 = __float2bfloat16_rn(re[2 * q] - __bfloat162float(h0));
                        const __nv_bfloat16 l1 =
                            __float2bfloat16_rn(re[2 * q + 1] - __bfloat162float(h1));
                        hre[q] = pack_bf16(h0, h1);
                        lre[q] = pack_bf16(l0, l1);
                        const __nv_bfloat16 g0 = __float2bfloat16_rn(im[2 * q]);
                        const __nv_bfloat16 g1 = __float2bfloat16_rn(im[2 * q + 1]);
                        const __nv_bfloat16 k0 = __float2bfloat16_rn(im[2 * q] - __bfloat162float(g0));
                        const __nv_bfloat16 k1 =
                            __float2bfloat16_rn(im[2 * q + 1] - __bfloat162float(g1));
                        him[q] = pack_bf16(g0, g1);
                        lim[q] = pack_bf16(k0, k1);
                    }
                    const uint32_t ore = kmajor_off(n, rb * 8, 128, 2);
                    const uint32_t oim = kmajor_off(n, 64 + rb * 8, 128, 2);
                    *reinterpret_cast<uint4*>(B + ore) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                    *reinterpret_cast<uint4*>(B + oim) = make_uint4(him[0], him[1], him[2], him[3]);
                    *reinterpret_cast<uint4*>(B + b_lo + ore) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
                    *reinterpret_cast<uint4*>(B + b_lo + oim) = make_uint4(lim[0], lim[1], lim[2], lim[3]);
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();

        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t d = tmem + uint32_t(j & 1) * TC_NSUB;
            const uint32_t bsm = sb + SM_B + uint32_t(j & 1) * 32768u;
            if (PREC == HQ_MM_TF32) {
                for (int kk = 0; kk < nsteps; kk++)
                    mma_tf32(d, make_desc(sb + SM_A + kk * kstep_bytes, 128, sbo),
                             make_desc(bsm + kk * kstep_bytes, 128, sbo), idesc, kk > 0);
            } else {
                for (int kk = 0; kk < nsteps; kk++)  // hi . hi
                    mma_f16(d, make_desc(sb + SM_A + kk * kstep_bytes, 128, sbo),
                            make_desc(bsm + kk * kstep_bytes, 128, sbo), idesc, kk > 0);
                for (int kk = 0; kk < nsteps; kk++)  // hi . lo
                    mma_f16(d, make_desc(sb + SM_A + kk * kstep_bytes, 128, sbo),
                            make_desc(bsm + b_lo + kk * kstep_bytes, 128, sbo), idesc, 1);
                for (int kk = 0; kk < nsteps; kk++)  // lo . hi
                    mma_f16(d, make_desc(sb + SM_A + 32768 + kk * kstep_bytes, 128, sbo),
                            make_desc(bsm + kk * kstep_bytes, 128, sbo), idesc, 1);
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    s_mbar + 8 * uint32_t(j & 1))
                : "memory");
        }
        if (j > 0) epilogue(j - 1);
        if (failed) break;
        load(j + 2);  // into R[(j+2)%3], the buffer sub-tile j-1 just left
    }
    if (!failed && J > 0) epilogue(J - 1);
    cp_async_wait_all();
    if (a_failed) mbar_wait(s_mbar + 24, 0);  // the operand copies still in flight, bounded
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
}

// A operand from the FP64 unitary U (64 x 64, column-major): the real form
// [[Ur, -Ui], [Ui, Ur]] (128 x 128) in the K-major core layout.
__global__ void k_u_to_tc(const double2* __restrict__ U, unsigned char* __restrict__ out, int prec) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 128 * 128) return;
    const int i = idx / 128, k = idx % 128;
    const int r = i & 63, c = k & 63;
    const double2 u = U[(size_t)c * 64 + r];
    double v;
    if (i < 64)
        v = k < 64 ? u.x : -u.y;
    else
        v = k < 64 ? u.y : u.x;
    if (prec == HQ_MM_TF32) {
        *reinterpret_cast<float*>(out + kmajor_off(i, k, 128, 4)) = to_tf32((float)v);
    } else {
        const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
        const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
        *reinterpret_cast<__nv_bfloat16*>(out + kmajor_off(i, k, 128, 2)) = hi;
        *reinterpret_cast<__nv_bfloat16*>(out + 32768 + kmajor_off(i, k, 128, 2)) = lo;
    }
}

// ---- 7- and 8-qubit groups: U streamed, whole tiles -------------------------
// U (2^KQ x 2^KQ complex) as split BF16 or TF32 is 128 KB (KQ = 7) or 512 KB
// (KQ = 8).  It streams from L2 (every CTA reads the same bytes) through a
// ring of three 32 KB chunks, each the Ur or Ui block of one 128-row half m of
// the output over a 64-wide K slice s, chunk (m * KS + s) * 2 + part.  One
// pass of the ring covers a whole 2^13-amplitude tile: ROWS = 2^KQ rows (the
// group's qubits) x NCOL = 2^(13-KQ) columns, so every MMA has N = NCOL
// (64 or 32; the tensor pipe's cost per MMA barely depends on N).  Per half m
// the complex product runs as four real GEMMs (M = 128, N = NCOL, K = ROWS in
// 64-wide slices) into three accumulators, the real part's two terms kept
// apart and subtracted in the epilogue:
//     P(m) = Ur(m,:).Br,  Q(m) = Ui(m,:).Bi,  Ci(m) = Ui(m,:).Br + Ur(m,:).Bi,
//     Cr(m) = P(m) - Q(m)
// Warp-specialised: warps 0-7 stage tiles (cp.async), build B = Br | Bi and
// run the epilogue; warp 8 (one thread) streams the A chunks with bulk copies
// and issues the MMAs.  Handshakes: bfull (B of tile j written, 256
// arrivals), acc[j&1] (MMAs of tile j complete, tcgen05.commit), afull /
// aempty per ring slot (bulk-copy bytes landed / the MMAs reading the slot
// complete).  Tile j + 1 is staged while the MMAs of tile j run; its B is
// built once they complete (one B buffer), while the accumulators are double
// buffered so the epilogue of tile j - 1 overlaps the MMAs of tile j.
template <int KQ>
struct TcsShape {
    static constexpr int ROWS = 1 << KQ;
    static constexpr int NCOL = (1 << 13) / ROWS;
    static constexpr int MB = ROWS / 128;        // 128-row output halves
    static constexpr int KS = ROWS / 64;         // 64-wide K slices
    static constexpr int CHUNKS = MB * KS * 2;   // A chunks per tile
    static constexpr int RPT = ROWS * NCOL / 256;  // B rows a worker converts
    static_assert(MB * 3 * NCOL <= 256, "accumulators of one buffer");
};
constexpr int TS_WORKERS = 256;
constexpr int TS_THREADS = TS_WORKERS + 32;
constexpr uint32_t SMS_R = 0;                         // the tile, float2[8192]
constexpr uint32_t SMS_B = 65536;                     // Br | Bi
constexpr uint32_t BS_COMP = 32768;
constexpr uint32_t SMS_A = SMS_B + 2 * BS_COMP;       // ring of A chunks
constexpr uint32_t AS_CHUNK = 32768;
constexpr int AS_SLOTS = 3;
constexpr uint32_t SMS_MISC = SMS_A + AS_SLOTS * AS_CHUNK;
constexpr uint32_t SMS_TOTAL = SMS_MISC + 2048;
static_assert(SMS_TOTAL <= 232448, "shared memory per block");
// MISC: mbarriers and the TMEM slot, piece tables at + 128, slot tables at + 512
constexpr uint32_t MBS_ACC = 8, MBS_AFULL = 24, MBS_AEMPTY = MBS_AFULL + 8 * AS_SLOTS,
                   MBS_FIN = MBS_AEMPTY + 8 * AS_SLOTS, MBS_TSLOT = MBS_FIN + 8;
static_assert(MBS_TSLOT + 4 <= 128, "MISC head");
constexpr uint32_t TMEMS_COLS = 512;  // accumulator buffer b at column 256 b

// bar.sync / bar.red over the 256 worker threads only (barrier 1)
__device__ __forceinline__ void workers_sync() { asm volatile("bar.sync 1, 256;\n" ::: "memory"); }
__device__ __forceinline__ bool workers_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, 1, 256, q;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void set_err(int* err, int site, uint64_t detail) {
    if (err) {
        atomicCAS(err, 0, 1);
        err[1] = site;
        err[2] = (int)(detail & 0x7fffffff);
    }
}

template <int KQ, int PREC>
__global__ void __launch_bounds__(TS_THREADS, 1) k_transmm_tcs(const TransmmLaunch p) {
    using S = TcsShape<KQ>;
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* poff = reinterpret_cast<uint64_t*>(smem + SMS_MISC + 128);     // 16 pieces
    uint32_t* pslot = reinterpret_cast<uint32_t*>(smem + SMS_MISC + 256);    // 16 pieces
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(smem + SMS_MISC + 512);  // up to 256
    uint32_t* colslot = rowslot + S::ROWS;                                   // up to 64
    const uint32_t sb = smem_u32(smem);
    const uint32_t m_bfull = sb + SMS_MISC, m_acc = m_bfull + MBS_ACC, m_afull = m_bfull + MBS_AFULL,
                   m_aempty = m_bfull + MBS_AEMPTY, m_fin = m_bfull + MBS_FIN, s_tslot = m_bfull + MBS_TSLOT;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_tslot),
                     "r"(TMEMS_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(m_bfull), "r"(TS_WORKERS));
        for (int i = 0; i < 2; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_acc + 8 * i));
        for (int i = 0; i < AS_SLOTS; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_afull + 8 * i));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_aempty + 8 * i));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_fin));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (t < 16) {  // piece mm of a thread = tile local index 2 t + 512 mm
        poff[t] = local_to_phys(uint32_t(t) << 9, TC_TILE_BITS, p.tile_phys);
        pslot[t] = tile_swz(uint32_t(t) << 9);
    }
    for (int r = t; r < S::ROWS; r += TS_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < KQ; b++)
            if ((r >> b) & 1) x |= 1u << p.row_local[b];
        rowslot[r] = tile_swz(x);
    }
    for (int c = t; c < S::NCOL; c += TS_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < TC_TILE_BITS - KQ; b++)
            if ((c >> b) & 1) x |= 1u << p.col_local[b];
        colslot[c] = tile_swz(x);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + SMS_MISC + MBS_TSLOT);

    constexpr uint32_t esize = PREC == HQ_MM_TF32 ? 4 : 2;
    constexpr uint32_t per_core = 16 / esize;
    const uint64_t G = gridDim.x;
    const uint64_t J = blockIdx.x < p.ntiles ? (p.ntiles - blockIdx.x + G - 1) / G : 0;

    if (warp == TS_WORKERS / 32) {
        // ---- A stream + MMA issue (one thread) ----
        if (lane == 0 && J > 0) {
            constexpr uint32_t sbo_a = (64 / per_core) * 128;        // A chunk: 128 rows x 64 K
            constexpr uint32_t sbo_b = (S::ROWS / per_core) * 128;   // B: NCOL rows x ROWS K
            constexpr uint32_t slice_b = (64 / per_core) * 128;      // B offset of one K slice
            constexpr uint32_t a_lo = 16384;                         // A chunk lo half (BF16x3)
            constexpr uint32_t b_lo = S::NCOL * S::ROWS * 2;         // B component lo half (BF16x3)
            constexpr uint32_t idesc = make_idesc(PREC == HQ_MM_TF32 ? 2u : 1u, 128, S::NCOL);
            constexpr int nsteps = PREC == HQ_MM_TF32 ? 8 : 4;       // 32 bytes of K per MMA
            const char* umat = reinterpret_cast<const char*>(p.umat);
            auto gemm = [&](uint32_t d, uint32_t a, uint32_t bm, bool first) {
                if (PREC == HQ_MM_TF32) {
                    for (int kk = 0; kk < nsteps; kk++)
                        mma_tf32(d, make_desc(a + kk * 256, 128, sbo_a), make_desc(bm + kk * 256, 128, sbo_b),
                                 idesc, !first || kk > 0);
                } else {
                    for (int kk = 0; kk < nsteps; kk++)  // hi . hi
                        mma_f16(d, make_desc(a + kk * 256, 128, sbo_a), make_desc(bm + kk * 256, 128, sbo_b),
                                idesc, !first || kk > 0);
                    for (int kk = 0; kk < nsteps; kk++)  // hi . lo
                        mma_f16(d, make_desc(a + kk * 256, 128, sbo_a),
                                make_desc(bm + b_lo + kk * 256, 128, sbo_b), idesc, 1);
                    for (int kk = 0; kk < nsteps; kk++)  // lo . hi
                        mma_f16(d, make_desc(a + a_lo + kk * 256, 128, sbo_a),
                                make_desc(bm + kk * 256, 128, sbo_b), idesc, 1);
                }
            };
            const uint64_t total = J * S::CHUNKS;
            uint64_t issued = 0, consumed = 0;
            auto fetch = [&](uint64_t h) {
                const uint32_t slot = uint32_t(h % AS_SLOTS);
                bulk_load(sb + SMS_A + slot * AS_CHUNK, umat + (h % S::CHUNKS) * AS_CHUNK, AS_CHUNK,
                          m_afull + 8 * slot);
                issued = h + 1;
            };
            for (uint64_t h = 0; h + 1 < AS_SLOTS && h < total; h++) fetch(h);
            bool ok = true;
            for (uint64_t j = 0; j < J && ok; j++) {
                if (!mbar_wait(m_bfull, uint32_t(j & 1))) {
                    set_err(p.err, 10, j);  // site: TransMM operand B handshake
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t accb = tmem + 256 * uint32_t(j & 1);
                for (int c = 0; c < S::CHUNKS; c++) {
                    const uint64_t g = j * S::CHUNKS + c;
                    const uint32_t slot = uint32_t(g % AS_SLOTS);
                    if (!mbar_wait(m_afull + 8 * slot, uint32_t((g / AS_SLOTS) & 1))) {
                        set_err(p.err, 9, g);  // site: TransMM operand load
                        ok = false;
                        break;
                    }
                    consumed = g + 1;
                    const int m = c / (2 * S::KS), s = (c >> 1) % S::KS, part = c & 1;
                    const uint32_t a = sb + SMS_A + slot * AS_CHUNK;
                    const uint32_t dp = accb + 3 * S::NCOL * m, dq = dp + S::NCOL, di = dp + 2 * S::NCOL;
                    const uint32_t br = sb + SMS_B + s * slice_b, bi = br + BS_COMP;
                    if (part == 0) {
                        gemm(dp, a, br, s == 0);
                        gemm(di, a, bi, s == 0);
                    } else {
                        gemm(dq, a, bi, s == 0);
                        gemm(di, a, br, false);
                    }
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                            m_aempty + 8 * slot)
                        : "memory");
                    // refill: chunk g + SLOTS - 1 goes where chunk g - 1 was, once its MMAs completed
                    const uint64_t h = g + AS_SLOTS - 1;
                    if (h < total) {
                        if (h >= AS_SLOTS && !mbar_wait(m_aempty + 8 * uint32_t(h % AS_SLOTS),
                                                        uint32_t(((h - AS_SLOTS) / AS_SLOTS) & 1))) {
                            set_err(p.err, 9, h);
                            ok = false;
                            break;
                        }
                        fetch(h);
                    }
                }
                if (!ok) break;
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                        m_acc + 8 * uint32_t(j & 1))
                    : "memory");
            }
            // drain: every issued MMA complete, every issued copy landed (bounded)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             m_fin)
                         : "memory");
            mbar_wait(m_fin, 0);
            for (uint64_t h = consumed; h < issued; h++)
                mbar_wait(m_afull + 8 * uint32_t(h % AS_SLOTS), uint32_t((h / AS_SLOTS) & 1));
        }
        __syncwarp();
    } else {
        // ---- workers: staging, B, epilogue ----
        const uint64_t toff = local_to_phys(uint32_t(t) << 1, TC_TILE_BITS, p.tile_phys);
        const uint32_t tsl = tile_swz(uint32_t(t) << 1);
        auto tbase = [&](uint64_t j) {
            return tile_base(blockIdx.x + j * G, p.nruns, p.run_src, p.run_dst, p.run_len);
        };
        auto load = [&](uint64_t j) {
            if (j < J) {
                const float2* gsrc = state + tbase(j) + toff;
#pragma unroll
                for (int mm = 0; mm < 16; mm++)
                    cp_async16(sb + SMS_R + (tsl ^ pslot[mm]) * 8u, gsrc + poff[mm]);
            }
            cp_async_commit();
        };
        float2* R = reinterpret_cast<float2*>(smem + SMS_R);
        // results of tile j: TMEM buffer j&1 -> R -> HBM.  Warp (q, h): TMEM
        // lanes 32 q .. 32 q + 31 of half m = h (KQ = 8) or of columns 32 h .. (KQ = 7)
        auto epilogue = [&](uint64_t j) {
            const uint32_t b = uint32_t(j & 1);
            const int q = warp & 3, h = warp >> 2;
            const int m = S::MB == 2 ? h : 0, c0 = S::MB == 2 ? 0 : 32 * h;
            const int i = 128 * m + 32 * q + lane;  // row of the group
            const uint32_t col = tmem + ((uint32_t)(32 * q) << 16) + 256 * b + 3 * S::NCOL * m + c0;
            const uint32_t rs = rowslot[i];
#pragma unroll
            for (int c8 = 0; c8 < 4; c8++) {
                uint32_t vp[8], vq[8], vi[8];
                tmem_ld8(col + 8 * c8, vp);
                tmem_ld8(col + S::NCOL + 8 * c8, vq);
                tmem_ld8(col + 2 * S::NCOL + 8 * c8, vi);
#pragma unroll
                for (int c = 0; c < 8; c++)
                    R[rs ^ colslot[c0 + 8 * c8 + c]] =
                        make_float2(__uint_as_float(vp[c]) - __uint_as_float(vq[c]), __uint_as_float(vi[c]));
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            workers_sync();
            float2* gdst = state + tbase(j) + toff;
            const float4* R4 = reinterpret_cast<const float4*>(R);
#pragma unroll
            for (int mm = 0; mm < 16; mm++)
                *reinterpret_cast<float4*>(gdst + poff[mm]) = R4[(tsl ^ pslot[mm]) >> 1];
            workers_sync();
        };
        bool failed = false;
        load(0);
        for (uint64_t j = 0; j < J; j++) {
            cp_async_wait_all();  // tile j staged
            workers_sync();
            if (j > 0) {  // MMAs of tile j - 1 complete: B is free, accumulators j - 1 ready
                const bool ok = mbar_wait(m_acc + 8 * uint32_t((j - 1) & 1), uint32_t(((j - 1) >> 1) & 1));
                if (workers_any(!ok)) {
                    if (t == 0) set_err(p.err, 7, j - 1);  // site: TransMM accumulator wait
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            }
            {
                unsigned char* B = smem + SMS_B;
                const int n = t % S::NCOL, rb = t / S::NCOL;  // column n, rows RPT rb .. RPT rb + RPT - 1
                const uint32_t cs = colslot[n];
                if (PREC == HQ_MM_TF32) {
#pragma unroll
                    for (int h4 = 0; h4 < S::RPT / 4; h4++) {
                        float re[4], im[4];
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            const float2 a = R[rowslot[rb * S::RPT + 4 * h4 + qq] ^ cs];
                            re[qq] = to_tf32(a.x);
                            im[qq] = to_tf32(a.y);
                        }
                        const uint32_t o = kmajor_off(n, rb * S::RPT + 4 * h4, S::ROWS, 4);
                        *reinterpret_cast<float4*>(B + o) = make_float4(re[0], re[1], re[2], re[3]);
                        *reinterpret_cast<float4*>(B + BS_COMP + o) = make_float4(im[0], im[1], im[2], im[3]);
                    }
                } else {
                    constexpr uint32_t b_lo = S::NCOL * S::ROWS * 2;
#pragma unroll
                    for (int h8 = 0; h8 < S::RPT / 8; h8++) {
                        uint32_t hre[4], lre[4], him[4], lim[4];
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            const float2 a0 = R[rowslot[rb * S::RPT + 8 * h8 + 2 * qq] ^ cs];
                            const float2 a1 = R[rowslot[rb * S::RPT + 8 * h8 + 2 * qq + 1] ^ cs];
                            const __nv_bfloat16 h0 = __float2bfloat16_rn(a0.x), h1 = __float2bfloat16_rn(a1.x);
                            const __nv_bfloat16 g0 = __float2bfloat16_rn(a0.y), g1 = __float2bfloat16_rn(a1.y);
                            hre[qq] = pack_bf16(h0, h1);
                            lre[qq] = pack_bf16(__float2bfloat16_rn(a0.x - __bfloat162float(h0)),
                                                __float2bfloat16_rn(a1.x - __bfloat162float(h1)));
                            him[qq] = pack_bf16(g0, g1);
                            lim[qq] = pack_bf16(__float2bfloat16_rn(a0.y - __bfloat162float(g0)),
                                                __float2bfloat16_rn(a1.y - __bfloat162float(g1)));
                        }
                        const uint32_t o = kmajor_off(n, rb * S::RPT + 8 * h8, S::ROWS, 2);
                        *reinterpret_cast<uint4*>(B + o) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                        *reinterpret_cast<uint4*>(B + b_lo + o) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
                        *reinterpret_cast<uint4*>(B + BS_COMP + o) = make_uint4(him[0], him[1], him[2], him[3]);
                        *reinterpret_cast<uint4*>(B + BS_COMP + b_lo + o) =
                            make_uint4(lim[0], lim[1], lim[2], lim[3]);
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(m_bfull) : "memory");
            workers_sync();  // R is read: the epilogue may write over it
            if (j > 0) epilogue(j - 1);
            load(j + 1);
        }
        if (!failed && J > 0) {
            const bool ok = mbar_wait(m_acc + 8 * uint32_t((J - 1) & 1), uint32_t(((J - 1) >> 1) & 1));
            if (workers_any(!ok)) {
                if (t == 0) set_err(p.err, 7, J - 1);
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                epilogue(J - 1);
            }
        }
        cp_async_wait_all();
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEMS_COLS));
}

// A operand of a 7- or 8-qubit group from U (2^KQ x 2^KQ, column-major
// complex128): the chunks in the order the kernel consumes them, chunk
// (m * KS + s) * 2 + part = Ur (part 0) or Ui (part 1) of output rows
// 128 m .. 128 m + 127 and K 64 s .. 64 s + 63, K-major (split BF16 hi at +0
// and lo at +16 KB, or TF32).
template <int KQ>
__global__ void k_u_to_tcs(const double2* __restrict__ U, unsigned char* __restrict__ out, int prec) {
    using S = TcsShape<KQ>;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= S::ROWS * S::ROWS) return;
    const int r = idx / S::ROWS, k = idx % S::ROWS;
    const double2 u = U[(size_t)k * S::ROWS + r];
    const double v[2] = {u.x, u.y};
    const int m = r >> 7, rr = r & 127, s = k >> 6, kk = k & 63;
    for (int part = 0; part < 2; part++) {
        unsigned char* base = out + size_t((m * S::KS + s) * 2 + part) * AS_CHUNK;
        if (prec == HQ_MM_TF32) {
            *reinterpret_cast<float*>(base + kmajor_off(rr, kk, 64, 4)) = to_tf32((float)v[part]);
        } else {
            const __nv_bfloat16 hi = __float2bfloat16_rn((float)v[part]);
            const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v[part] - (double)__bfloat162float(hi)));
            *reinterpret_cast<__nv_bfloat16*>(base + kmajor_off(rr, kk, 64, 2)) = hi;
            *reinterpret_cast<__nv_bfloat16*>(base + 16384 + kmajor_off(rr, kk, 64, 2)) = lo;
        }
    }
}

}  // namespace

size_t transmm_tc_operand_bytes(int m, int precision) {
    (void)precision;
    HQ_REQUIRE(m >= 6 && m <= 8, HQ_ERR_UNSUPPORTED,
               "tensor-core TransMM runs 6- to 8-qubit groups (got %d)", m);
    return m == 6 ? 65536 : m == 7 ? size_t(TcsShape<7>::CHUNKS) * AS_CHUNK : size_t(TcsShape<8>::CHUNKS) * AS_CHUNK;
}

void launch_u_to_tc_operand(int m, int precision, const double* d_u, void* d_out, cudaStream_t st) {
    HQ_REQUIRE(m >= 6 && m <= 8, HQ_ERR_UNSUPPORTED,
               "tensor-core TransMM runs 6- to 8-qubit groups (got %d)", m);
    if (m == 6)
        k_u_to_tc<<<64, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
    else if (m == 7)
        k_u_to_tcs<7><<<64, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
    else
        k_u_to_tcs<8><<<256, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
    HQ_CHECK_CUDA(cudaGetLastError());
}

template <int PREC>
static void launch_prec(const TransmmLaunch& p, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_tc<PREC>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM_TOTAL));
        attr = true;
    }
    const uint64_t slots = uint64_t(ctx().sm_count);
    const unsigned grid = (unsigned)(p.ntiles < slots ? p.ntiles : slots);
    k_transmm_tc<PREC><<<grid, TC_THREADS, SM_TOTAL, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

template <int KQ, int PREC>
static void launch_streamed(const TransmmLaunch& p, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_tcs<KQ, PREC>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMS_TOTAL));
        attr = true;
    }
    const uint64_t slots = uint64_t(ctx().sm_count);
    const unsigned grid = (unsigned)(p.ntiles < slots ? p.ntiles : slots);
    k_transmm_tcs<KQ, PREC><<<grid, TS_THREADS, SMS_TOTAL, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_transmm_tc(const TransmmLaunch& p, cudaStream_t st) {
    HQ_REQUIRE(p.m >= 6 && p.m <= 8 && p.k == TC_TILE_BITS, HQ_ERR_UNSUPPORTED,
               "tensor-core TransMM runs 6- to 8-qubit groups on 13-qubit tiles");
    const bool tf32 = p.precision == HQ_MM_TF32;
    if (p.m == 8) {
        if (tf32)
            launch_streamed<8, HQ_MM_TF32>(p, st);
        else
            launch_streamed<8, HQ_MM_BF16X3>(p, st);
    } else if (p.m == 7) {
        if (tf32)
            launch_streamed<7, HQ_MM_TF32>(p, st);
        else
            launch_streamed<7, HQ_MM_BF16X3>(p, st);
    } else if (tf32) {
        launch_prec<HQ_MM_TF32>(p, st);
    } else {
        launch_prec<HQ_MM_BF16X3>(p, st);
    }
}

}  // namespace hq
