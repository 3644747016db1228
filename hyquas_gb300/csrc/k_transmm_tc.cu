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

// ---- 7-qubit groups ---------------------------------------------------------
// U (128 x 128 complex) no longer fits shared memory in real form, so the
// product is taken in complex form over four real GEMMs into two accumulators:
//     Cr = Ur.Br + Ui.(-Bi),   Ci = Ui.Br + Ur.Bi      (M = 128, N = 16, K = 128)
// A holds Ur and Ui (split BF16 hi + lo, or TF32; 128 KB); each sub-tile of
// 128 rows x 16 columns stages Br, Bi and -Bi.  The pipeline is the one of the
// 6-qubit kernel (three staging buffers, two B buffers, two accumulator pairs).
constexpr int T7_ROWS = 128;
constexpr int T7_NSUB = 16;
constexpr uint32_t SUB7_BYTES = 16384;   // a sub-tile, float2[2048]
constexpr uint32_t SM7_A = 0;            // Ur, Ui: 128 KB
constexpr uint32_t SM7_UI = 65536;
constexpr uint32_t SM7_B = 131072;       // two buffers of 24 KB: Br | Bi | -Bi
constexpr uint32_t B7_BYTES = 24576;
constexpr uint32_t SM7_R = 180224;       // three staging buffers of 16 KB
constexpr uint32_t SM7_MISC = 229376;
constexpr uint32_t SM7_TOTAL = SM7_MISC + 1024;
constexpr uint32_t TMEM7_COLS = 64;      // two buffers x (Cr 16 + Ci 16 columns)
static_assert(SM7_TOTAL <= 232448, "shared memory per block");

template <int PREC>
__global__ void __launch_bounds__(TC_THREADS, 1) k_transmm_tc7(const TransmmLaunch p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(smem + SM7_MISC + 64);
    uint32_t* colslot = rowslot + T7_ROWS;
    const uint32_t sb = smem_u32(smem);
    const uint32_t s_mbar = sb + SM7_MISC;
    const uint32_t s_tslot = sb + SM7_MISC + 16;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_tslot),
                     "r"(TMEM7_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar + 8));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_mbar + 24));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (t == 0) bulk_load(sb + SM7_A, p.umat, 131072u, s_mbar + 24);  // Ur, Ui: 128 KB
    for (int r = t; r < T7_ROWS; r += TC_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 7; b++)
            if ((r >> b) & 1) x |= 1u << p.row_sub[b];
        rowslot[r] = tile_swz(x);
    }
    for (int c = t; c < T7_NSUB; c += TC_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 4; b++)
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
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + SM7_MISC + 16);

    const uint64_t toff = local_to_phys(uint32_t(t) << 1, TC_TILE_BITS - 2, p.sub_phys);
    const uint32_t tsl = tile_swz(uint32_t(t) << 1);
    constexpr uint32_t esize = PREC == HQ_MM_TF32 ? 4 : 2;
    constexpr uint32_t kstep_bytes = 256;
    constexpr uint32_t sbo = (128 / (16 / esize)) * 128;
    constexpr uint32_t a_lo = 32768;          // Ur / Ui lo halves (BF16x3)
    constexpr uint32_t b_lo = 4096;           // Br / Bi / -Bi lo halves (BF16x3)
    constexpr uint32_t idesc = make_idesc(PREC == HQ_MM_TF32 ? 2u : 1u, 128, T7_NSUB);
    constexpr int nsteps = PREC == HQ_MM_TF32 ? 16 : 8;

    const uint64_t nsub = p.ntiles * 4;
    const uint64_t G = gridDim.x;
    const uint64_t J = blockIdx.x < nsub ? (nsub - blockIdx.x + G - 1) / G : 0;
    auto sub_base = [&](uint64_t j) {
        const uint64_t v = blockIdx.x + j * G;
        return tile_base(v >> 2, p.nruns, p.run_src, p.run_dst, p.run_len) +
               (v & 1) * p.split_off[0] + ((v >> 1) & 1) * p.split_off[1];
    };
    auto load = [&](uint64_t j) {
        if (j < J) {
            const float2* gsrc = state + sub_base(j) + toff;
            const uint32_t rb = sb + SM7_R + uint32_t(j % 3) * SUB7_BYTES;
#pragma unroll
            for (int m = 0; m < 4; m++)
                cp_async16(rb + (tsl ^ p.sub_piece_slot[m]) * 8u, gsrc + p.sub_piece_off[m]);
        }
        cp_async_commit();
    };
    bool failed = a_failed;
    // results of sub-tile j: (Cr, Ci) in TMEM columns 32 (j&1) and + 16 -> staging -> HBM
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
        float2* Rj = reinterpret_cast<float2*>(smem + SM7_R + uint32_t(j % 3) * SUB7_BYTES);
        {
            const int q = warp & 3, half = warp >> 2;
            const int i = 32 * q + lane;  // D row = TMEM lane = row of the group
            const uint32_t col = tmem + ((uint32_t)(32 * q) << 16) + 32 * b + 8 * half;
            uint32_t vr[8], vi[8];
            tmem_ld8(col, vr);
            tmem_ld8(col + 16, vi);
            const uint32_t rs = rowslot[i];
#pragma unroll
            for (int c = 0; c < 8; c++)
                Rj[rs ^ colslot[8 * half + c]] = make_float2(__uint_as_float(vr[c]), __uint_as_float(vi[c]));
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        float2* gdst = state + sub_base(j) + toff;
        const float4* R4 = reinterpret_cast<const float4*>(Rj);
#pragma unroll
        for (int m = 0; m < 4; m++)
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
        // B blocks of sub-tile j: row n of each = column n; K = the group's row
        {
            const float2* Rj = reinterpret_cast<const float2*>(smem + SM7_R + uint32_t(j % 3) * SUB7_BYTES);
            unsigned char* B = smem + SM7_B + uint32_t(j & 1) * B7_BYTES;
            const int n = t & 15, rb = t >> 4;
            const uint32_t cs = colslot[n];
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
                    const uint32_t o = kmajor_off(n, rb * 8 + half * 4, 128, 4);
                    const float4 vr = make_float4(to_tf32(re[4 * half]), to_tf32(re[4 * half + 1]),
                                                  to_tf32(re[4 * half + 2]), to_tf32(re[4 * half + 3]));
                    const float4 vi = make_float4(to_tf32(im[4 * half]), to_tf32(im[4 * half + 1]),
                                                  to_tf32(im[4 * half + 2]), to_tf32(im[4 * half + 3]));
                    *reinterpret_cast<float4*>(B + o) = vr;
                    *reinterpret_cast<float4*>(B + 8192 + o) = vi;
                    *reinterpret_cast<float4*>(B + 16384 + o) = make_float4(-vi.x, -vi.y, -vi.z, -vi.w);
                }
            } else {
                uint32_t hre[4], lre[4], him[4], lim[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const __nv_bfloat16 h0 = __float2bfloat16_rn(re[2 * q]);
                    const __nv_bfloat16 h1 = __float2bfloat16_rn(re[2 * q + 1]);
                    const __nv_bfloat16 l0 = __float2bfloat16_rn(re[2 * q] - __bfloat162float(h0));
                    const __nv_bfloat16 l1 = __float2bfloat16_rn(re[2 * q + 1] - __bfloat162float(h1));
                    hre[q] = pack_bf16(h0, h1);
                    lre[q] = pack_bf16(l0, l1);
                    const __nv_bfloat16 g0 = __float2bfloat16_rn(im[2 * q]);
                    const __nv_bfloat16 g1 = __float2bfloat16_rn(im[2 * q + 1]);
                    const __nv_bfloat16 k0 = __float2bfloat16_rn(im[2 * q] - __bfloat162float(g0));
                    const __nv_bfloat16 k1 = __float2bfloat16_rn(im[2 * q + 1] - __bfloat162float(g1));
                    him[q] = pack_bf16(g0, g1);
                    lim[q] = pack_bf16(k0, k1);
                }
                const uint32_t o = kmajor_off(n, rb * 8, 128, 2);
                const uint32_t sg = 0x80008000u;  // BF16 sign bits: -Bi exactly
                *reinterpret_cast<uint4*>(B + o) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                *reinterpret_cast<uint4*>(B + b_lo + o) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
                *reinterpret_cast<uint4*>(B + 8192 + o) = make_uint4(him[0], him[1], him[2], him[3]);
                *reinterpret_cast<uint4*>(B + 8192 + b_lo + o) = make_uint4(lim[0], lim[1], lim[2], lim[3]);
                *reinterpret_cast<uint4*>(B + 16384 + o) =
                    make_uint4(him[0] ^ sg, him[1] ^ sg, him[2] ^ sg, him[3] ^ sg);
                *reinterpret_cast<uint4*>(B + 16384 + b_lo + o) =
                    make_uint4(lim[0] ^ sg, lim[1] ^ sg, lim[2] ^ sg, lim[3] ^ sg);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();

        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t dr = tmem + 32 * uint32_t(j & 1), di = dr + 16;
            const uint32_t bb = sb + SM7_B + uint32_t(j & 1) * B7_BYTES;
            const uint32_t ur = sb + SM7_A, ui = sb + SM7_UI;
            const uint32_t br = bb, bi = bb + 8192, bn = bb + 16384;
            // D += A . B over K = 128; first = the accumulator starts at zero
            auto gemm = [&](uint32_t d, uint32_t a, uint32_t bm, bool first) {
                if (PREC == HQ_MM_TF32) {
                    for (int kk = 0; kk < nsteps; kk++)
                        mma_tf32(d, make_desc(a + kk * kstep_bytes, 128, sbo),
                                 make_desc(bm + kk * kstep_bytes, 128, sbo), idesc, !first || kk > 0);
                } else {
                    for (int kk = 0; kk < nsteps; kk++)  // hi . hi
                        mma_f16(d, make_desc(a + kk * kstep_bytes, 128, sbo),
                                make_desc(bm + kk * kstep_bytes, 128, sbo), idesc, !first || kk > 0);
                    for (int kk = 0; kk < nsteps; kk++)  // hi . lo
                        mma_f16(d, make_desc(a + kk * kstep_bytes, 128, sbo),
                                make_desc(bm + b_lo + kk * kstep_bytes, 128, sbo), idesc, 1);
                    for (int kk = 0; kk < nsteps; kk++)  // lo . hi
                        mma_f16(d, make_desc(a + a_lo + kk * kstep_bytes, 128, sbo),
                                make_desc(bm + kk * kstep_bytes, 128, sbo), idesc, 1);
                }
            };
            gemm(dr, ur, br, true);
            gemm(dr, ui, bn, false);
            gemm(di, ui, br, true);
            gemm(di, ur, bi, false);
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    s_mbar + 8 * uint32_t(j & 1))
                : "memory");
        }
        if (j > 0) epilogue(j - 1);
        if (failed) break;
        load(j + 2);
    }
    if (!failed && J > 0) epilogue(J - 1);
    cp_async_wait_all();
    if (a_failed) mbar_wait(s_mbar + 24, 0);  // the operand copies still in flight, bounded
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM7_COLS));
}

// A operand of a 7-qubit group from U (128 x 128, column-major complex128):
// Ur and Ui, each 128 x 128 K-major (split BF16 hi at +0 and lo at +32 KB
// of its 64 KB half, or TF32).
__global__ void k_u_to_tc7(const double2* __restrict__ U, unsigned char* __restrict__ out, int prec) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 128 * 128) return;
    const int r = idx / 128, k = idx % 128;
    const double2 u = U[(size_t)k * 128 + r];
    const double v[2] = {u.x, u.y};
    for (int part = 0; part < 2; part++) {
        unsigned char* base = out + part * 65536;
        if (prec == HQ_MM_TF32) {
            *reinterpret_cast<float*>(base + kmajor_off(r, k, 128, 4)) = to_tf32((float)v[part]);
        } else {
            const __nv_bfloat16 hi = __float2bfloat16_rn((float)v[part]);
            const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v[part] - (double)__bfloat162float(hi)));
            *reinterpret_cast<__nv_bfloat16*>(base + kmajor_off(r, k, 128, 2)) = hi;
            *reinterpret_cast<__nv_bfloat16*>(base + 32768 + kmajor_off(r, k, 128, 2)) = lo;
        }
    }
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


// ---- 8-qubit groups ---------------------------------------------------------
// U (256 x 256 complex) as split BF16 or TF32 is 512 KB, more than shared
// memory: it streams from L2 (every CTA reads the same 512 KB) through a ring
// of three 32 KB chunks, each the Ur or Ui block of one 128-row half m of the
// output over a 64-wide K slice s.  A sub-tile is 256 rows x 16 columns
// (32 KB, the tile's top column bit fixed); per half m the complex product
// runs as four real GEMMs (M = 128, N = 16, K = 256 in four slices):
//     Cr(m) = Ur(m,:).Br + Ui(m,:).(-Bi),   Ci(m) = Ui(m,:).Br + Ur(m,:).Bi
// Warp-specialised: warps 0-7 stage sub-tiles (cp.async), build B = Br | Bi |
// -Bi and run the epilogue; warp 8 (one thread) streams the A chunks with bulk
// copies and issues the MMAs.  Handshakes: bfull (B of sub-tile j written,
// 256 arrivals), acc[j&1] (MMAs of j complete, tcgen05.commit), afull/aempty
// per ring slot (bulk-copy bytes landed / the MMAs reading the slot complete).
constexpr int T8_ROWS = 256;
constexpr int T8_NSUB = 16;
constexpr int T8_WORKERS = 256;
constexpr int T8_THREADS = T8_WORKERS + 32;
constexpr uint32_t SUB8_BYTES = 32768;  // a sub-tile, float2[4096]
constexpr uint32_t SM8_R = 0;           // two staging buffers of 32 KB
constexpr uint32_t SM8_B = 65536;       // Br | Bi | -Bi
constexpr uint32_t B8_COMP = 16384;
constexpr uint32_t SM8_A = SM8_B + 3 * B8_COMP;  // ring of A chunks
constexpr uint32_t A8_CHUNK = 32768;
constexpr int A8_SLOTS = 3;
constexpr int A8_CHUNKS = 16;  // per sub-tile, chunk c = (m * 4 + s) * 2 + (0: Ur, 1: Ui)
constexpr uint32_t SM8_MISC = SM8_A + A8_SLOTS * A8_CHUNK;
constexpr uint32_t SM8_TOTAL = SM8_MISC + 2048;
constexpr uint32_t TMEM8_COLS = 128;  // two buffers x (Cr0, Ci0, Cr1, Ci1) x 16 columns
static_assert(SM8_TOTAL <= 232448, "shared memory per block");

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

template <int PREC>
__global__ void __launch_bounds__(T8_THREADS, 1) k_transmm_tc8(const TransmmLaunch p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(smem + SM8_MISC + 256);
    uint32_t* colslot = rowslot + T8_ROWS;
    const uint32_t sb = smem_u32(smem);
    const uint32_t m_bfull = sb + SM8_MISC, m_acc = m_bfull + 8, m_afull = m_bfull + 24,
                   m_aempty = m_bfull + 48, m_fin = m_bfull + 72, s_tslot = m_bfull + 80;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_tslot),
                     "r"(TMEM8_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(m_bfull), "r"(T8_WORKERS));
        for (int i = 0; i < 2; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_acc + 8 * i));
        for (int i = 0; i < A8_SLOTS; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_afull + 8 * i));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_aempty + 8 * i));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(m_fin));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (int r = t; r < T8_ROWS; r += T8_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 8; b++)
            if ((r >> b) & 1) x |= 1u << p.row_sub[b];
        rowslot[r] = tile_swz(x);
    }
    for (int c = t; c < T8_NSUB; c += T8_THREADS) {
        uint32_t x = 0;
        for (int b = 0; b < 4; b++)
            if ((c >> b) & 1) x |= 1u << p.col_sub[b];
        colslot[c] = tile_swz(x);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + SM8_MISC + 80);

    constexpr uint32_t esize = PREC == HQ_MM_TF32 ? 4 : 2;
    const uint64_t nsub = p.ntiles * 2;
    const uint64_t G = gridDim.x;
    const uint64_t J = blockIdx.x < nsub ? (nsub - blockIdx.x + G - 1) / G : 0;

    if (warp == T8_WORKERS / 32) {
        // ---- A stream + MMA issue (one thread) ----
        if (lane == 0 && J > 0) {
            constexpr uint32_t sbo_a = (64 / (16 / esize)) * 128;   // A chunk: 128 rows x 64 K
            constexpr uint32_t sbo_b = (256 / (16 / esize)) * 128;  // B: 16 rows x 256 K
            constexpr uint32_t slice_b = (64 / (16 / esize)) * 128; // B offset of one K slice
            constexpr uint32_t a_lo = 16384;                        // A chunk lo half (BF16x3)
            constexpr uint32_t b_lo = 8192;                         // B component lo half
            constexpr uint32_t idesc = make_idesc(PREC == HQ_MM_TF32 ? 2u : 1u, 128, T8_NSUB);
            constexpr int nsteps = PREC == HQ_MM_TF32 ? 8 : 4;      // 32 bytes of K per MMA
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
            const uint64_t total = J * A8_CHUNKS;
            uint64_t issued = 0, consumed = 0;
            auto fetch = [&](uint64_t h) {
                const uint32_t slot = uint32_t(h % A8_SLOTS);
                bulk_load(sb + SM8_A + slot * A8_CHUNK, umat + (h % A8_CHUNKS) * A8_CHUNK, A8_CHUNK,
                          m_afull + 8 * slot);
                issued = h + 1;
            };
            fetch(0);
            if (total > 1) fetch(1);
            bool ok = true;
            for (uint64_t j = 0; j < J && ok; j++) {
                if (!mbar_wait(m_bfull, uint32_t(j & 1))) {
                    set_err(p.err, 10, j);  // site: TransMM operand B handshake
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t accb = tmem + 64 * uint32_t(j & 1);
                for (int c = 0; c < A8_CHUNKS; c++) {
                    const uint64_t g = j * A8_CHUNKS + c;
                    const uint32_t slot = uint32_t(g % A8_SLOTS);
                    if (!mbar_wait(m_afull + 8 * slot, uint32_t((g / A8_SLOTS) & 1))) {
                        set_err(p.err, 9, g);  // site: TransMM operand load
                        ok = false;
                        break;
                    }
                    consumed = g + 1;
                    const int m = c >> 3, s = (c >> 1) & 3, part = c & 1;
                    const uint32_t a = sb + SM8_A + slot * A8_CHUNK;
                    const uint32_t dr = accb + 32 * m, di = dr + 16;
                    const uint32_t br = sb + SM8_B + s * slice_b, bi = br + B8_COMP, bn = br + 2 * B8_COMP;
                    if (part == 0) {
                        gemm(dr, a, br, s == 0);
                        gemm(di, a, bi, s == 0);
                    } else {
                        gemm(dr, a, bn, false);
                        gemm(di, a, br, false);
                    }
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                            m_aempty + 8 * slot)
                        : "memory");
                    // refill: chunk g + 2 goes where chunk g - 1 was, once its MMAs completed
                    const uint64_t h = g + 2;
                    if (h < total) {
                        if (h >= A8_SLOTS &&
                            !mbar_wait(m_aempty + 8 * uint32_t(h % A8_SLOTS), uint32_t(((h - A8_SLOTS) / A8_SLOTS) & 1))) {
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
                mbar_wait(m_afull + 8 * uint32_t(h % A8_SLOTS), uint32_t((h / A8_SLOTS) & 1));
        }
        __syncwarp();
    } else {
        // ---- workers: staging, B, epilogue ----
        const uint64_t toff = local_to_phys(uint32_t(t) << 1, TC_TILE_BITS - 1, p.sub_phys);
        const uint32_t tsl = tile_swz(uint32_t(t) << 1);
        auto sub_base = [&](uint64_t j) {
            const uint64_t v = blockIdx.x + j * G;
            return tile_base(v >> 1, p.nruns, p.run_src, p.run_dst, p.run_len) + (v & 1) * p.split_off[0];
        };
        auto load = [&](uint64_t j) {
            if (j < J) {
                const float2* gsrc = state + sub_base(j) + toff;
                const uint32_t rb = sb + SM8_R + uint32_t(j & 1) * SUB8_BYTES;
#pragma unroll
                for (int m = 0; m < 8; m++)
                    cp_async16(rb + (tsl ^ p.sub_piece_slot[m]) * 8u, gsrc + p.sub_piece_off[m]);
            }
            cp_async_commit();
        };
        // results of sub-tile j: TMEM buffer j&1 -> over its staging buffer -> HBM
        auto epilogue = [&](uint64_t j) {
            const uint32_t b = uint32_t(j & 1);
            float2* Rj = reinterpret_cast<float2*>(smem + SM8_R + b * SUB8_BYTES);
            const int q = warp & 3, m = warp >> 2;
            const int i = 128 * m + 32 * q + lane;  // row of the group = TMEM lane 32 q + lane of half m
            const uint32_t col = tmem + ((uint32_t)(32 * q) << 16) + 64 * b + 32 * m;
            const uint32_t rs = rowslot[i];
#pragma unroll
            for (int half = 0; half < 2; half++) {
                uint32_t vr[8], vi[8];
                tmem_ld8(col + 8 * half, vr);
                tmem_ld8(col + 16 + 8 * half, vi);
#pragma unroll
                for (int c = 0; c < 8; c++)
                    Rj[rs ^ colslot[8 * half + c]] = make_float2(__uint_as_float(vr[c]), __uint_as_float(vi[c]));
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            workers_sync();
            float2* gdst = state + sub_base(j) + toff;
            const float4* R4 = reinterpret_cast<const float4*>(Rj);
#pragma unroll
            for (int mm = 0; mm < 8; mm++)
                *reinterpret_cast<float4*>(gdst + p.sub_piece_off[mm]) = R4[(tsl ^ p.sub_piece_slot[mm]) >> 1];
            workers_sync();
        };
        bool failed = false;
        load(0);
        for (uint64_t j = 0; j < J; j++) {
            cp_async_wait_all();  // sub-tile j staged
            workers_sync();
            if (j > 0) {  // MMAs of j - 1 complete: B is free, accumulators j - 1 ready
                const bool ok = mbar_wait(m_acc + 8 * uint32_t((j - 1) & 1), uint32_t(((j - 1) >> 1) & 1));
                if (workers_any(!ok)) {
                    if (t == 0) set_err(p.err, 7, j - 1);  // site: TransMM accumulator wait
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            }
            {
                const float2* Rj = reinterpret_cast<const float2*>(smem + SM8_R + uint32_t(j & 1) * SUB8_BYTES);
                unsigned char* B = smem + SM8_B;
                const int n = t & 15, rb = t >> 4;  // column n, rows 16 rb .. 16 rb + 15
                const uint32_t cs = colslot[n];
                float re[16], im[16];
#pragma unroll
                for (int qq = 0; qq < 16; qq++) {
                    const float2 a = Rj[rowslot[rb * 16 + qq] ^ cs];
                    re[qq] = a.x;
                    im[qq] = a.y;
                }
                if (PREC == HQ_MM_TF32) {
#pragma unroll
                    for (int h4 = 0; h4 < 4; h4++) {
                        const uint32_t o = kmajor_off(n, rb * 16 + 4 * h4, 256, 4);
                        const float4 vr = make_float4(to_tf32(re[4 * h4]), to_tf32(re[4 * h4 + 1]),
                                                      to_tf32(re[4 * h4 + 2]), to_tf32(re[4 * h4 + 3]));
                        const float4 vi = make_float4(to_tf32(im[4 * h4]), to_tf32(im[4 * h4 + 1]),
                                                      to_tf32(im[4 * h4 + 2]), to_tf32(im[4 * h4 + 3]));
                        *reinterpret_cast<float4*>(B + o) = vr;
                        *reinterpret_cast<float4*>(B + B8_COMP + o) = vi;
                        *reinterpret_cast<float4*>(B + 2 * B8_COMP + o) = make_float4(-vi.x, -vi.y, -vi.z, -vi.w);
                    }
                } else {
                    constexpr uint32_t b_lo = 8192;
                    const uint32_t sg = 0x80008000u;  // BF16 sign bits: -Bi exactly
#pragma unroll
                    for (int h8 = 0; h8 < 2; h8++) {
                        uint32_t hre[4], lre[4], him[4], lim[4];
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            const float x0 = re[8 * h8 + 2 * qq], x1 = re[8 * h8 + 2 * qq + 1];
                            const float y0 = im[8 * h8 + 2 * qq], y1 = im[8 * h8 + 2 * qq + 1];
                            const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
                            const __nv_bfloat16 g0 = __float2bfloat16_rn(y0), g1 = __float2bfloat16_rn(y1);
                            hre[qq] = pack_bf16(h0, h1);
                            lre[qq] = pack_bf16(__float2bfloat16_rn(x0 - __bfloat162float(h0)),
                                                __float2bfloat16_rn(x1 - __bfloat162float(h1)));
                            him[qq] = pack_bf16(g0, g1);
                            lim[qq] = pack_bf16(__float2bfloat16_rn(y0 - __bfloat162float(g0)),
                                                __float2bfloat16_rn(y1 - __bfloat162float(g1)));
                        }
                        const uint32_t o = kmajor_off(n, rb * 16 + 8 * h8, 256, 2);
                        *reinterpret_cast<uint4*>(B + o) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                        *reinterpret_cast<uint4*>(B + b_lo + o) = make_uint4(lre[0], lre[1], lre[2], lre[3]);
                        *reinterpret_cast<uint4*>(B + B8_COMP + o) = make_uint4(him[0], him[1], him[2], him[3]);
                        *reinterpret_cast<uint4*>(B + B8_COMP + b_lo + o) =
                            make_uint4(lim[0], lim[1], lim[2], lim[3]);
                        *reinterpret_cast<uint4*>(B + 2 * B8_COMP + o) =
                            make_uint4(him[0] ^ sg, him[1] ^ sg, him[2] ^ sg, him[3] ^ sg);
                        *reinterpret_cast<uint4*>(B + 2 * B8_COMP + b_lo + o) =
                            make_uint4(lim[0] ^ sg, lim[1] ^ sg, lim[2] ^ sg, lim[3] ^ sg);
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(m_bfull) : "memory");
            if (j > 0) epilogue(j - 1);
            load(j + 1);  // into the buffer sub-tile j - 1 just left
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM8_COLS));
}

// A operand of an 8-qubit group from U (256 x 256, column-major complex128):
// 16 chunks of 32 KB in the order the kernel consumes them, chunk
// (m * 4 + s) * 2 + part = Ur (part 0) or Ui (part 1) of rows 128 m .. 128 m + 127
// and K 64 s .. 64 s + 63, K-major (split BF16 hi at +0 and lo at +16 KB, or TF32).
__global__ void k_u_to_tc8(const double2* __restrict__ U, unsigned char* __restrict__ out, int prec) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 256 * 256) return;
    const int r = idx / 256, k = idx % 256;
    const double2 u = U[(size_t)k * 256 + r];
    const double v[2] = {u.x, u.y};
    const int m = r >> 7, rr = r & 127, s = k >> 6, kk = k & 63;
    for (int part = 0; part < 2; part++) {
        unsigned char* base = out + size_t((m * 4 + s) * 2 + part) * A8_CHUNK;
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
    return m == 6 ? 65536 : m == 7 ? 131072 : size_t(A8_CHUNKS) * A8_CHUNK;
}

void launch_u_to_tc_operand(int m, int precision, const double* d_u, void* d_out, cudaStream_t st) {
    HQ_REQUIRE(m >= 6 && m <= 8, HQ_ERR_UNSUPPORTED,
               "tensor-core TransMM runs 6- to 8-qubit groups (got %d)", m);
    if (m == 6)
        k_u_to_tc<<<64, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
    else if (m == 7)
        k_u_to_tc7<<<64, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
    else
        k_u_to_tc8<<<256, 256, 0, st>>>((const double2*)d_u, (unsigned char*)d_out, precision);
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

template <int PREC>
static void launch_prec7(const TransmmLaunch& p, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_tc7<PREC>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM7_TOTAL));
        attr = true;
    }
    const uint64_t slots = uint64_t(ctx().sm_count);
    const unsigned grid = (unsigned)(p.ntiles * 4 < slots ? p.ntiles * 4 : slots);
    k_transmm_tc7<PREC><<<grid, TC_THREADS, SM7_TOTAL, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

template <int PREC>
static void launch_prec8(const TransmmLaunch& p, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_tc8<PREC>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM8_TOTAL));
        attr = true;
    }
    const uint64_t slots = uint64_t(ctx().sm_count);
    const unsigned grid = (unsigned)(p.ntiles * 2 < slots ? p.ntiles * 2 : slots);
    k_transmm_tc8<PREC><<<grid, T8_THREADS, SM8_TOTAL, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_transmm_tc(const TransmmLaunch& p, cudaStream_t st) {
    HQ_REQUIRE(p.m >= 6 && p.m <= 8 && p.k == TC_TILE_BITS, HQ_ERR_UNSUPPORTED,
               "tensor-core TransMM runs 6- to 8-qubit groups on 13-qubit tiles");
    if (p.m == 8) {
        if (p.precision == HQ_MM_TF32)
            launch_prec8<HQ_MM_TF32>(p, st);
        else
            launch_prec8<HQ_MM_BF16X3>(p, st);
    } else if (p.m == 7) {
        if (p.precision == HQ_MM_TF32)
            launch_prec7<HQ_MM_TF32>(p, st);
        else
            launch_prec7<HQ_MM_BF16X3>(p, st);
    } else if (p.precision == HQ_MM_TF32) {
        launch_prec<HQ_MM_TF32>(p, st);
    } else {
        launch_prec<HQ_MM_BF16X3>(p, st);
    }
}

}  // namespace hq
