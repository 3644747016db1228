// TransMM path: FP64 composition of a group's 2^m x 2^m unitary on the GPU
// (GateGroup::initCPUMatrix, src/schedule.cpp:578-702, moved on-device), and
// its application over tiles gathered in place.  The reference transposes the
// whole state with cuTT so the group's qubits become the lowest ones and then
// runs cublasZgemm/Cgemm (src/executor.cpp:533-551); here each CTA gathers a
// tile whose rows are the group's qubits (the permutation is folded into the
// gather addresses) and contracts it, so there is no transpose pass and the
// layout never changes.
//
// This file holds the FP32-SIMT contraction (HQ_MM_FP32) and the host glue;
// the tensor-core contractions (split-BF16 x3, TF32) are in k_transmm_tc.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "common.h"
#include "tile_io.cuh"
#include "transmm.h"

namespace hq {

void launch_transmm_tc(const TransmmLaunch& p, cudaStream_t st);
size_t transmm_tc_operand_bytes(int m, int precision);
void launch_u_to_tc_operand(int m, int precision, const double* d_u, void* d_out, cudaStream_t st);

namespace {

// ---- FP64 composition: one CTA per column c, U e_c built gate by gate -------
__global__ void k_compose(int m, const ComposeGate* __restrict__ gates, int ngates,
                          double* __restrict__ U) {
    extern __shared__ double2 vec[];
    const int dim = 1 << m;
    const int c = blockIdx.x;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) vec[i] = make_double2(i == c ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int gi = 0; gi < ngates; gi++) {
        const ComposeGate g = gates[gi];
        const int t = g.target;
        for (int pidx = threadIdx.x; pidx < dim / 2; pidx += blockDim.x) {
            const int lo = ((pidx >> t) << (t + 1)) | (pidx & ((1 << t) - 1));
            if (g.control >= 0 && !((lo >> g.control) & 1)) continue;
            if (g.control2 >= 0 && !((lo >> g.control2) & 1)) continue;
            const int hi = lo | (1 << t);
            const double2 a = vec[lo], b = vec[hi];
            vec[lo] = make_double2(g.m[0] * a.x - g.m[1] * a.y + g.m[2] * b.x - g.m[3] * b.y,
                                   g.m[0] * a.y + g.m[1] * a.x + g.m[2] * b.y + g.m[3] * b.x);
            vec[hi] = make_double2(g.m[4] * a.x - g.m[5] * a.y + g.m[6] * b.x - g.m[7] * b.y,
                                   g.m[4] * a.y + g.m[5] * a.x + g.m[6] * b.y + g.m[7] * b.x);
        }
        __syncthreads();
    }
    double2* col = reinterpret_cast<double2*>(U) + size_t(c) * dim;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) col[i] = vec[i];
}

__global__ void k_u_to_f32(int m, const double2* __restrict__ U, float2* __restrict__ out) {
    const int dim2 = 1 << (2 * m);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < dim2; i += gridDim.x * blockDim.x)
        out[i] = make_float2((float)U[i].x, (float)U[i].y);
}

// ---- FP32 SIMT contraction -------------------------------------------------------
// Tile = 2^13 amplitudes: 2^M rows (the group's qubits) x 2^(13-M) columns.
// 512 threads; thread = (column j, block of 16 rows).  C[:, j] = U B[:, j] is
// written straight to HBM (every column is read into shared memory first).
constexpr int kSimtK = 13;
constexpr int kSimtThreads = 512;

template <int M>
__global__ void __launch_bounds__(kSimtThreads) k_transmm_simt(const TransmmLaunch p) {
    constexpr int K = kSimtK, R = 1 << M, C = 1 << (K - M), RPT = 16;
    static_assert((R / RPT) * C == kSimtThreads, "thread mapping");
    extern __shared__ float4 smem4[];
    float2* tile = reinterpret_cast<float2*>(smem4);
    float2* U = tile + (1 << K);
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(U + R * R);
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(rowoff + R);
    const int tid = threadIdx.x;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);
    const uint64_t base = tile_base(blockIdx.x, p.nruns, p.run_src, p.run_dst, p.run_len);

    // stage the tile (same piece layout as the OShareMem kernel)
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tile);
    {
        const uint64_t toff = local_to_phys(uint32_t(tid) << 1, K, p.tile_phys);
        const uint32_t tslot = tile_swz(uint32_t(tid) << 1);
        constexpr int PPT = (1 << (K - 1)) / kSimtThreads;
#pragma unroll
        for (int mm = 0; mm < PPT; mm++)
            cp_async16(sbase + (tslot ^ p.piece_slot[mm]) * 8u, state + base + toff + p.piece_off[mm]);
    }
    // stage U (FP32 complex, column-major)
    {
        const float4* usrc = reinterpret_cast<const float4*>(p.umat);
        const uint32_t ubase = (uint32_t)__cvta_generic_to_shared(U);
        for (int i = tid; i < R * R / 2; i += kSimtThreads) cp_async16(ubase + i * 16u, usrc + i);
    }
    cp_async_commit();
    for (int r = tid; r < R; r += kSimtThreads) {
        uint32_t x = 0;
        uint64_t off = 0;
        for (int b = 0; b < M; b++)
            if ((r >> b) & 1) {
                x |= 1u << p.row_local[b];
                off |= uint64_t(1) << p.tile_phys[p.row_local[b]];
            }
        rowslot[r] = tile_swz(x);
        rowoff[r] = off;
    }
    cp_async_wait_all();
    __syncthreads();

    const int j = tid % C, rg = tid / C;
    uint32_t cx = 0;
    uint64_t coff = 0;
    for (int b = 0; b < K - M; b++)
        if ((j >> b) & 1) {
            cx |= 1u << p.col_local[b];
            coff |= uint64_t(1) << p.tile_phys[p.col_local[b]];
        }
    const uint32_t cslot = tile_swz(cx);
    float2 acc[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) acc[i] = make_float2(0.f, 0.f);
    const float4* U4 = reinterpret_cast<const float4*>(U);
#pragma unroll 2
    for (int k = 0; k < R; k++) {
        const float2 b = tile[rowslot[k] ^ cslot];
#pragma unroll
        for (int i = 0; i < RPT; i += 2) {
            const float4 u = U4[(k * R + rg * RPT + i) >> 1];  // U(r,k), U(r+1,k)
            acc[i].x += u.x * b.x - u.y * b.y;
            acc[i].y += u.x * b.y + u.y * b.x;
            acc[i + 1].x += u.z * b.x - u.w * b.y;
            acc[i + 1].y += u.z * b.y + u.w * b.x;
        }
    }
#pragma unroll
    for (int i = 0; i < RPT; i++) state[base + rowoff[rg * RPT + i] + coff] = acc[i];
}

// 8-qubit groups: U (256 x 256 complex, 512 KB) does not fit shared memory, so
// it streams through two 64 KB buffers of 32 columns (K slices) while the
// tile (256 rows x 32 columns) stays resident; the thread mapping is the one
// above with R = 256, C = 32.
constexpr int kSimt8Slice = 32;
constexpr size_t kSimt8Smem = (sizeof(float2) << kSimtK) + 2 * sizeof(float2) * kSimt8Slice * 256 +
                              (sizeof(uint64_t) + sizeof(uint32_t)) * 256;

__global__ void __launch_bounds__(kSimtThreads) k_transmm_simt8(const TransmmLaunch p) {
    constexpr int K = kSimtK, M = 8, R = 1 << M, C = 1 << (K - M), RPT = 16, KC = kSimt8Slice;
    static_assert((R / RPT) * C == kSimtThreads, "thread mapping");
    extern __shared__ float4 smem4[];
    float2* tile = reinterpret_cast<float2*>(smem4);
    float2* Ubuf = tile + (1 << K);  // two slices of KC columns
    uint64_t* rowoff = reinterpret_cast<uint64_t*>(Ubuf + 2 * KC * R);
    uint32_t* rowslot = reinterpret_cast<uint32_t*>(rowoff + R);
    const int tid = threadIdx.x;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);
    const float4* usrc = reinterpret_cast<const float4*>(p.umat);
    const uint64_t base = tile_base(blockIdx.x, p.nruns, p.run_src, p.run_dst, p.run_len);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tile);
    const uint32_t ubase = (uint32_t)__cvta_generic_to_shared(Ubuf);
    // slice c = columns c*KC .. c*KC+KC-1 of U (column-major: contiguous)
    auto stage_slice = [&](int c) {
        const uint32_t dst = ubase + uint32_t(c & 1) * (KC * R * 8u);
        const float4* src = usrc + size_t(c) * (KC * R / 2);
        for (int i = tid; i < KC * R / 2; i += kSimtThreads) cp_async16(dst + i * 16u, src + i);
    };
    {
        const uint64_t toff = local_to_phys(uint32_t(tid) << 1, K, p.tile_phys);
        const uint32_t tslot = tile_swz(uint32_t(tid) << 1);
        constexpr int PPT = (1 << (K - 1)) / kSimtThreads;
#pragma unroll
        for (int mm = 0; mm < PPT; mm++)
            cp_async16(sbase + (tslot ^ p.piece_slot[mm]) * 8u, state + base + toff + p.piece_off[mm]);
    }
    stage_slice(0);
    cp_async_commit();
    for (int r = tid; r < R; r += kSimtThreads) {
        uint32_t x = 0;
        uint64_t off = 0;
        for (int b = 0; b < M; b++)
            if ((r >> b) & 1) {
                x |= 1u << p.row_local[b];
                off |= uint64_t(1) << p.tile_phys[p.row_local[b]];
            }
        rowslot[r] = tile_swz(x);
        rowoff[r] = off;
    }
    const int j = tid % C, rg = tid / C;
    uint32_t cx = 0;
    uint64_t coff = 0;
    for (int b = 0; b < K - M; b++)
        if ((j >> b) & 1) {
            cx |= 1u << p.col_local[b];
            coff |= uint64_t(1) << p.tile_phys[p.col_local[b]];
        }
    const uint32_t cslot = tile_swz(cx);
    float2 acc[RPT];
#pragma unroll
    for (int i = 0; i < RPT; i++) acc[i] = make_float2(0.f, 0.f);
    for (int c = 0; c < R / KC; c++) {
        if (c + 1 < R / KC) stage_slice(c + 1);
        cp_async_commit();
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        const float4* U4 = reinterpret_cast<const float4*>(Ubuf + (c & 1) * (KC * R));
#pragma unroll 2
        for (int kk = 0; kk < KC; kk++) {
            const float2 b = tile[rowslot[c * KC + kk] ^ cslot];
#pragma unroll
            for (int i = 0; i < RPT; i += 2) {
                const float4 u = U4[(kk * R + rg * RPT + i) >> 1];  // U(r,k), U(r+1,k)
                acc[i].x += u.x * b.x - u.y * b.y;
                acc[i].y += u.x * b.y + u.y * b.x;
                acc[i + 1].x += u.z * b.x - u.w * b.y;
                acc[i + 1].y += u.z * b.y + u.w * b.x;
            }
        }
        __syncthreads();  // slice buffer c & 1 is refilled next iteration
    }
#pragma unroll
    for (int i = 0; i < RPT; i++) state[base + rowoff[rg * RPT + i] + coff] = acc[i];
}

void launch_simt8(const TransmmLaunch& p, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_simt8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)kSimt8Smem));
        attr = true;
    }
    k_transmm_simt8<<<(unsigned)p.ntiles, kSimtThreads, kSimt8Smem, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

template <int M>
void launch_simt_m(const TransmmLaunch& p, cudaStream_t st) {
    constexpr int R = 1 << M;
    const size_t smem = (sizeof(float2) << kSimtK) + sizeof(float2) * R * R +
                        (sizeof(uint64_t) + sizeof(uint32_t)) * R;
    static bool attr = false;
    if (!attr) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_transmm_simt<M>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    k_transmm_simt<M><<<(unsigned)p.ntiles, kSimtThreads, smem, st>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

int transmm_tile_bits(int m) { return kSimtK; }

void launch_compose(int m, const ComposeGate* d_gates, int ngates, double* d_u, cudaStream_t st) {
    const int dim = 1 << m;
    const int threads = std::max(32, std::min(256, dim / 2));
    k_compose<<<dim, threads, sizeof(double2) * dim, st>>>(m, d_gates, ngates, d_u);
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_u_to_f32(int m, const double* d_u, void* d_out, cudaStream_t st) {
    k_u_to_f32<<<64, 256, 0, st>>>(m, (const double2*)d_u, (float2*)d_out);
    HQ_CHECK_CUDA(cudaGetLastError());
}

void launch_transmm_simt(const TransmmLaunch& p, cudaStream_t st) {
    switch (p.m) {
        case 4: launch_simt_m<4>(p, st); break;
        case 5: launch_simt_m<5>(p, st); break;
        case 6: launch_simt_m<6>(p, st); break;
        case 7: launch_simt_m<7>(p, st); break;
        case 8: launch_simt8(p, st); break;
        default: fail(HQ_ERR_UNSUPPORTED, "FP32 SIMT TransMM supports 4..8 group qubits, got %d", p.m);
    }
}

// ---- host glue ---------------------------------------------------------------------

// group widths each contraction runs (narrower groups are padded with idle qubits)
static int min_mm_qubits(int precision) { return precision == HQ_MM_FP32 ? 4 : 6; }
static int max_mm_qubits(int) { return 8; }

// Rows = the group's qubits padded up to the kernel's minimum with the lowest
// free physical qubits; tile = rows + lowest non-row qubits up to 13 bits.
static void choose_rows(int n, uint64_t related, int precision, uint64_t& rows, uint64_t& tile) {
    int m = __builtin_popcountll(related);
    HQ_REQUIRE(m <= max_mm_qubits(precision), HQ_ERR_UNSUPPORTED,
               "TransMM group of %d qubits exceeds the kernel maximum %d", m,
               max_mm_qubits(precision));
    rows = related;
    for (int b = 0; b < n && __builtin_popcountll(rows) < min_mm_qubits(precision); b++)
        rows |= uint64_t(1) << b;
    tile = rows;
    for (int b = 0; b < n && __builtin_popcountll(tile) < kSimtK; b++) tile |= uint64_t(1) << b;
    HQ_REQUIRE(__builtin_popcountll(tile) == kSimtK, HQ_ERR_UNSUPPORTED,
               "TransMM needs at least %d qubits", kSimtK);
}

static std::vector<ComposeGate> to_compose(const std::vector<hq_gate>& gates, uint64_t rows) {
    int local[64];
    for (int b = 0, j = 0; b < 64; b++) local[b] = ((rows >> b) & 1) ? j++ : -1;
    std::vector<ComposeGate> out;
    for (const hq_gate& g : gates) {
        ComposeGate c;
        std::memset(&c, 0, sizeof(c));
        HQ_REQUIRE(local[g.target] >= 0, HQ_ERR_INVALID, "TransMM: gate target outside the group");
        c.target = local[g.target];
        c.control = g.control >= 0 ? local[g.control] : -1;
        c.control2 = g.control2 >= 0 ? local[g.control2] : -1;
        HQ_REQUIRE((g.control < 0 || c.control >= 0) && (g.control2 < 0 || c.control2 >= 0),
                   HQ_ERR_INVALID, "TransMM: gate control outside the group");
        for (int i = 0; i < 8; i++) c.m[i] = g.mat[i];
        out.push_back(c);
    }
    return out;
}

static TransmmLaunch make_launch(int n, int m, uint64_t rows, uint64_t tile, int precision) {
    TransmmLaunch p;
    std::memset(&p, 0, sizeof(p));
    p.n = n;
    p.m = m;
    p.k = kSimtK;
    p.precision = precision;
    p.ntiles = uint64_t(1) << (n - kSimtK);
    int loc[64];
    for (int b = 0, j = 0; b < n; b++) {
        loc[b] = -1;
        if ((tile >> b) & 1) {
            loc[b] = j;
            p.tile_phys[j++] = (uint8_t)b;
        }
    }
    for (int b = 0, r = 0, c = 0; b < n; b++) {
        if (!((tile >> b) & 1)) continue;
        if ((rows >> b) & 1)
            p.row_local[r++] = (uint8_t)loc[b];
        else
            p.col_local[c++] = (uint8_t)loc[b];
    }
    int src = 0, nr = 0;
    for (int b = 0; b < n;) {
        if ((tile >> b) & 1) {
            b++;
            continue;
        }
        int len = 0;
        while (b + len < n && !((tile >> (b + len)) & 1)) len++;
        p.run_src[nr] = (uint8_t)src;
        p.run_dst[nr] = (uint8_t)b;
        p.run_len[nr] = (uint8_t)len;
        nr++;
        src += len;
        b += len;
    }
    p.nruns = nr;
    // piece tables for kSimtThreads threads (the tensor-core kernel uses the same)
    const int ppt = (1 << (kSimtK - 1)) / kSimtThreads;
    for (int mm = 0; mm < ppt; mm++) {
        const uint32_t local = uint32_t(2 * mm * kSimtThreads);
        uint64_t off = 0;
        for (int j = 0; j < kSimtK; j++)
            if ((local >> j) & 1) off |= uint64_t(1) << p.tile_phys[j];
        p.piece_off[mm] = off;
        p.piece_slot[mm] = tile_swz(local);
    }
    // sub-tiles for the 6-qubit tensor-core kernel: the top column bit fixed
    // (64 x 64 sub-tiles); the 7- and 8-qubit kernels take whole tiles
    if (m == 6) {
        const int ncol = kSimtK - m, nsplit = 1;
        const int sub_bits = kSimtK - nsplit;
        int sub[16];
        for (int j = 0; j < kSimtK; j++) sub[j] = 0;
        bool fixed[16] = {false};
        for (int f = 0; f < nsplit; f++) {
            const int j = p.col_local[ncol - nsplit + f];
            fixed[j] = true;
            p.split_off[f] = uint64_t(1) << p.tile_phys[j];
        }
        for (int j = 0, q = 0; j < kSimtK; j++) {
            sub[j] = fixed[j] ? -1 : q;
            if (!fixed[j]) p.sub_phys[q++] = p.tile_phys[j];
        }
        for (int r = 0; r < m; r++) p.row_sub[r] = (uint8_t)sub[p.row_local[r]];
        for (int c = 0; c < ncol - nsplit; c++) p.col_sub[c] = (uint8_t)sub[p.col_local[c]];
        const int ppt = (1 << (sub_bits - 1)) / 256;
        for (int mm = 0; mm < ppt; mm++) {
            const uint32_t local = uint32_t(2 * mm * 256);
            uint64_t off = 0;
            for (int j = 0; j < sub_bits; j++)
                if ((local >> j) & 1) off |= uint64_t(1) << p.sub_phys[j];
            p.sub_piece_off[mm] = off;
            p.sub_piece_slot[mm] = tile_swz(local);
        }
    }
    return p;
}

static size_t operand_bytes(int m, int precision) {
    if (precision == HQ_MM_FP32) return sizeof(float2) << (2 * m);
    return transmm_tc_operand_bytes(m, precision);
}

static void prepare_operand(int m, int precision, const double* d_u, void* d_out, cudaStream_t st) {
    if (precision == HQ_MM_FP32)
        launch_u_to_f32(m, d_u, d_out, st);
    else
        launch_u_to_tc_operand(m, precision, d_u, d_out, st);
}

static void launch_any(const TransmmLaunch& p, cudaStream_t st) {
    if (p.precision == HQ_MM_FP32)
        launch_transmm_simt(p, st);
    else
        launch_transmm_tc(p, st);
}

void transmm_prepare(int n, const GroupPlan& gp, DeviceGroup& dg, const CompileConfig& cfg,
                     std::vector<double>& umats) {
    (void)umats;
    HQ_REQUIRE(n >= kSimtK, HQ_ERR_UNSUPPORTED, "TransMM needs n >= %d", kSimtK);
    uint64_t rows, tile;
    choose_rows(n, gp.related, cfg.mm_precision, rows, tile);
    dg.mm_m = __builtin_popcountll(rows);
    dg.mm_rows = rows;
    dg.mm_tile = tile;
    dg.mm_precision = cfg.mm_precision;
}

void transmm_finalize(hq_circuit_s* c) {
    cudaStream_t st = ctx().stream;
    size_t u_off = 0, op_off = 0;
    for (DeviceGroup& dg : c->dgroups) {
        if (dg.backend != HQ_BACKEND_TRANSMM) continue;
        dg.umat_off = u_off;
        dg.operand_off = op_off;
        u_off += size_t(2) << (2 * dg.mm_m);
        op_off += (operand_bytes(dg.mm_m, dg.mm_precision) + 255) & ~size_t(255);
    }
    if (u_off == 0) return;
    c->umats_bytes = sizeof(double) * u_off;
    c->d_umats = (double*)dev_alloc_ordered(c->umats_bytes);
    c->mm_scratch_bytes = op_off;
    c->d_mm_scratch = dev_alloc_ordered(op_off);
    for (DeviceGroup& dg : c->dgroups) {
        if (dg.backend != HQ_BACKEND_TRANSMM) continue;
        std::vector<ComposeGate> cg = to_compose(dg.phys_gates, dg.mm_rows);
        const size_t gb = sizeof(ComposeGate) * std::max<size_t>(1, cg.size());
        ComposeGate* d_g = (ComposeGate*)dev_alloc_ordered(gb);
        HQ_CHECK_CUDA(cudaMemcpyAsync(d_g, cg.data(), sizeof(ComposeGate) * cg.size(),
                                      cudaMemcpyHostToDevice, st));
        launch_compose(dg.mm_m, d_g, (int)cg.size(), c->d_umats + dg.umat_off, st);
        prepare_operand(dg.mm_m, dg.mm_precision, c->d_umats + dg.umat_off,
                        (char*)c->d_mm_scratch + dg.operand_off, st);
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
        dev_free_ordered(d_g, gb);
    }
}

void transmm_launch(hq_circuit_s* c, const DeviceGroup& dg, void* state, cudaStream_t st) {
    TransmmLaunch p = make_launch(c->n, dg.mm_m, dg.mm_rows, dg.mm_tile, dg.mm_precision);
    p.state = state;
    p.umat = (const char*)c->d_mm_scratch + dg.operand_off;
    p.err = ctx().d_error;
    launch_any(p, st);
}

void compose_unitary(int m, const std::vector<ComposeGate>& gates, double* d_u, cudaStream_t st) {
    const size_t gb = sizeof(ComposeGate) * std::max<size_t>(1, gates.size());
    ComposeGate* d_g = (ComposeGate*)dev_alloc_ordered(gb);
    try {
        HQ_CHECK_CUDA(cudaMemcpyAsync(d_g, gates.data(), sizeof(ComposeGate) * gates.size(),
                                      cudaMemcpyHostToDevice, st));
        launch_compose(m, d_g, (int)gates.size(), d_u, st);
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        dev_free_ordered(d_g, gb);
        throw;
    }
    dev_free_ordered(d_g, gb);
}

void apply_unitary_device(hq_state_s* s, const double* d_u, int m, uint64_t rows_phys,
                          int precision) {
    state_wait_copy(s);
    cudaStream_t st = ctx().stream;
    uint64_t rows = rows_phys, tile;
    HQ_REQUIRE(__builtin_popcountll(rows) == m, HQ_ERR_INVALID, "row mask/width mismatch");
    HQ_REQUIRE(m >= min_mm_qubits(precision) && m <= max_mm_qubits(precision), HQ_ERR_UNSUPPORTED,
               "unitary width %d unsupported for precision %d", m, precision);
    HQ_REQUIRE(s->n >= kSimtK, HQ_ERR_UNSUPPORTED, "TransMM needs n >= %d", kSimtK);
    tile = rows;
    for (int b = 0; b < s->n && __builtin_popcountll(tile) < kSimtK; b++) tile |= uint64_t(1) << b;
    const size_t ob = operand_bytes(m, precision);
    void* d_op = dev_alloc_ordered(ob);
    try {
        prepare_operand(m, precision, d_u, d_op, st);
        TransmmLaunch p = make_launch(s->n, m, rows, tile, precision);
        p.state = s->d;
        p.umat = d_op;
        p.err = ctx().d_error;
        launch_any(p, st);
        HQ_CHECK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        dev_free_ordered(d_op, ob);
        throw;
    }
    dev_free_ordered(d_op, ob);
    check_device_error();
}

}  // namespace hq

// ---- C-ABI entry points for single TransMM groups --------------------------------
using namespace hq;

#define HQ_API_TRY try {
#define HQ_API_CATCH                              \
    }                                             \
    catch (const Failure& f) {                    \
        set_last_error(f.what());                 \
        return f.code;                            \
    }                                             \
    catch (const std::exception& e) {             \
        set_last_error(e.what());                 \
        return HQ_ERR_INVALID;                    \
    }                                             \
    return HQ_OK;

// widen a row set to the contraction's minimum width with the lowest free
// physical qubits (the fused unitary acts as identity on them)
static uint64_t pad_rows(int n, uint64_t rows, int precision) {
    for (int b = 0; b < n && __builtin_popcountll(rows) < min_mm_qubits(precision); b++)
        rows |= uint64_t(1) << b;
    return rows;
}

static uint64_t logical_to_phys_mask(const hq_state_s* s, uint64_t logical) {
    uint64_t m = 0;
    for (int q = 0; q < s->n; q++)
        if ((logical >> q) & 1) m |= uint64_t(1) << s->pos[q];
    return m;
}

extern "C" hq_status hq_group_unitary(const hq_gate* gates, int32_t num_gates, uint64_t group_mask,
                                      double* out) {
    HQ_API_TRY
    clear_last_error();
    HQ_REQUIRE(out != nullptr, HQ_ERR_INVALID, "unitary_out must not be NULL");
    HQ_REQUIRE(num_gates >= 0 && (num_gates == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    const int m = __builtin_popcountll(group_mask);
    HQ_REQUIRE(m >= 1 && m <= 10, HQ_ERR_INVALID, "group width %d out of range [1,10]", m);
    std::vector<hq_gate> v(gates, gates + num_gates);
    for (auto& g : v) validate_gate(g, 64);
    std::vector<ComposeGate> cg = to_compose(v, group_mask);
    const size_t ub = sizeof(double) * (size_t(2) << (2 * m));
    double* d_u = (double*)dev_alloc_ordered(ub);
    try {
        compose_unitary(m, cg, d_u, ctx().stream);
        HQ_CHECK_CUDA(cudaMemcpy(out, d_u, ub, cudaMemcpyDeviceToHost));
    } catch (...) {
        dev_free_ordered(d_u, ub);
        throw;
    }
    dev_free_ordered(d_u, ub);
    HQ_API_CATCH
}

extern "C" hq_status hq_apply_transmm_group(hq_state s, const hq_gate* gates, int32_t num_gates,
                                            uint64_t group_mask, int32_t precision) {
    HQ_API_TRY
    clear_last_error();
    HQ_REQUIRE(s != nullptr, HQ_ERR_INVALID, "state must not be NULL");
    HQ_REQUIRE(num_gates >= 0 && (num_gates == 0 || gates), HQ_ERR_INVALID, "bad gate list");
    std::vector<hq_gate> phys;
    for (int i = 0; i < num_gates; i++) {
        validate_gate(gates[i], s->n);
        hq_gate g = gates[i];
        g.target = s->pos[g.target];
        if (g.control >= 0) g.control = s->pos[g.control];
        if (g.control2 >= 0) g.control2 = s->pos[g.control2];
        phys.push_back(g);
    }
    uint64_t rows = logical_to_phys_mask(s, group_mask);
    rows = pad_rows(s->n, rows, precision);
    const int m = __builtin_popcountll(rows);
    std::vector<ComposeGate> cg = to_compose(phys, rows);
    const size_t ub = sizeof(double) * (size_t(2) << (2 * m));
    double* d_u = (double*)dev_alloc_ordered(ub);
    try {
        compose_unitary(m, cg, d_u, ctx().stream);
        apply_unitary_device(s, d_u, m, rows, precision);
    } catch (...) {
        dev_free_ordered(d_u, ub);
        throw;
    }
    dev_free_ordered(d_u, ub);
    HQ_API_CATCH
}

extern "C" hq_status hq_apply_unitary(hq_state s, const double* unitary, uint64_t group_mask,
                                      int32_t precision) {
    HQ_API_TRY
    clear_last_error();
    HQ_REQUIRE(s != nullptr && unitary != nullptr, HQ_ERR_INVALID, "null argument");
    const uint64_t rows = logical_to_phys_mask(s, group_mask);
    const int m = __builtin_popcountll(rows);
    HQ_REQUIRE(m >= 1 && m <= 8, HQ_ERR_INVALID, "unitary width %d", m);
    // local row bit j = j-th lowest PHYSICAL row; reorder the caller's logical
    // bit order (bit j = j-th lowest logical qubit of the mask) if they differ
    std::vector<int> lq;
    for (int q = 0; q < s->n; q++)
        if ((group_mask >> q) & 1) lq.push_back(q);
    std::vector<int> lbit(m);  // caller bit j -> physical-order bit
    for (int j = 0; j < m; j++) {
        int rank = 0;
        for (int x = 0; x < m; x++)
            if (s->pos[lq[x]] < s->pos[lq[j]]) rank++;
        lbit[j] = rank;
    }
    const size_t dim = size_t(1) << m;
    auto remap = [&](size_t i) {
        size_t o = 0;
        for (int j = 0; j < m; j++)
            if ((i >> j) & 1) o |= size_t(1) << lbit[j];
        return o;
    };
    std::vector<double> u(2 * dim * dim);
    for (size_t c = 0; c < dim; c++)
        for (size_t r = 0; r < dim; r++) {
            const size_t src = 2 * (c * dim + r), dst = 2 * (remap(c) * dim + remap(r));
            u[dst] = unitary[src];
            u[dst + 1] = unitary[src + 1];
        }
    // pad to the contraction's width: U' = U on the original rows, identity on the added ones
    const uint64_t prow = pad_rows(s->n, rows, precision);
    const int pm = __builtin_popcountll(prow);
    if (pm != m) {
        std::vector<int> orig_bit;  // padded local bit -> original local bit or -1
        for (int b = 0, j = 0; b < s->n; b++) {
            if (!((prow >> b) & 1)) continue;
            int o = -1;
            if ((rows >> b) & 1) o = __builtin_popcountll(rows & ((uint64_t(1) << b) - 1));
            orig_bit.push_back(o);
            j++;
        }
        const size_t pdim = size_t(1) << pm;
        std::vector<double> pu(2 * pdim * pdim, 0.0);
        for (size_t c = 0; c < pdim; c++)
            for (size_t r = 0; r < pdim; r++) {
                size_t oc = 0, orr = 0;
                bool same_extra = true;
                for (int b = 0; b < pm; b++) {
                    const int o = orig_bit[b];
                    const size_t cb = (c >> b) & 1, rb = (r >> b) & 1;
                    if (o < 0) {
                        if (cb != rb) same_extra = false;
                    } else {
                        oc |= cb << o;
                        orr |= rb << o;
                    }
                }
                if (!same_extra) continue;
                pu[2 * (c * pdim + r)] = u[2 * (oc * dim + orr)];
                pu[2 * (c * pdim + r) + 1] = u[2 * (oc * dim + orr) + 1];
            }
        u.swap(pu);
    }
    const size_t ub = sizeof(double) * u.size();
    double* d_u = (double*)dev_alloc_ordered(ub);
    try {
        HQ_CHECK_CUDA(cudaMemcpy(d_u, u.data(), ub, cudaMemcpyHostToDevice));
        apply_unitary_device(s, d_u, pm, prow, precision);
    } catch (...) {
        dev_free_ordered(d_u, ub);
        throw;
    }
    dev_free_ordered(d_u, ub);
    HQ_API_CATCH
}
