// Plain-path kernels: one launch per gate (the reference's BACKEND=serial,
// src/kernelSimple.cu:335-446), |0..0> initialisation (src/kernelSimple.cu:9-37),
// FP64 probability reductions (src/kernelSimple.cu:467-516), amplitude gather
// (src/kernelSimple.cu:518-522) and the in-HBM qubit exchange used by remaps.
//
// All indices are 64-bit (the reference's `int nVec` overflows at n >= 32,
// src/kernelSimple.cu:338).  Every kernel is HBM-bound.
#include <cuda_runtime.h>

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
