// Sampling computational-basis outcomes of a state vector.
//
// The reference measures one qubit's probability (kernelMeasure,
// src/kernelSimple.cu:482-512) and prints amplitudes (src/circuit.cpp:285-308);
// it has no sampler.  Here the state is cut into blocks of 2^12 amplitudes,
// the FP64 probability of every block is summed and scanned into a
// cumulative distribution, and each shot draws u in [0, 1) from a
// SplitMix64 stream (Steele, Lea and Flood, 2014), finds its block by binary
// search over the block CDF and its amplitude by a warp-wide FP64 scan of the
// block.  Probabilities are |a|^2 of the complex64 amplitudes in FP64.
#include <cuda_runtime.h>

#include "common.h"
#include "device.h"

namespace hq {

namespace {

constexpr int kBlk = 1 << kSampleBlockBits;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double prob(const float2* a, uint64_t i) {
    const float2 v = a[i];
    return double(v.x) * double(v.x) + double(v.y) * double(v.y);
}

// one CTA of 256 threads per block of 2^12 amplitudes
__global__ void __launch_bounds__(256) k_block_prob(const float2* __restrict__ a, uint64_t namps,
                                                    double* __restrict__ out) {
    const uint64_t base = uint64_t(blockIdx.x) * kBlk;
    double s = 0.0;
    for (int j = threadIdx.x; j < kBlk; j += 256) {
        const uint64_t i = base + j;
        if (i < namps) s += prob(a, i);
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// inclusive scan of v[0..nb) in place, one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_scan(double* __restrict__ v, uint64_t nb) {
    const int t = threadIdx.x;
    const uint64_t per = (nb + 1023) / 1024;
    const uint64_t lo = uint64_t(t) * per, hi = lo + per < nb ? lo + per : nb;
    double s = 0.0;
    for (uint64_t i = lo; i < hi; i++) {
        s += v[i];
        v[i] = s;
    }
    __shared__ double part[1024];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        double run = 0.0;
        for (int j = 0; j < 1024; j++) {
            const double x = part[j];
            part[j] = run;
            run += x;
        }
    }
    __syncthreads();
    const double off = part[t];
    for (uint64_t i = lo; i < hi; i++) v[i] += off;
}

// one warp per shot
__global__ void k_draw(const float2* __restrict__ a, uint64_t namps, const double* __restrict__ cdf,
                       uint64_t nb, int shots, uint64_t seed, uint64_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int shot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (shot >= shots) return;
    const double total = cdf[nb - 1];
    const double u = double(mix64(seed + 0x9e3779b97f4a7c15ull * uint64_t(shot + 1)) >> 11) *
                     (1.0 / 9007199254740992.0);
    // rounded product (never fused into the subtraction below), so the FP64
    // steps of a draw are fixed and can be restated exactly on the host
    const double target = __dmul_rn(u, total);
    // first block whose cumulative probability exceeds the target
    uint64_t lo = 0, hi = nb - 1;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (cdf[mid] > target)
            hi = mid;
        else
            lo = mid + 1;
    }
    double rem = target - (lo ? cdf[lo - 1] : 0.0);
    const uint64_t base = lo * kBlk;
    const uint64_t end = base + kBlk < namps ? base + kBlk : namps;
    uint64_t pick = ~uint64_t(0), last_nz = base;
    for (uint64_t c = base; c < end && pick == ~uint64_t(0); c += 32) {
        const uint64_t i = c + lane;
        const double p = i < end ? prob(a, i) : 0.0;
        double run = p;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, run, d);
            if (lane >= d) run += y;
        }
        const unsigned hit = __ballot_sync(0xffffffffu, i < end && p > 0.0 && run > rem);
        const unsigned nz = __ballot_sync(0xffffffffu, i < end && p > 0.0);
        if (nz) last_nz = c + 31 - __clz(nz);
        if (hit) {
            pick = c + __ffs(hit) - 1;
        } else {
            rem -= __shfl_sync(0xffffffffu, run, 31);
        }
    }
    // rounding left the target past the block's sum: take its last non-zero amplitude
    if (lane == 0) out[shot] = pick != ~uint64_t(0) ? pick : last_nz;
}

}  // namespace

uint64_t sample_mix64(uint64_t z) { return mix64(z); }

size_t sample_scratch_doubles(int n) {
    const uint64_t namps = uint64_t(1) << n;
    return size_t((namps + kBlk - 1) / kBlk);
}

void launch_sample(const void* state, int n, int shots, uint64_t seed, double* d_cdf,
                   uint64_t* d_out, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t namps = uint64_t(1) << n;
    const uint64_t nb = (namps + kBlk - 1) / kBlk;
    const float2* a = (const float2*)state;
    k_block_prob<<<(unsigned)nb, 256, 0, st>>>(a, namps, d_cdf);
    HQ_CHECK_CUDA(cudaGetLastError());
    k_scan<<<1, 1024, 0, st>>>(d_cdf, nb);
    HQ_CHECK_CUDA(cudaGetLastError());
    if (shots > 0) {
        const int threads = 256;
        const unsigned blocks = (unsigned)((uint64_t(shots) * 32 + threads - 1) / threads);
        k_draw<<<blocks, threads, 0, st>>>(a, namps, d_cdf, nb, shots, seed, d_out);
        HQ_CHECK_CUDA(cudaGetLastError());
    }
}

}  // namespace hq
