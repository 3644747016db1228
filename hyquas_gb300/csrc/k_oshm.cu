// OShareMem gate-group kernel for sm_103a.
//
// What it computes is the reference's OShareMem pass (src/kernelOpt.cu:426-433:
// fetchData 388-411, doCompute 215-386, saveData 413-423): a tile of 2^K
// amplitudes spanning K qubits is staged in shared memory, every gate of the
// group is applied to it, and the tile is written back in place.  Out-of-tile
// controls and diagonal gates become predicates/phases on the tile index, as
// the reference's GOC/GCC/GII/GZZ lowering does (src/executor.cpp:190-403).
//
// How it differs (GB300 design):
//   * Tiles are 2^13 amplitudes (64 KB of complex64), 8x the reference's 2^10.
//   * Gates are not applied one smem sweep + barrier each.  The host lowers a
//     group into PHASES: in a phase every thread holds 2^R amplitudes (R = 5,
//     the phase's "register qubits") in registers and applies all the phase's
//     gates there; only one shared-memory round trip per phase.
//   * Tiles are staged with 16-byte cp.async copies (LDGSTS), whose 2^c-amplitude
//     runs over the lowest physical qubits are coalesced; shared memory is
//     XOR-swizzled (linear map S below) so the phase gathers are conflict-free
//     for the lane-bit choices the host makes.
//   * 64-bit tile bases: works to n = 34 on one GPU.
#include <cuda_runtime.h>

#include "common.h"
#include "device.h"
#include "tile_io.cuh"

namespace hq {

namespace {

__host__ __device__ __forceinline__ uint32_t swz(uint32_t x) { return tile_swz(x); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int J, int NR>
__device__ __forceinline__ void op_u(float2 (&v)[NR], const float (&m)[8], uint32_t creg) {
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if (i & (1 << J)) continue;
        if ((uint32_t(i) & creg) != creg) continue;
        const int h = i | (1 << J);
        const float2 a = v[i], b = v[h];
        v[i].x = m[0] * a.x - m[1] * a.y + m[2] * b.x - m[3] * b.y;
        v[i].y = m[0] * a.y + m[1] * a.x + m[2] * b.y + m[3] * b.x;
        v[h].x = m[4] * a.x - m[5] * a.y + m[6] * b.x - m[7] * b.y;
        v[h].y = m[4] * a.y + m[5] * a.x + m[6] * b.y + m[7] * b.x;
    }
}

// real 2x2: [[m0, m2], [m4, m6]]
template <int J, int NR>
__device__ __forceinline__ void op_real(float2 (&v)[NR], const float (&m)[8], uint32_t creg) {
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if (i & (1 << J)) continue;
        if ((uint32_t(i) & creg) != creg) continue;
        const int h = i | (1 << J);
        const float2 a = v[i], b = v[h];
        v[i].x = m[0] * a.x + m[2] * b.x;
        v[i].y = m[0] * a.y + m[2] * b.y;
        v[h].x = m[4] * a.x + m[6] * b.x;
        v[h].y = m[4] * a.y + m[6] * b.y;
    }
}

template <int J, int NR>
__device__ __forceinline__ void op_x(float2 (&v)[NR], uint32_t creg) {
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if (i & (1 << J)) continue;
        if ((uint32_t(i) & creg) != creg) continue;
        const int h = i | (1 << J);
        const float2 a = v[i];
        v[i] = v[h];
        v[h] = a;
    }
}

template <int J, int NR>
__device__ __forceinline__ void op_dreg(float2 (&v)[NR], const float (&m)[8], uint32_t creg,
                                        bool d0_is_one) {
    const float2 d0 = make_float2(m[0], m[1]), d1 = make_float2(m[6], m[7]);
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if ((uint32_t(i) & creg) != creg) continue;
        if (i & (1 << J)) {
            v[i] = cmul(v[i], d1);
        } else if (!d0_is_one) {
            v[i] = cmul(v[i], d0);
        }
    }
}

template <int NR>
__device__ __forceinline__ void op_scale(float2 (&v)[NR], float2 f, uint32_t creg) {
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if ((uint32_t(i) & creg) != creg) continue;
        v[i] = cmul(v[i], f);
    }
}

#define HQ_DISPATCH_TBIT(R, TBIT, CALL)                 \
    switch (TBIT) {                                     \
        case 0: { constexpr int J = 0; CALL; } break;   \
        case 1: if constexpr (R > 1) { constexpr int J = 1; CALL; } break; \
        case 2: if constexpr (R > 2) { constexpr int J = 2; CALL; } break; \
        case 3: if constexpr (R > 3) { constexpr int J = 3; CALL; } break; \
        case 4: if constexpr (R > 4) { constexpr int J = 4; CALL; } break; \
        default: break;                                 \
    }

template <int K, int R>
__global__ void __launch_bounds__(1 << (K - R)) k_oshm(const OshmLaunch p) {
    constexpr int T = 1 << (K - R);      // threads per tile
    constexpr int NR = 1 << R;           // amplitudes per thread in a phase
    constexpr int PPT = (1 << (K - 1)) / T;  // 16-byte pieces per thread
    static_assert(PPT >= 1 && PPT <= 32, "piece count");
    extern __shared__ float4 smem4[];
    float2* sm = reinterpret_cast<float2*>(smem4);
    const int t = threadIdx.x;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    // Tile base: deposit the tile index into the non-tile (block) bits.
    const uint64_t base = tile_base(blockIdx.x, p.nruns, p.run_src, p.run_dst, p.run_len);

    // Stage the tile: piece (t + m*T) holds local amplitudes 2(t + m*T) and +1.
    const uint64_t toff = local_to_phys(uint32_t(t) << 1, K, p.tile_phys);  // local index 2t
    const uint32_t tslot = swz(uint32_t(t) << 1);
    const float2* __restrict__ gsrc = state + base + toff;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
#pragma unroll
    for (int m = 0; m < PPT; m++) {
        const uint32_t slot = tslot ^ p.piece_slot[m];
        const float2* g = gsrc + p.piece_off[m];
        cp_async16(sbase + slot * 8u, g);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();

    for (int ph = 0; ph < p.nphases; ph++) {
        const OshmPhase P = p.phases[ph];
        uint32_t gl = 0;
        uint64_t gphys = 0;
#pragma unroll
        for (int j = 0; j < K - R; j++) {
            if ((t >> j) & 1) {
                gl |= 1u << P.g_local[j];
                gphys |= uint64_t(1) << P.g_phys[j];
            }
        }
        const uint64_t pidx = base | gphys;  // physical index of this thread's register 0
        const uint32_t sb = swz(gl);
        uint32_t col[R];
#pragma unroll
        for (int j = 0; j < R; j++) col[j] = swz(1u << P.r_local[j]);

        float2 v[NR];
        if (P.pair0) {
#pragma unroll
            for (int i = 0; i < NR; i += 2) {
                uint32_t s = sb;
#pragma unroll
                for (int j = 1; j < R; j++)
                    if ((i >> j) & 1) s ^= col[j];
                const float4 q = smem4[s >> 1];
                v[i] = make_float2(q.x, q.y);
                v[i + 1] = make_float2(q.z, q.w);
            }
        } else {
#pragma unroll
            for (int i = 0; i < NR; i++) {
                uint32_t s = sb;
#pragma unroll
                for (int j = 0; j < R; j++)
                    if ((i >> j) & 1) s ^= col[j];
                v[i] = sm[s];
            }
        }

        float2 acc = make_float2(1.f, 0.f);
        for (uint32_t oi = P.op_begin; oi < P.op_end; oi++) {
            const OshmOp& o = p.ops[oi];
            const uint8_t kind = o.kind;
            const uint32_t creg = o.creg;
            const uint64_t cout = o.cout;
            if ((pidx & cout) != cout) continue;
            float m[8];
#pragma unroll
            for (int q = 0; q < 8; q++) m[q] = o.m[q];
            const int tb = o.tbit;
            switch (kind) {
                case OP_U: HQ_DISPATCH_TBIT(R, tb, (op_u<J, NR>(v, m, creg))); break;
                case OP_REAL: HQ_DISPATCH_TBIT(R, tb, (op_real<J, NR>(v, m, creg))); break;
                case OP_X: HQ_DISPATCH_TBIT(R, tb, (op_x<J, NR>(v, creg))); break;
                case OP_DREG: {
                    const bool d0one = o.d0_is_one != 0;
                    HQ_DISPATCH_TBIT(R, tb, (op_dreg<J, NR>(v, m, creg, d0one)));
                    break;
                }
                case OP_DOUT: {
                    const bool hi = (pidx & o.tout) != 0;
                    if (!hi && o.d0_is_one) break;
                    const float2 f = hi ? make_float2(m[6], m[7]) : make_float2(m[0], m[1]);
                    if (creg == 0)
                        acc = cmul(acc, f);
                    else
                        op_scale<NR>(v, f, creg);
                    break;
                }
                default: break;
            }
        }
        if (acc.x != 1.f || acc.y != 0.f) op_scale<NR>(v, acc, 0u);

        if (P.pair0) {
#pragma unroll
            for (int i = 0; i < NR; i += 2) {
                uint32_t s = sb;
#pragma unroll
                for (int j = 1; j < R; j++)
                    if ((i >> j) & 1) s ^= col[j];
                smem4[s >> 1] = make_float4(v[i].x, v[i].y, v[i + 1].x, v[i + 1].y);
            }
        } else {
#pragma unroll
            for (int i = 0; i < NR; i++) {
                uint32_t s = sb;
#pragma unroll
                for (int j = 0; j < R; j++)
                    if ((i >> j) & 1) s ^= col[j];
                sm[s] = v[i];
            }
        }
        __syncthreads();
    }

    // Write the tile back in place.
    float2* __restrict__ gdst = state + base + toff;
#pragma unroll
    for (int m = 0; m < PPT; m++) {
        const uint32_t slot = tslot ^ p.piece_slot[m];
        const float4 q = smem4[slot >> 1];
        *reinterpret_cast<float4*>(gdst + p.piece_off[m]) = q;
    }
}

template <int K, int R>
void launch_k(const OshmLaunch& p, cudaStream_t s) {
    constexpr int T = 1 << (K - R);
    const size_t smem = sizeof(float2) << K;
    static bool attr_set = false;
    if (!attr_set) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_oshm<K, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        attr_set = true;
    }
    HQ_REQUIRE(p.ntiles >= 1 && p.ntiles <= 0x7fffffffull, HQ_ERR_INVALID, "oshm: %llu tiles",
               (unsigned long long)p.ntiles);
    k_oshm<K, R><<<(unsigned)p.ntiles, T, smem, s>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

uint32_t oshm_swizzle(uint32_t x) { return swz(x); }

int oshm_reg_bits(int k) { return k >= 10 ? 5 : (k > 5 ? k - 5 : 1); }

int oshm_threads(int k, int r) { return 1 << (k - r); }

void launch_oshm(const OshmLaunch& p, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    switch (p.k) {
        case 6: launch_k<6, 1>(p, s); break;
        case 7: launch_k<7, 2>(p, s); break;
        case 8: launch_k<8, 3>(p, s); break;
        case 9: launch_k<9, 4>(p, s); break;
        case 10: launch_k<10, 5>(p, s); break;
        case 11: launch_k<11, 5>(p, s); break;
        case 12: launch_k<12, 5>(p, s); break;
        case 13: launch_k<13, 5>(p, s); break;
        default: fail(HQ_ERR_INVALID, "oshm: tile width %d not built (6..13)", p.k);
    }
}

}  // namespace hq
