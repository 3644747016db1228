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
//   * Registers hold structure-of-arrays f32x2 vectors pairing the two
//     amplitudes that differ in physical qubit 0, so the gate arithmetic runs
//     on Blackwell's packed FFMA2/FADD2/FMUL2 (two amplitudes per instruction).
//   * Hadamard-like gates (H, sqrt(X) = RX(pi/2), sqrt(Y) = RY(pi/2)) run as
//     adds/subtracts; their 1/sqrt(2) factors are collected by the host and
//     applied as one multiply per phase that needs it.
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

// Packed f32x2 arithmetic on native 64-bit registers (PTX add/sub/mul/fma
// .f32x2, sm_100+): a v2 holds two fp32 values and never round-trips
// through a float pair.
typedef unsigned long long v2;
__device__ __forceinline__ v2 vmul(v2 a, v2 b) {
    v2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ v2 vfma(v2 a, v2 b, v2 c) {
    v2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ v2 vpack(float lo, float hi) {
    v2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void vunpack(v2 a, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a));
}
__device__ __forceinline__ v2 vdup(float x) { return vpack(x, x); }
__device__ __forceinline__ v2 vswap(v2 a) {
    float l, h;
    vunpack(a, l, h);
    return vpack(h, l);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Amplitudes of one thread: register index i = 2 j + lane, vectors
// re[j] = (re(2j), re(2j+1)), im[j] likewise.  Register bit J >= 1 is bit
// J-1 of the vector index; register bit 0 is the lane.
template <int NV>
struct Amps {
    v2 re[NV], im[NV];
};

// ---- in-place register updates ----------------------------------------------
// Every amplitude register is read and written through the same asm operand,
// so each amplitude stays in one register through the op dispatch (no copies
// where the dispatch's branches merge).

// (l, h) <- (a l + b h, c l + d h), real coefficients (applied to re and im alike)
__device__ __forceinline__ void ip_real(v2& l, v2& h, v2 a, v2 b, v2 c, v2 d) {
    asm("{\n\t.reg .b64 t;\n\t"
        "mul.rn.f32x2 t, %2, %0;\n\tfma.rn.f32x2 t, %3, %1, t;\n\t"
        "mul.rn.f32x2 %1, %5, %1;\n\tfma.rn.f32x2 %1, %4, %0, %1;\n\t"
        "mov.b64 %0, t;\n\t}"
        : "+l"(l), "+l"(h) : "l"(a), "l"(b), "l"(c), "l"(d));
}
// (l, h) <- (l + h, l - h)
__device__ __forceinline__ void ip_bfly(v2& l, v2& h) {
    asm("{\n\t.reg .b64 t;\n\tadd.rn.f32x2 t, %0, %1;\n\tsub.rn.f32x2 %1, %0, %1;\n\tmov.b64 %0, t;\n\t}"
        : "+l"(l), "+l"(h));
}
// (l, h) <- (l - h, l + h)
__device__ __forceinline__ void ip_bfly_y(v2& l, v2& h) {
    asm("{\n\t.reg .b64 t;\n\tsub.rn.f32x2 t, %0, %1;\n\tadd.rn.f32x2 %1, %0, %1;\n\tmov.b64 %0, t;\n\t}"
        : "+l"(l), "+l"(h));
}
// sqrt(X) without its 1/sqrt2: (l, h) <- (l - i h, h - i l)
__device__ __forceinline__ void ip_sx(v2& lr, v2& li, v2& hr, v2& hi) {
    asm("{\n\t.reg .b64 a, b;\n\t"
        "add.rn.f32x2 a, %0, %3;\n\tsub.rn.f32x2 b, %1, %2;\n\t"
        "add.rn.f32x2 %2, %2, %1;\n\tsub.rn.f32x2 %3, %3, %0;\n\t"
        "mov.b64 %0, a;\n\tmov.b64 %1, b;\n\t}"
        : "+l"(lr), "+l"(li), "+l"(hr), "+l"(hi));
}
__device__ __forceinline__ void ip_swap(v2& l, v2& h) {
    asm("{\n\t.reg .b64 t;\n\tmov.b64 t, %0;\n\tmov.b64 %0, %1;\n\tmov.b64 %1, t;\n\t}" : "+l"(l), "+l"(h));
}
// (r, i) <- (er r - ei i, ei r + er i); ein = -ei
__device__ __forceinline__ void ip_cmul(v2& r, v2& i, v2 er, v2 ei, v2 ein) {
    asm("{\n\t.reg .b64 t;\n\t"
        "mul.rn.f32x2 t, %2, %0;\n\tfma.rn.f32x2 t, %4, %1, t;\n\t"
        "mul.rn.f32x2 %1, %2, %1;\n\tfma.rn.f32x2 %1, %3, %0, %1;\n\t"
        "mov.b64 %0, t;\n\t}"
        : "+l"(r), "+l"(i) : "l"(er), "l"(ei), "l"(ein));
}
__device__ __forceinline__ void ip_xor(v2& x, v2 m) { asm("xor.b64 %0, %0, %1;" : "+l"(x) : "l"(m)); }
// general complex 2x2: l' = a l + b h, h' = c l + d h (x = re, y = im, n = -im)
__device__ __forceinline__ void ip_u(v2& lr, v2& li, v2& hr, v2& hi, const v2 (&k)[12]) {
    asm("{\n\t.reg .b64 tr, ti, u;\n\t"
        "mul.rn.f32x2 tr, %4, %0;\n\tfma.rn.f32x2 tr, %6, %1, tr;\n\t"
        "fma.rn.f32x2 tr, %7, %2, tr;\n\tfma.rn.f32x2 tr, %9, %3, tr;\n\t"
        "mul.rn.f32x2 ti, %4, %1;\n\tfma.rn.f32x2 ti, %5, %0, ti;\n\t"
        "fma.rn.f32x2 ti, %7, %3, ti;\n\tfma.rn.f32x2 ti, %8, %2, ti;\n\t"
        "mul.rn.f32x2 u, %13, %3;\n\tfma.rn.f32x2 u, %14, %2, u;\n\t"
        "fma.rn.f32x2 u, %10, %1, u;\n\tfma.rn.f32x2 u, %11, %0, u;\n\t"
        "mul.rn.f32x2 %2, %13, %2;\n\tfma.rn.f32x2 %2, %15, %3, %2;\n\t"
        "fma.rn.f32x2 %2, %10, %0, %2;\n\tfma.rn.f32x2 %2, %12, %1, %2;\n\t"
        "mov.b64 %3, u;\n\tmov.b64 %0, tr;\n\tmov.b64 %1, ti;\n\t}"
        : "+l"(lr), "+l"(li), "+l"(hr), "+l"(hi)
        : "l"(k[0]), "l"(k[1]), "l"(k[2]), "l"(k[3]), "l"(k[4]), "l"(k[5]), "l"(k[6]),
          "l"(k[7]), "l"(k[8]), "l"(k[9]), "l"(k[10]), "l"(k[11]));
}
// [[a, i b], [i c, d]], real a..d: l' = a l + i b h, h' = i c l + d h
__device__ __forceinline__ void ip_imoff(v2& lr, v2& li, v2& hr, v2& hi, v2 a, v2 b, v2 bn, v2 c,
                                         v2 cn, v2 d) {
    asm("{\n\t.reg .b64 tr, ti, u;\n\t"
        "mul.rn.f32x2 tr, %4, %0;\n\tfma.rn.f32x2 tr, %6, %3, tr;\n\t"
        "mul.rn.f32x2 ti, %4, %1;\n\tfma.rn.f32x2 ti, %5, %2, ti;\n\t"
        "mul.rn.f32x2 u, %9, %3;\n\tfma.rn.f32x2 u, %7, %0, u;\n\t"
        "mul.rn.f32x2 %2, %9, %2;\n\tfma.rn.f32x2 %2, %8, %1, %2;\n\t"
        "mov.b64 %3, u;\n\tmov.b64 %0, tr;\n\tmov.b64 %1, ti;\n\t}"
        : "+l"(lr), "+l"(li), "+l"(hr), "+l"(hi)
        : "l"(a), "l"(b), "l"(bn), "l"(c), "l"(cn), "l"(d));
}

// rotation by the shears x += a y; y += b x; x += a y (a = -tan(phi/2), b = sin(phi))
__device__ __forceinline__ void ip_shear(v2& x, v2& y, v2 a, v2 b) {
    asm("fma.rn.f32x2 %0, %2, %1, %0;\n\tfma.rn.f32x2 %1, %3, %0, %1;\n\tfma.rn.f32x2 %0, %2, %1, %0;"
        : "+l"(x), "+l"(y) : "l"(a), "l"(b));
}

// ---- uncontrolled ops on register bit J >= 1 --------------------------------
#define HQ_PAIRS_IP(J, NV, BODY)                           \
    _Pragma("unroll") for (int j = 0; j < NV; j++) {        \
        if (j & (1 << (J - 1))) continue;                    \
        const int h = j | (1 << (J - 1));                    \
        BODY                                                 \
    }
// read-only pair access for the register-controlled ops below
#define HQ_PAIRS(J, NV, BODY)                              \
    _Pragma("unroll") for (int j = 0; j < NV; j++) {        \
        if (j & (1 << (J - 1))) continue;                    \
        const int h = j | (1 << (J - 1));                    \
        const v2 lr = A.re[j], li = A.im[j], hr = A.re[h], hi = A.im[h]; \
        BODY                                                 \
    }

template <int J, int NV>
__device__ __forceinline__ void op_u(Amps<NV>& A, const float (&m)[8]) {
    const v2 k[12] = {vdup(m[0]), vdup(m[1]), vdup(-m[1]), vdup(m[2]), vdup(m[3]), vdup(-m[3]),
                      vdup(m[4]), vdup(m[5]), vdup(-m[5]), vdup(m[6]), vdup(m[7]), vdup(-m[7])};
    HQ_PAIRS_IP(J, NV, { ip_u(A.re[j], A.im[j], A.re[h], A.im[h], k); })
}

template <int J, int NV>
__device__ __forceinline__ void op_real(Amps<NV>& A, const float (&m)[8]) {
    const v2 a = vdup(m[0]), b = vdup(m[2]), c = vdup(m[4]), d = vdup(m[6]);
    HQ_PAIRS_IP(J, NV, {
        ip_real(A.re[j], A.re[h], a, b, c, d);
        ip_real(A.im[j], A.im[h], a, b, c, d);
    })
}

// [[a, i b], [i c, d]]
template <int J, int NV>
__device__ __forceinline__ void op_imoff(Amps<NV>& A, const float (&m)[8]) {
    const v2 a = vdup(m[0]), b = vdup(m[3]), bn = vdup(-m[3]), c = vdup(m[5]), cn = vdup(-m[5]),
             d = vdup(m[6]);
    HQ_PAIRS_IP(J, NV, { ip_imoff(A.re[j], A.im[j], A.re[h], A.im[h], a, b, bn, c, cn, d); })
}

template <int J, int NV>
__device__ __forceinline__ void op_h(Amps<NV>& A) {
    HQ_PAIRS_IP(J, NV, {
        ip_bfly(A.re[j], A.re[h]);
        ip_bfly(A.im[j], A.im[h]);
    })
}

template <int J, int NV>
__device__ __forceinline__ void op_sy(Amps<NV>& A) {
    HQ_PAIRS_IP(J, NV, {
        ip_bfly_y(A.re[j], A.re[h]);
        ip_bfly_y(A.im[j], A.im[h]);
    })
}

template <int J, int NV>
__device__ __forceinline__ void op_sx(Amps<NV>& A) {
    HQ_PAIRS_IP(J, NV, { ip_sx(A.re[j], A.im[j], A.re[h], A.im[h]); })
}

template <int J, int NV>
__device__ __forceinline__ void op_x(Amps<NV>& A) {
    HQ_PAIRS_IP(J, NV, {
        ip_swap(A.re[j], A.re[h]);
        ip_swap(A.im[j], A.im[h]);
    })
}

template <int J, int NV>
__device__ __forceinline__ void op_dreg(Amps<NV>& A, const float (&m)[8], bool d0one) {
    const v2 er = vdup(m[6]), ei = vdup(m[7]), ein = vdup(-m[7]);
    const v2 fr = vdup(m[0]), fi = vdup(m[1]), fin = vdup(-m[1]);
    HQ_PAIRS_IP(J, NV, {
        ip_cmul(A.re[h], A.im[h], er, ei, ein);
        if (!d0one) ip_cmul(A.re[j], A.im[j], fr, fi, fin);
    })
}

template <int J, int NV>
__device__ __forceinline__ void op_drot(Amps<NV>& A, const float (&m)[8], bool neg) {
    const v2 a = vdup(m[0]), b = vdup(m[1]), sgn = 0x8000000080000000ull;
    HQ_PAIRS_IP(J, NV, {
        ip_shear(A.re[h], A.im[h], a, b);
        if (neg) {
            ip_xor(A.re[h], sgn);
            ip_xor(A.im[h], sgn);
        }
    })
}

// [[c, -s], [s, c]]: (lo, hi) rotated in the real and in the imaginary plane
// with three shears each (the negation of an angle reduced by pi covers every
// register of the thread, so apply_op folds it into the phase factor)
template <int J, int NV>
__device__ __forceinline__ void op_rrot(Amps<NV>& A, const float (&m)[8]) {
    const v2 a = vdup(m[0]), b = vdup(m[1]);
    HQ_PAIRS_IP(J, NV, {
        ip_shear(A.re[j], A.re[h], a, b);
        ip_shear(A.im[j], A.im[h], a, b);
    })
}

template <int J, int NV>
__device__ __forceinline__ void op_neghi(Amps<NV>& A) {
    const v2 sgn = 0x8000000080000000ull;
    HQ_PAIRS_IP(J, NV, {
        ip_xor(A.re[h], sgn);
        ip_xor(A.im[h], sgn);
    })
}

// ---- ops on register bit 0 (the vector lane: lo = low half, hi = high half) -----
template <int NV>
__device__ __forceinline__ void lane_u(Amps<NV>& A, const float (&m)[8], uint32_t creg) {
    const v2 P = vpack(m[0], m[6]), Q = vpack(m[1], m[7]), Qn = vpack(-m[1], -m[7]);
    const v2 S = vpack(m[2], m[4]), Tt = vpack(m[3], m[5]), Tn = vpack(-m[3], -m[5]);
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        const v2 r = A.re[j], i = A.im[j], rs = vswap(r), is = vswap(i);
        A.re[j] = vfma(Tn, is, vfma(S, rs, vfma(Qn, i, vmul(P, r))));
        A.im[j] = vfma(Tt, rs, vfma(S, is, vfma(Q, r, vmul(P, i))));
    }
}

template <int NV>
__device__ __forceinline__ void lane_x(Amps<NV>& A, uint32_t creg) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        A.re[j] = vswap(A.re[j]);
        A.im[j] = vswap(A.im[j]);
    }
}

template <int NV>
__device__ __forceinline__ void lane_diag(Amps<NV>& A, const float (&m)[8], uint32_t creg) {
    const v2 R = vpack(m[0], m[6]), I = vpack(m[1], m[7]), In = vpack(-m[1], -m[7]);
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        const v2 r = A.re[j], i = A.im[j];
        A.re[j] = vfma(In, i, vmul(R, r));
        A.im[j] = vfma(I, r, vmul(R, i));
    }
}

// Lane ops with a structured matrix: the other lane's value comes from a
// swapped copy (register renaming) and one packed constant holds both lanes'
// coefficients, so a component costs one or two packed instructions instead
// of four.  In place, like the helpers above.
// x <- P x + S swap(x): real [[a, b], [c, d]] with P = (a, d), S = (b, c)
__device__ __forceinline__ void ip_lane_real(v2& x, v2 P, v2 S) {
    asm("{\n\t.reg .b32 a, b;\n\t.reg .b64 s, t;\n\t"
        "mov.b64 {a, b}, %0;\n\tmov.b64 s, {b, a};\n\t"
        "mul.rn.f32x2 t, %1, %0;\n\tfma.rn.f32x2 %0, %2, s, t;\n\t}"
        : "+l"(x) : "l"(P), "l"(S));
}
// x <- K x + swap(x)  (H: K = (1, -1))
__device__ __forceinline__ void ip_lane_h(v2& x, v2 K) {
    asm("{\n\t.reg .b32 a, b;\n\t.reg .b64 s;\n\t"
        "mov.b64 {a, b}, %0;\n\tmov.b64 s, {b, a};\n\tfma.rn.f32x2 %0, %1, %0, s;\n\t}"
        : "+l"(x) : "l"(K));
}
// x <- x + K swap(x)  (sqrt(Y): K = (-1, 1))
__device__ __forceinline__ void ip_lane_y(v2& x, v2 K) {
    asm("{\n\t.reg .b32 a, b;\n\t.reg .b64 s;\n\t"
        "mov.b64 {a, b}, %0;\n\tmov.b64 s, {b, a};\n\tfma.rn.f32x2 %0, %1, s, %0;\n\t}"
        : "+l"(x) : "l"(K));
}
// sqrt(X) without its 1/sqrt2 on the lane: re <- re + swap(im), im <- im - swap(re)
__device__ __forceinline__ void ip_lane_sx(v2& r, v2& i) {
    asm("{\n\t.reg .b32 a, b, c, d;\n\t.reg .b64 s, u;\n\t"
        "mov.b64 {a, b}, %0;\n\tmov.b64 s, {b, a};\n\t"
        "mov.b64 {c, d}, %1;\n\tmov.b64 u, {d, c};\n\t"
        "add.rn.f32x2 %0, %0, u;\n\tsub.rn.f32x2 %1, %1, s;\n\t}"
        : "+l"(r), "+l"(i));
}
// [[a, i b], [i c, d]] on the lane: re <- P re + Xn swap(im), im <- P im + X swap(re)
// with P = (a, d), X = (b, c), Xn = -X
__device__ __forceinline__ void ip_lane_imoff(v2& r, v2& i, v2 P, v2 X, v2 Xn) {
    asm("{\n\t.reg .b32 a, b, c, d;\n\t.reg .b64 s, u, t;\n\t"
        "mov.b64 {a, b}, %0;\n\tmov.b64 s, {b, a};\n\t"
        "mov.b64 {c, d}, %1;\n\tmov.b64 u, {d, c};\n\t"
        "mul.rn.f32x2 t, %2, %0;\n\tfma.rn.f32x2 %0, %4, u, t;\n\t"
        "mul.rn.f32x2 t, %2, %1;\n\tfma.rn.f32x2 %1, %3, s, t;\n\t}"
        : "+l"(r), "+l"(i) : "l"(P), "l"(X), "l"(Xn));
}

template <int NV>
__device__ __forceinline__ void lane_real(Amps<NV>& A, const float (&m)[8], uint32_t creg) {
    const v2 P = vpack(m[0], m[6]), S = vpack(m[2], m[4]);
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        ip_lane_real(A.re[j], P, S);
        ip_lane_real(A.im[j], P, S);
    }
}

template <int NV>
__device__ __forceinline__ void lane_imoff(Amps<NV>& A, const float (&m)[8], uint32_t creg) {
    const v2 P = vpack(m[0], m[6]), X = vpack(m[3], m[5]), Xn = vpack(-m[3], -m[5]);
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        ip_lane_imoff(A.re[j], A.im[j], P, X, Xn);
    }
}

// H, sqrt(Y), sqrt(X) without their 1/sqrt2 (deferred to the phase scale):
// H: (lo + hi, lo - hi); sqrt(Y): (lo - hi, lo + hi); sqrt(X): (lo - i hi, hi - i lo)
template <int KIND, int NV>
__device__ __forceinline__ void lane_had(Amps<NV>& A, uint32_t creg) {
    const v2 K = KIND == OP_H ? vpack(1.f, -1.f) : vpack(-1.f, 1.f);
#pragma unroll
    for (int j = 0; j < NV; j++) {
        if ((uint32_t(2 * j) & creg) != creg) continue;
        if (KIND == OP_H) {
            ip_lane_h(A.re[j], K);
            ip_lane_h(A.im[j], K);
        } else if (KIND == OP_SY) {
            ip_lane_y(A.re[j], K);
            ip_lane_y(A.im[j], K);
        } else {
            ip_lane_sx(A.re[j], A.im[j]);
        }
    }
}

// ---- register-controlled ops on bit J >= 1: compute, then keep per lane ----------
__device__ __forceinline__ v2 pick(bool o0, bool o1, v2 nw, v2 old) {
    if (o0 && o1) return nw;
    if (!o0 && !o1) return old;
    float nl, nh, ol, oh;
    vunpack(nw, nl, nh);
    vunpack(old, ol, oh);
    return vpack(o0 ? nl : ol, o1 ? nh : oh);
}

template <int J, int NV>
__device__ __forceinline__ void ctl_u(Amps<NV>& A, const float (&m)[8], uint32_t creg) {
    const v2 a = vdup(m[0]), ai = vdup(m[1]), ain = vdup(-m[1]);
    const v2 b = vdup(m[2]), bi = vdup(m[3]), bin = vdup(-m[3]);
    const v2 c = vdup(m[4]), ci = vdup(m[5]), cin = vdup(-m[5]);
    const v2 d = vdup(m[6]), di = vdup(m[7]), din = vdup(-m[7]);
    HQ_PAIRS(J, NV, {
        const bool o0 = (uint32_t(2 * j) & creg) == creg;
        const bool o1 = (uint32_t(2 * j + 1) & creg) == creg;
        A.re[j] = pick(o0, o1, vfma(bin, hi, vfma(b, hr, vfma(ain, li, vmul(a, lr)))), lr);
        A.im[j] = pick(o0, o1, vfma(bi, hr, vfma(b, hi, vfma(ai, lr, vmul(a, li)))), li);
        A.re[h] = pick(o0, o1, vfma(din, hi, vfma(d, hr, vfma(cin, li, vmul(c, lr)))), hr);
        A.im[h] = pick(o0, o1, vfma(di, hr, vfma(d, hi, vfma(ci, lr, vmul(c, li)))), hi);
    })
}

template <int J, int NV>
__device__ __forceinline__ void ctl_x(Amps<NV>& A, uint32_t creg) {
    HQ_PAIRS(J, NV, {
        const bool o0 = (uint32_t(2 * j) & creg) == creg;
        const bool o1 = (uint32_t(2 * j + 1) & creg) == creg;
        A.re[j] = pick(o0, o1, hr, lr);
        A.im[j] = pick(o0, o1, hi, li);
        A.re[h] = pick(o0, o1, lr, hr);
        A.im[h] = pick(o0, o1, li, hi);
    })
}

template <int J, int NV>
__device__ __forceinline__ void ctl_diag(Amps<NV>& A, const float (&m)[8], uint32_t creg,
                                         bool d0one) {
    HQ_PAIRS(J, NV, {
        const bool o0 = (uint32_t(2 * j) & creg) == creg;
        const bool o1 = (uint32_t(2 * j + 1) & creg) == creg;
        const v2 er = vpack(o0 ? m[6] : 1.f, o1 ? m[6] : 1.f);
        const v2 ei = vpack(o0 ? m[7] : 0.f, o1 ? m[7] : 0.f);
        const v2 ein = vpack(o0 ? -m[7] : 0.f, o1 ? -m[7] : 0.f);
        A.re[h] = vfma(ein, hi, vmul(er, hr));
        A.im[h] = vfma(ei, hr, vmul(er, hi));
        if (!d0one) {
            const v2 fr = vpack(o0 ? m[0] : 1.f, o1 ? m[0] : 1.f);
            const v2 fi = vpack(o0 ? m[1] : 0.f, o1 ? m[1] : 0.f);
            const v2 fin = vpack(o0 ? -m[1] : 0.f, o1 ? -m[1] : 0.f);
            A.re[j] = vfma(fin, li, vmul(fr, lr));
            A.im[j] = vfma(fi, lr, vmul(fr, li));
        }
    })
}

// multiply the registers selected by creg by the complex factor f
template <int NV>
__device__ __forceinline__ void scale_sel(Amps<NV>& A, float2 f, uint32_t creg) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
        const bool o0 = (uint32_t(2 * j) & creg) == creg;
        const bool o1 = (uint32_t(2 * j + 1) & creg) == creg;
        if (!o0 && !o1) continue;
        const v2 R = vpack(o0 ? f.x : 1.f, o1 ? f.x : 1.f);
        const v2 I = vpack(o0 ? f.y : 0.f, o1 ? f.y : 0.f);
        const v2 In = vpack(o0 ? -f.y : 0.f, o1 ? -f.y : 0.f);
        const v2 r = A.re[j], i = A.im[j];
        A.re[j] = vfma(In, i, vmul(R, r));
        A.im[j] = vfma(I, r, vmul(R, i));
    }
}

// One flat dispatch on (register control?, kind, register bit): a single
// switch, rather than nested ones, keeps the amplitude registers in place
// across the cases (measured: ~25 % fewer instructions per op).
#define HQ_CODE(CTL, KIND, TB) ((((CTL) ? 1u : 0u) << 7) | (uint32_t(KIND) << 3) | uint32_t(TB))
#define HQ_CASE_J(CTL, KIND, CALL)                                                            \
    case HQ_CODE(CTL, KIND, 1): if constexpr (R > 1) { constexpr int J = 1; CALL; } break;    \
    case HQ_CODE(CTL, KIND, 2): if constexpr (R > 2) { constexpr int J = 2; CALL; } break;    \
    case HQ_CODE(CTL, KIND, 3): if constexpr (R > 3) { constexpr int J = 3; CALL; } break;    \
    case HQ_CODE(CTL, KIND, 4): if constexpr (R > 4) { constexpr int J = 4; CALL; } break;
#define HQ_CASE_LANE(KIND, CALL)      \
    case HQ_CODE(0, KIND, 0):         \
    case HQ_CODE(1, KIND, 0): CALL; break;

template <int R>
__device__ __forceinline__ void apply_op(Amps<(1 << (R - 1))>& A, const uint4 hdr,
                                         const OshmOp* __restrict__ op, uint64_t pidx,
                                         float2& acc) {
    constexpr int NV = 1 << (R - 1);
    const uint32_t kind = hdr.x & 0xffu, tb = (hdr.x >> 8) & 0xffu, flags = (hdr.x >> 16) & 0xffu;
    const uint32_t creg = hdr.y;
    if (flags & OPF_COUT) {
        const uint64_t cout = (uint64_t(hdr.w) << 32) | hdr.z;
        if ((pidx & cout) != cout) return;
    }
    float m[8];
    if (kind != OP_H && kind != OP_SY && kind != OP_SX && kind != OP_X && kind != OP_NEGHI) {
        const float4* mp = reinterpret_cast<const float4*>(op->m);
        const float4 m0 = __ldg(mp), m1 = __ldg(mp + 1);
        m[0] = m0.x; m[1] = m0.y; m[2] = m0.z; m[3] = m0.w;
        m[4] = m1.x; m[5] = m1.y; m[6] = m1.z; m[7] = m1.w;
    } else {
        // the sign flip as a diagonal with d0 = 1, d1 = -1
        m[0] = 1.f; m[1] = 0.f; m[2] = 0.f; m[3] = 0.f;
        m[4] = 0.f; m[5] = 0.f; m[6] = -1.f; m[7] = 0.f;
    }
    const bool d0one = (flags & OPF_D0_ONE) != 0;
    if (kind == OP_DOUT) {
        const uint64_t tout = __ldg(reinterpret_cast<const unsigned long long*>(&op->tout));
        const bool hiset = (pidx & tout) != 0;
        if (!hiset && d0one) return;
        const float2 f = hiset ? make_float2(m[6], m[7]) : make_float2(m[0], m[1]);
        if (creg == 0)
            acc = cmul(acc, f);
        else
            scale_sel<NV>(A, f, creg);
        return;
    }
    if (kind == OP_RROT && (flags & OPF_NEG)) acc = make_float2(-acc.x, -acc.y);
    switch (HQ_CODE(flags & OPF_CREG, kind, tb)) {
        HQ_CASE_LANE(OP_X, (lane_x<NV>(A, creg)))
        HQ_CASE_LANE(OP_DREG, (lane_diag<NV>(A, m, creg)))
        HQ_CASE_LANE(OP_NEGHI, (lane_diag<NV>(A, m, creg)))
        HQ_CASE_LANE(OP_U, (lane_u<NV>(A, m, creg)))
        HQ_CASE_LANE(OP_REAL, (lane_real<NV>(A, m, creg)))
        HQ_CASE_LANE(OP_IMOFF, (lane_imoff<NV>(A, m, creg)))
        HQ_CASE_LANE(OP_H, (lane_had<OP_H, NV>(A, creg)))
        HQ_CASE_LANE(OP_SY, (lane_had<OP_SY, NV>(A, creg)))
        HQ_CASE_LANE(OP_SX, (lane_had<OP_SX, NV>(A, creg)))
        HQ_CASE_J(0, OP_U, (op_u<J, NV>(A, m)))
        HQ_CASE_J(0, OP_REAL, (op_real<J, NV>(A, m)))
        HQ_CASE_J(0, OP_IMOFF, (op_imoff<J, NV>(A, m)))
        HQ_CASE_J(0, OP_H, (op_h<J, NV>(A)))
        HQ_CASE_J(0, OP_SY, (op_sy<J, NV>(A)))
        HQ_CASE_J(0, OP_SX, (op_sx<J, NV>(A)))
        HQ_CASE_J(0, OP_X, (op_x<J, NV>(A)))
        HQ_CASE_J(0, OP_DREG, (op_dreg<J, NV>(A, m, d0one)))
        HQ_CASE_J(0, OP_NEGHI, (op_neghi<J, NV>(A)))
        HQ_CASE_J(0, OP_DROT, (op_drot<J, NV>(A, m, (flags & OPF_NEG) != 0)))
        HQ_CASE_J(0, OP_RROT, (op_rrot<J, NV>(A, m)))
        HQ_CASE_J(1, OP_X, (ctl_x<J, NV>(A, creg)))
        HQ_CASE_J(1, OP_NEGHI, (ctl_diag<J, NV>(A, m, creg, true)))
        HQ_CASE_J(1, OP_DREG, (ctl_diag<J, NV>(A, m, creg, d0one)))
        HQ_CASE_J(1, OP_U, (ctl_u<J, NV>(A, m, creg)))
        HQ_CASE_J(1, OP_REAL, (ctl_u<J, NV>(A, m, creg)))
        HQ_CASE_J(1, OP_IMOFF, (ctl_u<J, NV>(A, m, creg)))
        default: break;
    }
}

// Every phase of the group program on one tile staged in `buf` (pieces as
// loaded; they hold (re0, re1, im0, im1) afterwards).  Thread t of the tile's
// 2^(p.k-R) threads; threads of the block beyond those pass `active` = false
// and only take part in the barriers.
template <int K, int R>
__device__ __forceinline__ void run_phases(const OshmLaunch& p, float4* buf, uint64_t base, int t,
                                           bool active) {
    constexpr int NV = 1 << (R - 1);
    for (int ph = 0; ph < p.nphases; ph++) {
        if (active) {
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
            const uint64_t pidx = base | gphys;  // physical index of register 0
            const uint32_t sb = swz(gl);
            uint32_t col[R];
#pragma unroll
            for (int j = 1; j < R; j++) col[j] = swz(1u << P.r_local[j]);

            Amps<NV> A;
            // gather: pieces are (re0, im0, re1, im1) before the first phase and
            // (re0, re1, im0, im1) after it
#pragma unroll
            for (int j = 0; j < NV; j++) {
                uint32_t s = sb;
#pragma unroll
                for (int b = 1; b < R; b++)
                    if ((j >> (b - 1)) & 1) s ^= col[b];
                if (ph == 0) {
                    const float4 q = buf[s >> 1];
                    A.re[j] = vpack(q.x, q.z);
                    A.im[j] = vpack(q.y, q.w);
                } else {
                    const ulonglong2 q = reinterpret_cast<const ulonglong2*>(buf)[s >> 1];
                    A.re[j] = q.x;
                    A.im[j] = q.y;
                }
            }

            float2 acc = make_float2(1.f, 0.f);
            const OshmOp* __restrict__ ops = p.ops;
            uint4 nxt = make_uint4(0, 0, 0, 0);
            if (P.op_begin < P.op_end) nxt = __ldg(reinterpret_cast<const uint4*>(ops + P.op_begin));
            for (uint32_t oi = P.op_begin; oi < P.op_end; oi++) {
                const uint4 hdr = nxt;
                if (oi + 1 < P.op_end) nxt = __ldg(reinterpret_cast<const uint4*>(ops + oi + 1));
                apply_op<R>(A, hdr, ops + oi, pidx, acc);
            }
            float2 f = acc;
            if (P.scale != 1.f) f = make_float2(f.x * P.scale, f.y * P.scale);
            if (f.y != 0.f) {
                const v2 R2 = vdup(f.x), I2 = vdup(f.y), In2 = vdup(-f.y);
#pragma unroll
                for (int j = 0; j < NV; j++) {
                    const v2 r = A.re[j], i = A.im[j];
                    A.re[j] = vfma(In2, i, vmul(R2, r));
                    A.im[j] = vfma(I2, r, vmul(R2, i));
                }
            } else if (f.x != 1.f) {
                const v2 R2 = vdup(f.x);
#pragma unroll
                for (int j = 0; j < NV; j++) {
                    A.re[j] = vmul(R2, A.re[j]);
                    A.im[j] = vmul(R2, A.im[j]);
                }
            }

#pragma unroll
            for (int j = 0; j < NV; j++) {
                uint32_t s = sb;
#pragma unroll
                for (int b = 1; b < R; b++)
                    if ((j >> (b - 1)) & 1) s ^= col[b];
                reinterpret_cast<ulonglong2*>(buf)[s >> 1] = make_ulonglong2(A.re[j], A.im[j]);
            }
        }
        __syncthreads();
    }
}

template <int K, int R>
__global__ void __launch_bounds__(1 << (K - R)) k_oshm(const OshmLaunch p) {
    constexpr int T = 1 << (K - R);      // threads per tile
    constexpr int PPT = (1 << (K - 1)) / T;  // 16-byte pieces per thread
    static_assert(PPT >= 1 && PPT <= 32, "piece count");
    constexpr int TILE4 = 1 << (K - 1);  // float4 pieces per tile buffer
    extern __shared__ float4 smem4[];     // two tile buffers
    const int t = threadIdx.x;
    float2* __restrict__ state = reinterpret_cast<float2*>(p.state);

    // Piece (t + m*T) of a tile holds local amplitudes 2(t + m*T) and +1.
    const uint64_t toff = local_to_phys(uint32_t(t) << 1, K, p.tile_phys);
    const uint32_t tslot = swz(uint32_t(t) << 1);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem4);

    // stage tile u into buffer b, as loaded: (re0, im0, re1, im1)
    auto load_tile = [&](uint64_t u, int b) {
        const uint64_t tb = tile_base(u, p.nruns, p.run_src, p.run_dst, p.run_len);
        const float2* __restrict__ gsrc = state + tb + toff;
        const uint32_t bb = sbase + uint32_t(b) * TILE4 * 16u;
#pragma unroll
        for (int m = 0; m < PPT; m++)
            cp_async16(bb + (tslot ^ p.piece_slot[m]) * 8u, gsrc + p.piece_off[m]);
        cp_async_commit();
    };

    // Persistent loop over tiles; the next tile's copy is in flight while the
    // current one is computed.
    uint64_t u = blockIdx.x;
    if (u < p.ntiles) load_tile(u, 0);
    for (int it = 0; u < p.ntiles; it++, u += gridDim.x) {
        const uint64_t un = u + gridDim.x;
        if (un < p.ntiles) {
            load_tile(un, (it + 1) & 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            cp_async_wait_all();
        }
        __syncthreads();
        float4* buf = smem4 + (it & 1) * TILE4;
        const uint64_t base = tile_base(u, p.nruns, p.run_src, p.run_dst, p.run_len);

        run_phases<K, R>(p, buf, base, t, true);

        // write back in place, (re0, re1, im0, im1) -> (re0, im0, re1, im1)
        float2* __restrict__ gdst = state + base + toff;
        const bool soa = p.nphases > 0;
#pragma unroll
        for (int m = 0; m < PPT; m++) {
            const uint32_t piece = (tslot ^ p.piece_slot[m]) >> 1;
            float4 out;
            if (soa) {
                const ulonglong2 q = reinterpret_cast<const ulonglong2*>(buf)[piece];
                vunpack(q.x, out.x, out.z);
                vunpack(q.y, out.y, out.w);
            } else {
                out = buf[piece];
            }
            *reinterpret_cast<float4*>(gdst + p.piece_off[m]) = out;
        }
        __syncthreads();  // this buffer is refilled two iterations on
    }
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for *ctr >= need (acquire).  Gives up after about two seconds,
// or as soon as another block has recorded an error, and returns false; the
// first block to give up records err = {1, site 8, item}.
__device__ bool wait_counter(const uint32_t* ctr, uint32_t need, int* err, uint32_t item) {
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 0;; spin++) {
        uint32_t v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= need) return true;
        if (*reinterpret_cast<volatile int*>(err) != 0) return false;
        if (spin >= (1u << 24) || globaltimer_ns() - t0 > 2000000000ull) {
            if (atomicCAS(err, 0, 1) == 0) {
                err[1] = 8;  // site: batched item dependency wait
                err[2] = (int)item;
            }
            return false;
        }
        __nanosleep(128);
    }
}

// Batched OShareMem: persistent blocks pull (circuit, group, tile range) items.
// Tiles of every width k in [10, K] run with R = 5 register qubits: the
// 2^(k-5) threads of a tile each hold 32 amplitudes and move 16 pieces; the
// other threads of the block only join the barriers.
template <int K, int R>
__global__ void __launch_bounds__(1 << (K - R)) k_oshm_batch(const BatchLaunch b) {
    constexpr int T = 1 << (K - R);
    constexpr int PPT = 1 << (R - 1);    // pieces per thread, any tile width
    constexpr int TILE4 = 1 << (K - 1);
    extern __shared__ float4 smem4[];
    __shared__ OshmLaunch sp;            // the current item's group
    __shared__ uint32_t s_item;
    __shared__ int s_ok;
    const int t = threadIdx.x;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem4);
    const uint32_t tslot = swz(uint32_t(t) << 1);

    for (;;) {
        if (t == 0) s_item = atomicAdd(b.head, 1u);
        __syncthreads();
        const uint32_t i = s_item;
        if (i >= b.nitems) return;
        const BatchItem it = b.items[i];
        if (t == 0) {
            bool ok = true;
            const uint32_t need = i == b.stall_item ? 0xffffffffu : it.need;
            if (need) ok = wait_counter(b.done + it.circuit, need, b.err, i);
            __threadfence();
            s_ok = ok;
        }
        {
            const uint4* src = reinterpret_cast<const uint4*>(b.groups + it.group);
            for (int w = t; w < int(sizeof(OshmLaunch) / 16); w += T)
                reinterpret_cast<uint4*>(&sp)[w] = src[w];
        }
        __syncthreads();
        if (!s_ok) return;

        const int kc = sp.k;
        const bool active = t < (1 << (kc - R));
        const bool zero = (it.flags & ITEM_FIRST) && b.zero_init;
        float2* __restrict__ state = reinterpret_cast<float2*>(sp.state);
        const uint64_t toff = active ? local_to_phys(uint32_t(t) << 1, kc, sp.tile_phys) : 0;

        auto stage = [&](uint64_t u, int bsel) {
            if (active) {
                if (zero) {
                    float4* dst = smem4 + bsel * TILE4;
#pragma unroll
                    for (int m = 0; m < PPT; m++)
                        dst[(tslot ^ sp.piece_slot[m]) >> 1] =
                            make_float4((u == 0 && t == 0 && m == 0) ? 1.f : 0.f, 0.f, 0.f, 0.f);
                } else {
                    const uint64_t tb = tile_base(u, sp.nruns, sp.run_src, sp.run_dst, sp.run_len);
                    const float2* __restrict__ gsrc = state + tb + toff;
                    const uint32_t bb = sbase + uint32_t(bsel) * TILE4 * 16u;
#pragma unroll
                    for (int m = 0; m < PPT; m++)
                        cp_async16(bb + (tslot ^ sp.piece_slot[m]) * 8u, gsrc + sp.piece_off[m]);
                }
            }
            cp_async_commit();
        };

        const uint64_t uend = uint64_t(it.tile0) + it.count;
        uint64_t u = it.tile0;
        stage(u, 0);
        for (int j = 0; u < uend; j++, u++) {
            if (u + 1 < uend) {
                stage(u + 1, (j + 1) & 1);
                asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            } else {
                cp_async_wait_all();
            }
            __syncthreads();
            float4* buf = smem4 + (j & 1) * TILE4;
            const uint64_t base = tile_base(u, sp.nruns, sp.run_src, sp.run_dst, sp.run_len);
            run_phases<K, R>(sp, buf, base, t, active);
            if (active) {
                float2* __restrict__ gdst = state + base + toff;
                const bool soa = sp.nphases > 0;
#pragma unroll
                for (int m = 0; m < PPT; m++) {
                    const uint32_t piece = (tslot ^ sp.piece_slot[m]) >> 1;
                    float4 out;
                    if (soa) {
                        const ulonglong2 q = reinterpret_cast<const ulonglong2*>(buf)[piece];
                        vunpack(q.x, out.x, out.z);
                        vunpack(q.y, out.y, out.w);
                    } else {
                        out = buf[piece];
                    }
                    *reinterpret_cast<float4*>(gdst + sp.piece_off[m]) = out;
                }
            }
            __syncthreads();
        }
        // publish: every thread's stores, then one release of the tile count
        __threadfence();
        __syncthreads();
        if (t == 0) atomicAdd(b.done + it.circuit, it.count);
    }
}

template <int K, int R>
void launch_k(const OshmLaunch& p, cudaStream_t s) {
    constexpr int T = 1 << (K - R);
    const size_t smem = 2 * (sizeof(float2) << K);  // double-buffered tile
    static int blocks_per_sm = 0;
    if (!blocks_per_sm) {
        HQ_CHECK_CUDA(cudaFuncSetAttribute(k_oshm<K, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        HQ_CHECK_CUDA(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_oshm<K, R>, T, smem));
        HQ_REQUIRE(blocks_per_sm >= 1, HQ_ERR_UNSUPPORTED, "oshm<%d>: does not fit on an SM", K);
    }
    HQ_REQUIRE(p.ntiles >= 1, HQ_ERR_INVALID, "oshm: no tiles");
    const uint64_t slots = uint64_t(compute_sms()) * blocks_per_sm;
    const unsigned grid = (unsigned)(p.ntiles < slots ? p.ntiles : slots);
    k_oshm<K, R><<<grid, T, smem, s>>>(p);
    HQ_CHECK_CUDA(cudaGetLastError());
}

constexpr int kBatchR = 5;
constexpr size_t kBatchSmem = 2 * (sizeof(float2) << kBatchTile);

int batch_blocks_per_sm() {
    static int bps = 0;
    if (!bps) {
        auto kern = k_oshm_batch<kBatchTile, kBatchR>;
        HQ_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)kBatchSmem));
        HQ_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &bps, kern, 1 << (kBatchTile - kBatchR), kBatchSmem));
        HQ_REQUIRE(bps >= 1, HQ_ERR_UNSUPPORTED, "batched OShareMem kernel does not fit on an SM");
    }
    return bps;
}

}  // namespace

int oshm_batch_slots() { return ctx().sm_count * batch_blocks_per_sm(); }

void launch_oshm_batch(const BatchLaunch& b, int grid, bool cooperative, void* stream) {
    const int slots = oshm_batch_slots();
    HQ_REQUIRE(grid >= 1 && grid <= slots, HQ_ERR_INVALID,
               "batched launch: %d blocks, %d can be resident", grid, slots);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(1u << (kBatchTile - kBatchR));
    cfg.dynamicSmemBytes = kBatchSmem;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = cooperative ? 1 : 0;
    HQ_CHECK_CUDA(cudaLaunchKernelEx(&cfg, k_oshm_batch<kBatchTile, kBatchR>, b));
}

uint32_t oshm_swizzle(uint32_t x) { return swz(x); }

// register bits per tile width: 5 from 10 tile qubits up; at least 2 so that a
// phase always has a register qubit besides the f32x2 lane
int oshm_reg_bits(int k) { return k >= 10 ? 5 : (k >= 7 ? k - 5 : 2); }

int oshm_threads(int k, int r) { return 1 << (k - r); }

void launch_oshm(const OshmLaunch& p, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    switch (p.k) {
        case 6: launch_k<6, 2>(p, s); break;
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
