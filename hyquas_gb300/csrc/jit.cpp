// Specialised OShareMem kernels: one straight-line kernel per gate group.
//
// The interpreter kernel (k_oshm.cu) runs any group, but every op pays a
// dispatch and, because 64 live amplitude registers cross a dynamic op loop,
// register copies at each iteration.  For a compiled circuit the group is
// known in full, so this file writes the group as CUDA C++ -- tile bits,
// gathers, every op with its matrix as literals, register controls resolved
// per amplitude at generation time -- and compiles it with NVRTC for sm_103a
// (loaded through the runtime's library API).  The tile framework (persistent
// CTAs, cp.async staging, swizzled shared memory, f32x2 math) is the
// interpreter's; only the op stream becomes straight-line code, with the
// vectors' scales and signs tracked at generation time.
//
// NVRTC is opened at run time; when it is missing, compile falls back to the
// interpreter kernel (both are GPU paths).
#include "jit.h"

#include <dlfcn.h>

#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <thread>

#include "common.h"

namespace hq {

// ---- NVRTC entry points (dlopen) ----------------------------------------------
namespace {

typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;
struct Nvrtc {
    bool ok = false;
    std::string why;
    nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*,
                            const char* const*) = nullptr;
    nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*) = nullptr;
    nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t*) = nullptr;
    nvrtcResult_t (*log)(nvrtcProgram_t, char*) = nullptr;
    nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t*) = nullptr;
    nvrtcResult_t (*cubin)(nvrtcProgram_t, char*) = nullptr;
    nvrtcResult_t (*destroy)(nvrtcProgram_t*) = nullptr;
};

Nvrtc& nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* cands[] = {"libnvrtc.so.13", "libnvrtc.so",
                               "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/targets/sbsa-linux/lib/libnvrtc.so.13",
                               "/usr/local/cuda/targets/x86_64-linux/lib/libnvrtc.so.13"};
        void* h = nullptr;
        if (const char* home = getenv("CUDA_HOME")) {
            std::string p = std::string(home) + "/lib64/libnvrtc.so.13";
            h = dlopen(p.c_str(), RTLD_NOW | RTLD_LOCAL);
        }
        for (const char* c : cands) {
            if (h) break;
            h = dlopen(c, RTLD_NOW | RTLD_LOCAL);
        }
        if (!h) {
            n.why = "libnvrtc.so.13 not found";
            return;
        }
        n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
        n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
        n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
        n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
        n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
        n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
        n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
        n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
        if (!n.ok) n.why = "libnvrtc.so.13 lacks the expected symbols";
    });
    return n;
}

// ---- source generation -----------------------------------------------------------

const char* kPrelude = R"(
typedef unsigned long long v2;
typedef unsigned long long u64;
#define DI __device__ __forceinline__
DI v2 vadd(v2 a, v2 b) { v2 d; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
DI v2 vsub(v2 a, v2 b) { v2 d; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
DI v2 vmul(v2 a, v2 b) { v2 d; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
DI v2 vfma(v2 a, v2 b, v2 c) { v2 d; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c)); return d; }
DI v2 vpack(float lo, float hi) { v2 d; asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi)); return d; }
DI void vunpack(v2 a, float& lo, float& hi) { asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a)); }
DI v2 vdup(float x) { return vpack(x, x); }
DI v2 vswap(v2 a) { float l, h; vunpack(a, l, h); return vpack(h, l); }
DI v2 vlane(v2 nw, v2 old, bool k0, bool k1) { float a, b, c, d; vunpack(nw, a, b); vunpack(old, c, d); return vpack(k0 ? a : c, k1 ? b : d); }
DI float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
DI unsigned swz(unsigned x) { unsigned f = ((x >> 4) ^ (x >> 7) ^ (x >> 10) ^ (x >> 13)) & 7u; return x ^ (f << 1); }
DI void cpa16(unsigned s, const void* g) { asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(g) : "memory"); }
DI float F(unsigned b) { return __int_as_float((int)b); }
// a finished amplitude pair to the state and, when the run also leaves a copy
// of the final state in (device-mapped) host memory, to that copy; the
// kernel's stores are emitted twice, under one test of `copy`, so that the
// common form is plain stores
template <bool C> DI void st_amps(float2* state, float2* copy, u64 idx, float4 w) {
    *(float4*)(state + idx) = w;
    if (C) *(float4*)(copy + idx) = w;
}
// Bounded wait for phase `par` of the mbarrier at `addr`, decided by the whole
// group (barrier `gbar`, `cnt` threads): either every thread of the group saw
// the data land or none goes on.  After about two seconds the group records a
// timeout in err[0..2] (1, site 40, buffer), waits for its own copies in flight
// and returns false.
DI bool wait_full(unsigned addr, unsigned par, unsigned gbar, unsigned cnt, int* err, unsigned b) {
    unsigned ok = 0;
    const long long t0 = clock64();
    // each try suspends the thread for up to ~20 us unless the phase completes
    // first, so a waiting group issues few instructions
    for (unsigned it = 0; it < (1u << 20); it++) {
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok) : "r"(addr), "r"(par) : "memory");
        if (ok || clock64() - t0 > 4000000000ll) break;
    }
    unsigned all;
    asm volatile("{ .reg .pred p, q; setp.ne.u32 p, %1, 0; bar.red.and.pred q, %2, %3, p; selp.u32 %0, 1, 0, q; }"
                 : "=r"(all) : "r"(ok), "r"(gbar), "r"(cnt) : "memory");
    if (all) return true;
    if ((threadIdx.x % cnt) == 0 && atomicCAS(err, 0, 1) == 0) { err[1] = 40; err[2] = (int)b; }
    asm volatile("cp.async.wait_all;" ::: "memory");
    return false;
}
)";

std::string flit(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    char buf[32];
    snprintf(buf, sizeof(buf), "F(0x%08xu)", b);
    return buf;
}

std::string hex64(uint64_t x) {
    char buf[32];
    snprintf(buf, sizeof(buf), "0x%llxull", (unsigned long long)x);
    return buf;
}

uint32_t swz_host(uint32_t x) {
    const uint32_t f = ((x >> 4) ^ (x >> 7) ^ (x >> 10) ^ (x >> 13)) & 7u;
    return x ^ (f << 1);
}

struct Gen {
    std::ostringstream o;
    int nv = 16;
    int tmp = 0;
    std::string t(const char* p) { return std::string(p) + std::to_string(tmp++); }
    static std::string R(int j) { return "r" + std::to_string(j); }
    static std::string I(int j) { return "i" + std::to_string(j); }

    // lane-control mask for the vector pair starting at j: ok lanes
    static void lanes(uint32_t creg, int j, bool& k0, bool& k1) {
        k0 = ((uint32_t(2 * j)) & creg) == creg;
        k1 = ((uint32_t(2 * j + 1)) & creg) == creg;
    }

    void assign(const std::string& dst, const std::string& expr, const std::string& old, bool k0,
                bool k1) {
        if (k0 && k1)
            o << dst << " = " << expr << ";\n";
        else if (k0 || k1)
            o << dst << " = vlane(" << expr << ", " << old << ", " << (k0 ? "true" : "false") << ", "
              << (k1 ? "true" : "false") << ");\n";
    }

    // Per-lane signed scales within a phase: lane l of register vector j (and
    // of its imaginary partner), flat index 2 j + l, holds
    // sigma = (neg ? -1 : 1) sqrt(2)^e times its true amplitude.  Exact
    // 45-degree phases (T, T^dagger) then cost one add per component, the
    // scale growing by sqrt 2; a sign flip on a register qubit (Z, CZ) only
    // flips the sign; the adds of H, sqrt(X) and sqrt(Y) absorb a scale ratio
    // as one FMA (a packed constant when the two lanes' ratios differ); the
    // phase's closing multiply divides every lane by its scale.
    std::vector<int> se;
    std::vector<char> sn;
    void reset_scales() {
        se.assign(2 * nv, 0);
        sn.assign(2 * nv, 0);
    }
    double sigma(int x) const {
        double r = std::ldexp(1.0, se[x] >= 0 ? se[x] / 2 : -((-se[x]) / 2));
        if (se[x] & 1) r = se[x] > 0 ? r * std::sqrt(2.0) : r / std::sqrt(2.0);
        return (sn[x] ? -1.0 : 1.0) * r;
    }
    // sigma_a / sigma_b (flat indices), exact for even exponent differences
    double ratio(int a, int b) const {
        const int d = se[a] - se[b];
        double r = std::ldexp(1.0, d >= 0 ? d / 2 : -((-d) / 2));
        if (d & 1) r = d > 0 ? r * std::sqrt(2.0) : r / std::sqrt(2.0);
        return (sn[a] != sn[b] ? -1.0 : 1.0) * r;
    }
    // lane l of slot a over lane l of slot b
    double ra(int a, int b, int l) const { return ratio(2 * a + l, 2 * b + l); }
    static std::string vconst(double x) { return "vdup(" + flit((float)x) + ")"; }
    // k0 in the low lane, k1 in the high one
    static std::string kpair(double k0, double k1) {
        if ((float)k0 == (float)k1) return vconst(k0);
        return "vpack(" + flit((float)k0) + ", " + flit((float)k1) + ")";
    }
    // base + k * other as one instruction, k per lane
    static std::string comb(const std::string& base, double k0, double k1, const std::string& other) {
        if (k0 == 1.0 && k1 == 1.0) return "vadd(" + base + ", " + other + ")";
        if (k0 == -1.0 && k1 == -1.0) return "vsub(" + base + ", " + other + ")";
        return "vfma(" + kpair(k0, k1) + ", " + other + ", " + base + ")";
    }
    static std::string comb(const std::string& base, double k, const std::string& other) {
        return comb(base, k, k, other);
    }
    bool same(int a, int b) const { return se[a] == se[b] && sn[a] == sn[b]; }
    // v *= k for the lanes' factors k0, k1: sign flips only as bit XORs (ALU
    // pipe), anything else as one multiply per component
    void rescale(int j, double k0, double k1) {
        if (k0 == 1.0 && k1 == 1.0) return;
        if (std::fabs(k0) == 1.0 && std::fabs(k1) == 1.0) {
            const char* mask = k0 < 0 && k1 < 0 ? "0x8000000080000000ull"
                                                 : (k0 < 0 ? "0x80000000ull" : "0x8000000000000000ull");
            o << R(j) << " ^= " << mask << "; " << I(j) << " ^= " << mask << ";\n";
            return;
        }
        const std::string k = kpair(k0, k1);
        o << R(j) << " = vmul(" << k << ", " << R(j) << "); " << I(j) << " = vmul(" << k << ", " << I(j)
          << ");\n";
    }
    // give slot h the scales of slot j
    void align(int j, int h) {
        rescale(h, ra(j, h, 0), ra(j, h, 1));
        for (int l = 0; l < 2; l++) {
            se[2 * h + l] = se[2 * j + l];
            sn[2 * h + l] = sn[2 * j + l];
        }
    }
    // give lane 1 of slot j the scale of its lane 0
    void align_lanes(int j) {
        rescale(j, 1.0, ratio(2 * j, 2 * j + 1));
        se[2 * j + 1] = se[2 * j];
        sn[2 * j + 1] = sn[2 * j];
    }
    void flip(int j) {
        sn[2 * j] = !sn[2 * j];
        sn[2 * j + 1] = !sn[2 * j + 1];
    }

    // scaled forms: sqrt(X) / sqrt(Y) keep both scales, so they also run under a
    // run-time control; H and X change them, so only unconditionally
    static bool pair_fast(int kind, bool full, bool has_cout) {
        return (full && !has_cout && (kind == OP_H || kind == OP_X)) ||
               (full && (kind == OP_SY || kind == OP_SX));
    }
    static bool pair_needs_align(int kind, bool full, bool has_cout) {
        if (kind == OP_U || kind == OP_REAL || kind == OP_IMOFF || kind == OP_RROT) return true;
        if (kind == OP_H || kind == OP_SY || kind == OP_SX || kind == OP_X)
            return !pair_fast(kind, full, has_cout);
        return false;
    }

    bool uses_neg = false;  // phase has sign-only factors outside the register set
    void op(const OshmOp& op, bool& uses_acc) {
        const int kind = op.kind, J = op.tbit;
        const float* m = op.m;
        const bool has_cout = (op.flags & OPF_COUT) != 0;
        // slots an op combines at their plain values are given equal scales
        // first, outside any run-time control (the scales are compile-time facts)
        if (kind != OP_DOUT && J >= 1) {
            for (int j = 0; j < nv; j++) {
                if (j & (1 << (J - 1))) continue;
                bool k0, k1;
                lanes(op.creg, j, k0, k1);
                if ((k0 || k1) && pair_needs_align(kind, k0 && k1, has_cout)) align(j, j | (1 << (J - 1)));
            }
        }
        // an exchange of the lanes under a run-time control needs them at one scale
        if (kind == OP_X && J == 0 && has_cout)
            for (int j = 0; j < nv; j++)
                if ((uint32_t(2 * j) & op.creg) == op.creg) align_lanes(j);
        if (has_cout) o << "if ((pidx & " << hex64(op.cout) << ") == " << hex64(op.cout) << ") {\n";
        o << "{\n";
        if (kind == OP_DOUT) {
            const bool d0one = (op.flags & OPF_D0_ONE) != 0;
            const bool neg = d0one && m[6] == -1.f && m[7] == 0.f;
            o << "const bool hb = (pidx & " << hex64(op.tout) << ") != 0ull;\n";
            if (neg && op.creg != 0) {
                o << "if (hb) {\n";
                for (int j = 0; j < nv; j++) {
                    bool k0, k1;
                    lanes(op.creg, j, k0, k1);
                    if (!k0 && !k1) continue;
                    const char* mask = k0 && k1 ? "0x8000000080000000ull"
                                                : (k0 ? "0x80000000ull" : "0x8000000000000000ull");
                    o << R(j) << " ^= " << mask << "; " << I(j) << " ^= " << mask << ";\n";
                }
                o << "}\n}\n";
                if (has_cout) o << "}\n";
                return;
            }
            o << "const float2 f = hb ? make_float2(" << flit(m[6]) << ", " << flit(m[7])
              << ") : make_float2(" << flit(m[0]) << ", " << flit(m[1]) << ");\n";
            if (op.creg == 0 && neg) {
                uses_neg = true;
                o << "if (hb) negf = !negf;\n";
            } else if (op.creg == 0) {
                uses_acc = true;
                if (d0one)
                    o << "if (hb) acc = cmul(acc, f);\n";
                else
                    o << "acc = cmul(acc, f);\n";
            } else {
                o << "const v2 fr = vdup(f.x), fi = vdup(f.y), fin = vdup(-f.y);\n";
                for (int j = 0; j < nv; j++) {
                    bool k0, k1;
                    lanes(op.creg, j, k0, k1);
                    if (!k0 && !k1) continue;
                    o << "{ const v2 a = " << R(j) << ", b = " << I(j) << ";\n";
                    assign(R(j), "vfma(fin, b, vmul(fr, a))", R(j), k0, k1);
                    assign(I(j), "vfma(fi, a, vmul(fr, b))", I(j), k0, k1);
                    o << "}\n";
                }
            }
            o << "}\n";
            if (has_cout) o << "}\n";
            return;
        }
        if (J == 0) {
            // target = the vector lane
            const double h2 = std::sqrt(0.5);
            const bool lane_rot45 = kind == OP_DREG && !has_cout && m[0] == 1.f && m[1] == 0.f &&
                                    std::fabs(std::fabs(m[6]) - h2) < 1e-6 && std::fabs(std::fabs(m[7]) - h2) < 1e-6;
            if (kind == OP_X) {
                for (int j = 0; j < nv; j++) {
                    if ((uint32_t(2 * j) & op.creg) != op.creg) continue;
                    o << R(j) << " = vswap(" << R(j) << "); " << I(j) << " = vswap(" << I(j) << ");\n";
                    if (!has_cout) {  // the lanes' scales go with their values
                        std::swap(se[2 * j], se[2 * j + 1]);
                        std::swap(sn[2 * j], sn[2 * j + 1]);
                    }
                }
            } else if (kind == OP_NEGHI) {
                for (int j = 0; j < nv; j++) {
                    if ((uint32_t(2 * j) & op.creg) != op.creg) continue;
                    if (!has_cout)  // a sign: folded into the high lane's scale
                        sn[2 * j + 1] = !sn[2 * j + 1];
                    else
                        o << R(j) << " ^= 0x8000000000000000ull; " << I(j) << " ^= 0x8000000000000000ull;\n";
                }
            } else if (lane_rot45) {
                // T or T^dagger on the lane: the high lane's (x, y) -> (x + t y, y - t x), its
                // scale growing by sqrt 2 (negated when the real part of the phase is -1)
                const double c = m[6] > 0 ? 1.0 : -1.0, sgn = m[7] > 0 ? 1.0 : -1.0;
                const double t = c > 0 ? -sgn : sgn;
                o << "const v2 Kt = vpack(0.f, " << flit((float)t) << "), Ktn = vpack(0.f, " << flit((float)-t)
                  << ");\n";
                for (int j = 0; j < nv; j++) {
                    if ((uint32_t(2 * j) & op.creg) != op.creg) continue;
                    o << "{ const v2 a = " << R(j) << ", b = " << I(j) << "; " << R(j) << " = vfma(Kt, b, a); "
                      << I(j) << " = vfma(Ktn, a, b); }\n";
                    se[2 * j + 1] += 1;
                    if (c < 0) sn[2 * j + 1] = !sn[2 * j + 1];
                }
            } else if (kind == OP_DREG) {
                const float d0r = m[0], d0i = m[1], d1r = m[6], d1i = m[7];
                o << "const v2 Rr = vpack(" << flit(d0r) << ", " << flit(d1r) << "), Ii = vpack("
                  << flit(d0i) << ", " << flit(d1i) << "), In = vpack(" << flit(-d0i) << ", "
                  << flit(-d1i) << ");\n";
                for (int j = 0; j < nv; j++) {
                    if ((uint32_t(2 * j) & op.creg) != op.creg) continue;
                    o << "{ const v2 a = " << R(j) << ", b = " << I(j) << "; " << R(j)
                      << " = vfma(In, b, vmul(Rr, a)); " << I(j) << " = vfma(Ii, a, vmul(Rr, b)); }\n";
                }
            } else {
                // the other lane from a swapped copy, both lanes' coefficients in one
                // packed constant that also absorbs the ratio of the lanes' scales:
                // one or two instructions per component for the structured
                // matrices, four for a general one
                const bool gen = kind == OP_U || kind == OP_DREG || kind == OP_DROT || kind == OP_RROT;
                if (kind == OP_REAL || kind == OP_IMOFF || gen)
                    o << "const v2 P = vpack(" << flit(m[0]) << ", " << flit(m[6]) << ");\n";
                if (gen)
                    o << "const v2 Q = vpack(" << flit(m[1]) << ", " << flit(m[7]) << "), Qn = vpack("
                      << flit(-m[1]) << ", " << flit(-m[7]) << ");\n";
                for (int j = 0; j < nv; j++) {
                    if ((uint32_t(2 * j) & op.creg) != op.creg) continue;
                    const double r01 = ratio(2 * j, 2 * j + 1), r10 = ratio(2 * j + 1, 2 * j);
                    o << "{ const v2 a = " << R(j) << ", b = " << I(j) << ", as = vswap(a), bs = vswap(b); ";
                    if (kind == OP_REAL) {  // (a lo + b hi, c lo + d hi)
                        const std::string S = kpair(m[2] * r01, m[4] * r10);
                        o << R(j) << " = vfma(" << S << ", as, vmul(P, a)); " << I(j) << " = vfma(" << S
                          << ", bs, vmul(P, b));";
                    } else if (kind == OP_IMOFF) {  // (a lo + i b hi, i c lo + d hi)
                        o << R(j) << " = vfma(" << kpair(-m[3] * r01, -m[5] * r10) << ", bs, vmul(P, a)); "
                          << I(j) << " = vfma(" << kpair(m[3] * r01, m[5] * r10) << ", as, vmul(P, b));";
                    } else if (kind == OP_H && !has_cout) {  // (lo + hi, hi - lo): the high lane negated
                        const std::string K = kpair(r01, -r10);
                        o << R(j) << " = vfma(" << K << ", as, a); " << I(j) << " = vfma(" << K << ", bs, b);";
                        sn[2 * j + 1] = !sn[2 * j + 1];
                    } else if (kind == OP_H) {  // (lo + hi, lo - hi)
                        const std::string K = kpair(r01, r10), pm = kpair(1.0, -1.0);
                        o << R(j) << " = vfma(" << pm << ", a, vmul(" << K << ", as)); " << I(j) << " = vfma("
                          << pm << ", b, vmul(" << K << ", bs));";
                    } else if (kind == OP_SY) {  // (lo - hi, lo + hi)
                        const std::string K = kpair(-r01, r10);
                        o << R(j) << " = vfma(" << K << ", as, a); " << I(j) << " = vfma(" << K << ", bs, b);";
                    } else if (kind == OP_SX) {  // (lo - i hi, hi - i lo)
                        if (r01 == 1.0 && r10 == 1.0)
                            o << R(j) << " = vadd(a, bs); " << I(j) << " = vsub(b, as);";
                        else
                            o << R(j) << " = vfma(" << kpair(r01, r10) << ", bs, a); " << I(j) << " = vfma("
                              << kpair(-r01, -r10) << ", as, b);";
                    } else {  // general complex 2x2
                        const std::string S = kpair(m[2] * r01, m[4] * r10), T = kpair(m[3] * r01, m[5] * r10),
                                          Tn = kpair(-m[3] * r01, -m[5] * r10);
                        o << R(j) << " = vfma(" << Tn << ", bs, vfma(" << S << ", as, vfma(Qn, b, vmul(P, a)))); "
                          << I(j) << " = vfma(" << T << ", as, vfma(" << S << ", bs, vfma(Q, a, vmul(P, b))));";
                    }
                    o << " }\n";
                }
            }
            o << "}\n";
            if (has_cout) o << "}\n";
            return;
        }
        // target = register bit J >= 1: vector pairs (j, j | 1 << (J-1))
        auto consts = [&](const char* names[], const float* vals, int cnt) {
            for (int q = 0; q < cnt; q++)
                o << "const v2 " << names[q] << " = vdup(" << flit(vals[q]) << ");\n";
        };
        switch (kind) {
            case OP_U: {
                const char* nm[] = {"a", "ai", "ain", "b", "bi", "bin", "c", "ci", "cin", "d", "di", "din"};
                const float v[] = {m[0], m[1], -m[1], m[2], m[3], -m[3], m[4], m[5], -m[5], m[6], m[7], -m[7]};
                consts(nm, v, 12);
                break;
            }
            case OP_REAL: {
                const char* nm[] = {"a", "b", "c", "d"};
                const float v[] = {m[0], m[2], m[4], m[6]};
                consts(nm, v, 4);
                break;
            }
            case OP_IMOFF: {
                const char* nm[] = {"a", "b", "bn", "c", "cn", "d"};
                const float v[] = {m[0], m[3], -m[3], m[5], -m[5], m[6]};
                consts(nm, v, 6);
                break;
            }
            case OP_DREG: {
                const char* nm[] = {"er", "ei", "ein", "fr", "fi", "fin"};
                const float v[] = {m[6], m[7], -m[7], m[0], m[1], -m[1]};
                consts(nm, v, 6);
                break;
            }
            case OP_DROT:
            case OP_RROT: {
                const char* nm[] = {"sa", "sb"};
                const float v[] = {m[0], m[1]};
                consts(nm, v, 2);
                break;
            }
            case OP_NEGHI: break;
            default: break;
        }
        const bool d0one = (op.flags & OPF_D0_ONE) != 0;
        const bool negf_op = (op.flags & OPF_NEG) != 0;
        // in-place rotation of (x, y) by the three shears, then the optional negation
        auto shear = [&](const std::string& x, const std::string& y, const char* x0, const char* y0) {
            o << "{ v2 x = " << x0 << ", y = " << y0 << "; x = vfma(sa, y, x); y = vfma(sb, x, y); "
              << "x = vfma(sa, y, x); ";
            if (negf_op) o << "x ^= 0x8000000080000000ull; y ^= 0x8000000080000000ull; ";
            o << x << " = x; " << y << " = y; }\n";
        };
        // DROT by an odd multiple of pi/4 (T, T^dagger): d1 = m6 + i m7 with |m6| = |m7|
        const double h2 = std::sqrt(0.5);
        const bool rot45 = kind == OP_DROT && !has_cout && std::fabs(std::fabs(m[6]) - h2) < 1e-6 &&
                           std::fabs(std::fabs(m[7]) - h2) < 1e-6;
        for (int j = 0; j < nv; j++) {
            if (j & (1 << (J - 1))) continue;
            const int h = j | (1 << (J - 1));
            bool k0, k1;
            lanes(op.creg, j, k0, k1);
            if (!k0 && !k1) continue;
            const bool full = k0 && k1;
            const bool fast = pair_fast(kind, full, has_cout);
            if (kind == OP_NEGHI && !has_cout) {  // a sign: folded into the lanes' scales
                if (k0) sn[2 * h] = !sn[2 * h];
                if (k1) sn[2 * h + 1] = !sn[2 * h + 1];
                continue;
            }
            o << "{ const v2 lr = " << R(j) << ", li = " << I(j) << ", hr = " << R(h) << ", hi = " << I(h)
              << ";\n";
            if (fast && (kind == OP_H || kind == OP_SY || kind == OP_SX)) {
                const double rj0 = ra(j, h, 0), rj1 = ra(j, h, 1), rh0 = ra(h, j, 0), rh1 = ra(h, j, 1);
                if (kind == OP_H) {  // L' = L + H, H' = L - H (stored as H - L, scale negated)
                    o << R(j) << " = " << comb("lr", rj0, rj1, "hr") << "; " << I(j) << " = "
                      << comb("li", rj0, rj1, "hi") << "; " << R(h) << " = " << comb("hr", -rh0, -rh1, "lr") << "; "
                      << I(h) << " = " << comb("hi", -rh0, -rh1, "li") << ";\n";
                    flip(h);
                } else if (kind == OP_SY) {  // L' = L - H, H' = L + H
                    o << R(j) << " = " << comb("lr", -rj0, -rj1, "hr") << "; " << I(j) << " = "
                      << comb("li", -rj0, -rj1, "hi") << "; " << R(h) << " = " << comb("hr", rh0, rh1, "lr") << "; "
                      << I(h) << " = " << comb("hi", rh0, rh1, "li") << ";\n";
                } else {  // L' = L - i H, H' = H - i L
                    o << R(j) << " = " << comb("lr", rj0, rj1, "hi") << "; " << I(j) << " = "
                      << comb("li", -rj0, -rj1, "hr") << "; " << R(h) << " = " << comb("hr", rh0, rh1, "li") << "; "
                      << I(h) << " = " << comb("hi", -rh0, -rh1, "lr") << ";\n";
                }
                o << "}\n";
                continue;
            }
            if (fast && kind == OP_X) {
                o << R(j) << " = hr; " << I(j) << " = hi; " << R(h) << " = lr; " << I(h) << " = li;\n}\n";
                for (int l = 0; l < 2; l++) {
                    std::swap(se[2 * j + l], se[2 * h + l]);
                    std::swap(sn[2 * j + l], sn[2 * h + l]);
                }
                continue;
            }
            if (full && rot45) {
                // (x, y) -> (c x - s y, s x + c y) sqrt 2, c, s = +-1; c = -1 is stored negated
                const double c = m[6] > 0 ? 1.0 : -1.0, sgn = m[7] > 0 ? 1.0 : -1.0;
                if (c > 0)
                    o << R(h) << " = " << comb("hr", -sgn, "hi") << "; " << I(h) << " = " << comb("hi", sgn, "hr")
                      << ";\n}\n";
                else
                    o << R(h) << " = " << comb("hr", sgn, "hi") << "; " << I(h) << " = " << comb("hi", -sgn, "hr")
                      << ";\n}\n";
                se[2 * h] += 1;
                se[2 * h + 1] += 1;
                if (c < 0) flip(h);
                continue;
            }
            switch (kind) {
                case OP_U:
                    assign(R(j), "vfma(bin, hi, vfma(b, hr, vfma(ain, li, vmul(a, lr))))", "lr", k0, k1);
                    assign(I(j), "vfma(bi, hr, vfma(b, hi, vfma(ai, lr, vmul(a, li))))", "li", k0, k1);
                    assign(R(h), "vfma(din, hi, vfma(d, hr, vfma(cin, li, vmul(c, lr))))", "hr", k0, k1);
                    assign(I(h), "vfma(di, hr, vfma(d, hi, vfma(ci, lr, vmul(c, li))))", "hi", k0, k1);
                    break;
                case OP_REAL:
                    assign(R(j), "vfma(b, hr, vmul(a, lr))", "lr", k0, k1);
                    assign(I(j), "vfma(b, hi, vmul(a, li))", "li", k0, k1);
                    assign(R(h), "vfma(d, hr, vmul(c, lr))", "hr", k0, k1);
                    assign(I(h), "vfma(d, hi, vmul(c, li))", "hi", k0, k1);
                    break;
                case OP_IMOFF:
                    assign(R(j), "vfma(bn, hi, vmul(a, lr))", "lr", k0, k1);
                    assign(I(j), "vfma(b, hr, vmul(a, li))", "li", k0, k1);
                    assign(R(h), "vfma(cn, li, vmul(d, hr))", "hr", k0, k1);
                    assign(I(h), "vfma(c, lr, vmul(d, hi))", "hi", k0, k1);
                    break;
                case OP_H:
                    assign(R(j), "vadd(lr, hr)", "lr", k0, k1);
                    assign(I(j), "vadd(li, hi)", "li", k0, k1);
                    assign(R(h), "vsub(lr, hr)", "hr", k0, k1);
                    assign(I(h), "vsub(li, hi)", "hi", k0, k1);
                    break;
                case OP_SY:
                    assign(R(j), "vsub(lr, hr)", "lr", k0, k1);
                    assign(I(j), "vsub(li, hi)", "li", k0, k1);
                    assign(R(h), "vadd(lr, hr)", "hr", k0, k1);
                    assign(I(h), "vadd(li, hi)", "hi", k0, k1);
                    break;
                case OP_SX:
                    assign(R(j), "vadd(lr, hi)", "lr", k0, k1);
                    assign(I(j), "vsub(li, hr)", "li", k0, k1);
                    assign(R(h), "vadd(hr, li)", "hr", k0, k1);
                    assign(I(h), "vsub(hi, lr)", "hi", k0, k1);
                    break;
                case OP_X:
                    assign(R(j), "hr", "lr", k0, k1);
                    assign(I(j), "hi", "li", k0, k1);
                    assign(R(h), "lr", "hr", k0, k1);
                    assign(I(h), "li", "hi", k0, k1);
                    break;
                case OP_DREG:
                    assign(R(h), "vfma(ein, hi, vmul(er, hr))", "hr", k0, k1);
                    assign(I(h), "vfma(ei, hr, vmul(er, hi))", "hi", k0, k1);
                    if (!d0one) {
                        assign(R(j), "vfma(fin, li, vmul(fr, lr))", "lr", k0, k1);
                        assign(I(j), "vfma(fi, lr, vmul(fr, li))", "li", k0, k1);
                    }
                    break;
                case OP_DROT:
                    shear(R(h), I(h), "hr", "hi");
                    break;
                case OP_RROT: {
                    // (lo, hi) rotated in the real and in the imaginary plane;
                    // a negation (phi reduced by pi) flips both slots' signs,
                    // at run time only under a run-time control
                    const bool xneg = negf_op && has_cout;
                    for (int comp = 0; comp < 2; comp++) {
                        o << "{ v2 x = " << (comp ? "li" : "lr") << ", y = " << (comp ? "hi" : "hr")
                          << "; x = vfma(sa, y, x); y = vfma(sb, x, y); x = vfma(sa, y, x); ";
                        if (xneg) o << "x ^= 0x8000000080000000ull; y ^= 0x8000000080000000ull; ";
                        o << (comp ? I(j) : R(j)) << " = x; " << (comp ? I(h) : R(h)) << " = y; }\n";
                    }
                    if (negf_op && !has_cout) {
                        flip(j);
                        flip(h);
                    }
                    break;
                }
                case OP_NEGHI: {
                    // sign flips as bit XORs: they run on the ALU pipe, not the FMA pipe
                    const char* mask = k0 && k1 ? "0x8000000080000000ull"
                                                : (k0 ? "0x80000000ull" : "0x8000000000000000ull");
                    o << R(h) << " = hr ^ " << mask << "; " << I(h) << " = hi ^ " << mask << ";\n";
                    break;
                }
                default: break;
            }
            o << "}\n";
        }
        o << "}\n";
        if (has_cout) o << "}\n";
    }
};

std::string deposit_expr(const char* var, uint32_t nbits, const uint8_t* dst, bool is64) {
    std::ostringstream e;
    e << "(";
    bool first = true;
    for (uint32_t j = 0; j < nbits; j++) {
        if (!first) e << " | ";
        first = false;
        if (is64)
            e << "((u64)((" << var << " >> " << j << ") & 1u) << " << int(dst[j]) << ")";
        else
            e << "((((unsigned)" << var << " >> " << j << ") & 1u) << " << int(dst[j]) << ")";
    }
    if (first) e << "0";
    e << ")";
    return e.str();
}

// Three shapes of the same kernel.
//   RING: one CTA per SM with two groups of T threads, each group working on
//     its own tile (16 warps per SM, registers capped at 128), and three tile
//     buffers in a ring: tile i of the CTA uses buffer i mod 3 and is computed
//     by group i mod 2; when a group is done reading tile i's buffer it issues
//     the cp.async loads of tile i + 3 into it (for the other group).  Their
//     completion is tracked by cp.async.mbarrier.arrive on mbarrier
//     (i + 3) mod 6, one per (buffer, consuming group): each mbarrier's
//     phases are then consumed by one group, in order, so the parity a group
//     waits for is never that of an older phase still pending.  A group never
//     waits for a load issued less than a tile's compute earlier, so HBM
//     traffic overlaps the arithmetic.
//   PAIRED: two CTAs per SM, one tile buffer each; a CTA loads, computes and
//     stores in turn (the other CTA computing meanwhile).
//   SINGLE: one CTA per SM that double-buffers its tiles; used when the
//     128-register builds would spill.
enum class Shape { RING, PAIRED, SINGLE };

std::string generate(const OshmProgram& prog, int& threads, size_t& smem, Shape shape) {
    const bool paired = shape == Shape::PAIRED;
    const bool ring = shape == Shape::RING;
    const int K = prog.k, R = prog.r, NV = 1 << (R - 1);
    const int T = 1 << (K - R);
    const int PPT = (1 << (K - 1)) / T;
    const size_t tile_bytes = sizeof(float) * 2 << K;
    threads = ring ? 2 * T : T;
    smem = ring ? 3 * tile_bytes + 64 : (paired ? 1 : 2) * tile_bytes;
    // a group-wide barrier: the whole CTA, or in RING the group's named barrier
    const std::string SYNC = ring ? "asm volatile(\"bar.sync %0, " + std::to_string(T) +
                                        ";\" :: \"r\"(gbar) : \"memory\");\n"
                                  : std::string("__syncthreads();\n");
    const int n = prog.n;
    uint8_t tile_phys[OSHM_MAX_K];
    for (int b = 0, j = 0; b < n; b++)
        if ((prog.tile_mask >> b) & 1) tile_phys[j++] = (uint8_t)b;

    Gen g;
    g.nv = NV;
    std::ostringstream& o = g.o;
    o << kPrelude;
    // PAIRED and RING keep 128 registers per thread: RING with narrower tiles
    // (fewer threads per CTA) asks for as many CTAs per SM as fill 64K registers
    const int ring_min_blocks = std::max(1, 65536 / (threads * 128));
    o << "extern \"C\" __global__ void __launch_bounds__(" << threads
      << (paired ? ", 2" : ring ? ", " + std::to_string(ring_min_blocks) : std::string(""))
      << ") hq_oshm_group(float2* __restrict__ state, u64 ntiles, int* __restrict__ err, "
         "float2* __restrict__ copy) {\n";
    if (ring)
        o << "extern __shared__ float4 smem4[];\nconst unsigned grp = threadIdx.x / " << T
          << "u, t = threadIdx.x % " << T << "u, gbar = 1u + grp;\n";
    else
        o << "extern __shared__ float4 smem4[];\nconst unsigned t = threadIdx.x;\n(void)err;\n";
    // physical offset of local index 2t and its slot
    {
        uint8_t dst[OSHM_MAX_K];
        for (int j = 0; j < K - R; j++) dst[j] = tile_phys[j + 1];
        o << "const u64 toff = " << deposit_expr("t", K - R, dst, true) << ";\n";
        o << "const unsigned tslot = swz(t << 1);\n";
    }
    o << "unsigned sbase; asm(\"{ .reg .u64 p; cvta.to.shared.u64 p, %1; cvt.u32.u64 %0, p; }\" : "
         "\"=r\"(sbase) : \"l\"(smem4));\n";
    if (ring) {
        // six mbarriers after the buffers, T arrivals each (one per loading thread)
        o << "const unsigned mbar = sbase + " << 3 * tile_bytes << "u;\n"
          << "if (threadIdx.x == 0) for (unsigned b = 0; b < 6; b++) asm volatile("
             "\"mbarrier.init.shared::cta.b64 [%0], %1;\" :: \"r\"(mbar + 8u * b), \"n\"("
          << T << ") : \"memory\");\n__syncthreads();\n";
    }
    // tile base: constant runs of block bits
    o << "auto tile_base = [&](u64 u) -> u64 { return 0ull";
    {
        int src = 0;
        for (int b = 0; b < n;) {
            if ((prog.tile_mask >> b) & 1) {
                b++;
                continue;
            }
            int len = 0;
            while (b + len < n && !((prog.tile_mask >> (b + len)) & 1)) len++;
            o << " | (((u >> " << src << ") & " << hex64((uint64_t(1) << len) - 1) << ") << " << b << ")";
            src += len;
            b += len;
        }
    }
    o << "; };\n";
    // piece offsets/slots per m
    std::vector<uint64_t> poff(PPT);
    std::vector<uint32_t> pslot(PPT);
    for (int m = 0; m < PPT; m++) {
        const uint32_t local = uint32_t(2 * m * T);
        uint64_t off = 0;
        for (int j = 0; j < K; j++)
            if ((local >> j) & 1) off |= uint64_t(1) << tile_phys[j];
        poff[m] = off;
        pslot[m] = swz_host(local);
    }
    o << (ring ? "auto load_tile = [&](u64 u, int b, u64 i) {\n" : "auto load_tile = [&](u64 u, int b) {\n")
      << "const float2* gsrc = state + tile_base(u) + toff;\n"
      << "const unsigned bb = sbase + (unsigned)b * " << ((1u << (K - 1)) * 16u) << "u;\n";
    for (int m = 0; m < PPT; m++)
        o << "cpa16(bb + ((tslot ^ " << pslot[m] << "u) << 3), gsrc + " << hex64(poff[m]) << ");\n";
    if (ring)  // this thread's copies arrive on the tile's mbarrier (tile index mod 6) when they land
        o << "asm volatile(\"cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\" :: \"r\"(mbar + 8u * "
             "(unsigned)(i % 6)) : \"memory\");\n};\n";
    else
        o << "asm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n};\n";
    // the last phase stores its amplitudes straight from registers to HBM, so
    // the tile buffer is free once that phase has gathered them: a paired CTA
    // then starts loading its next tile under the last phase's arithmetic
    // Only when the last phase's first thread bit is physical qubit 1: then the
    // 16-byte stores of neighbouring threads fill whole 32-byte sectors
    // (otherwise the staged write-back through shared memory coalesces better).
    const bool direct = !prog.phases.empty() && prog.phases.back().g_phys[0] == 1;
    if (ring) {
        // tile i of this CTA is tile blockIdx.x + i * gridDim.x: group 0 takes the
        // even i, group 1 the odd; the first three tiles are loaded up front
        o << "auto tile_of = [&](u64 i) -> u64 { return (u64)blockIdx.x + i * (u64)gridDim.x; };\n"
             "if (grp == 0) { if (tile_of(0) < ntiles) load_tile(tile_of(0), 0, 0); "
             "if (tile_of(2) < ntiles) load_tile(tile_of(2), 2, 2); }\n"
             "else if (tile_of(1) < ntiles) load_tile(tile_of(1), 1, 1);\n"
             "for (u64 i = grp; tile_of(i) < ntiles; i += 2) {\n"
             "const u64 u = tile_of(i);\n"
             "const unsigned bi = (unsigned)(i % 3);\n"
             "if (!wait_full(mbar + 8u * (unsigned)(i % 6), (unsigned)((i / 6) & 1), gbar, "
          << T << "u, err, bi)) return;\n"
          << "float4* buf = smem4 + bi * " << (1 << (K - 1)) << "u;\n";
    } else if (paired && direct) {
        o << "u64 u = blockIdx.x;\nif (u < ntiles) load_tile(u, 0);\n";
        o << "for (int it = 0; u < ntiles; it++, u += gridDim.x) {\n"
             "asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n"
             "__syncthreads();\n"
             "float4* buf = smem4;\n";
    } else if (paired) {
        o << "u64 u = blockIdx.x;\n";
        o << "for (int it = 0; u < ntiles; it++, u += gridDim.x) {\n"
             "load_tile(u, 0); asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n"
             "__syncthreads();\n"
             "float4* buf = smem4;\n";
    } else {
        o << "u64 u = blockIdx.x;\nif (u < ntiles) load_tile(u, 0);\n";
        o << "for (int it = 0; u < ntiles; it++, u += gridDim.x) {\n"
             "const u64 un = u + gridDim.x;\n"
             "if (un < ntiles) { load_tile(un, (it + 1) & 1); asm volatile(\"cp.async.wait_group 1;\\n\" ::: "
             "\"memory\"); }\n"
             "else { asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\"); }\n"
             "__syncthreads();\n"
          << "float4* buf = smem4 + (it & 1) * " << (1 << (K - 1)) << ";\n";
    }
    o << "const u64 base = tile_base(u);\n";
    o << "v2 ";
    for (int j = 0; j < NV; j++) o << (j ? ", " : "") << "r" << j << ", i" << j;
    o << ";\n";
    for (size_t p = 0; p < prog.phases.size(); p++) {
        const OshmPhase& P = prog.phases[p];
        const bool lastp = direct && p + 1 == prog.phases.size();
        // the phase's thread constants, from an opaque copy of the thread index
        // so that they are made here and not kept live across the whole kernel
        o << "{ // phase " << p << "\n";
        o << "unsigned tp; asm volatile(\"mov.u32 %0, %1;\" : \"=r\"(tp) : \"r\"(t));\n";
        o << "const unsigned sb" << p << " = swz(" << deposit_expr("tp", K - R, P.g_local, false) << ");\n";
        o << "const u64 gp" << p << " = " << deposit_expr("tp", K - R, P.g_phys, true) << ";\n";
        o << "const u64 pidx = base | gp" << p << ";\n(void)pidx;\n";
        uint32_t col[OSHM_MAX_R];
        for (int j = 1; j < R; j++) col[j] = swz_host(1u << P.r_local[j]);
        for (int j = 0; j < NV; j++) {
            uint32_t c = 0;
            for (int b = 1; b < R; b++)
                if ((j >> (b - 1)) & 1) c ^= col[b];
            if (p == 0)
                o << "{ const float4 q = buf[(sb" << p << " ^ " << c << "u) >> 1]; r" << j
                  << " = vpack(q.x, q.z); i" << j << " = vpack(q.y, q.w); }\n";
            else
                o << "{ const ulonglong2 q = ((const ulonglong2*)buf)[(sb" << p << " ^ " << c
                  << "u) >> 1]; r" << j << " = q.x; i" << j << " = q.y; }\n";
        }
        if (lastp) {
            o << SYNC;  // every amplitude is in registers: the buffer is free
            if (paired) o << "if (u + gridDim.x < ntiles) load_tile(u + gridDim.x, 0);\n";
            if (ring) o << "if (tile_of(i + 3) < ntiles) load_tile(tile_of(i + 3), bi, i + 3);\n";
        }
        o << "float2 acc = make_float2(1.f, 0.f);\n(void)acc;\nbool negf = false;\n(void)negf;\n";
        bool uses_acc = false;
        g.uses_neg = false;
        g.reset_scales();
        // A phase whose closing multiply would be the per-thread factor alone
        // (every lane's scale 1 at its end) applies that factor first: the ops
        // that make it (diagonals on thread bits, no register control) commute
        // with the phase's other ops.  The same arithmetic, but NVRTC has
        // scheduled the factor-only block at the phase end far worse (a
        // 30-qubit group: 5.2 against 3.1 ms).
        auto is_factor = [](const OshmOp& op) { return op.kind == OP_DOUT && op.creg == 0; };
        bool early = false;
        bool has_factor = false;
        for (uint32_t oi = P.op_begin; oi < P.op_end; oi++) has_factor = has_factor || is_factor(prog.ops[oi]);
        if (has_factor) {
            Gen d;
            d.nv = g.nv;
            d.reset_scales();
            bool ua = false;
            for (uint32_t oi = P.op_begin; oi < P.op_end; oi++) d.op(prog.ops[oi], ua);
            bool ones = true;
            for (int x = 0; x < 2 * NV; x++) ones = ones && (float)(double(P.scale) / d.sigma(x)) == 1.f;
            early = ua && ones;
        }
        if (early) {
            for (uint32_t oi = P.op_begin; oi < P.op_end; oi++)
                if (is_factor(prog.ops[oi])) g.op(prog.ops[oi], uses_acc);
            if (g.uses_neg) o << "if (negf) { acc.x = -acc.x; acc.y = -acc.y; }\n";
            o << "{ const float2 f = acc;\nconst v2 fr = vdup(f.x), fi = vdup(f.y), fin = vdup(-f.y);\n";
            for (int j = 0; j < NV; j++)
                o << "{ const v2 a = r" << j << ", b = i" << j << "; r" << j << " = vfma(fin, b, vmul(fr, a)); i"
                  << j << " = vfma(fi, a, vmul(fr, b)); }\n";
            o << "}\n";
            for (uint32_t oi = P.op_begin; oi < P.op_end; oi++)
                if (!is_factor(prog.ops[oi])) g.op(prog.ops[oi], uses_acc);
            uses_acc = false;  // applied; every lane's scale ends at 1
            g.uses_neg = false;
        } else {
            for (uint32_t oi = P.op_begin; oi < P.op_end; oi++) g.op(prog.ops[oi], uses_acc);
        }
        // closing multiply: the phase's deferred scale and the per-thread factor,
        // each lane divided by its own scale
        std::vector<float> kf(2 * NV);
        bool any_k = false;
        for (int x = 0; x < 2 * NV; x++) {
            kf[x] = (float)(double(P.scale) / g.sigma(x));
            any_k = any_k || kf[x] != 1.f;
        }
        // the packed factor of vector j, each lane's constant times `mul` (a run-time
        // float expression) or plain
        auto kvec = [&](int j, const std::string& mul) {
            const float k0 = kf[2 * j], k1 = kf[2 * j + 1];
            const std::string s0 = mul.empty() ? flit(k0) : mul + " * " + flit(k0);
            if (k0 == k1) return "vdup(" + s0 + ")";
            return "vpack(" + s0 + ", " + (mul.empty() ? flit(k1) : mul + " * " + flit(k1)) + ")";
        };
        const bool neg_in_mul = g.uses_neg && !uses_acc && any_k;  // the sign rides on the multiply
        if (g.uses_neg && uses_acc) {
            o << "if (negf) { acc.x = -acc.x; acc.y = -acc.y; }\n";
        } else if (g.uses_neg && !neg_in_mul) {
            // a sign: flip the sign bits (ALU pipe) of every amplitude
            o << "if (negf) {\n";
            for (int j = 0; j < NV; j++)
                o << "r" << j << " ^= 0x8000000080000000ull; i" << j << " ^= 0x8000000080000000ull;\n";
            o << "}\n";
        }
        if (uses_acc) {
            // the vectors sharing a factor together, each factor in a scope of its
            // own: few factors are live at once (with many, NVRTC's schedule of
            // the block has measured 1.6x slower)
            o << "{ const float2 f = acc;\n";
            std::map<std::pair<float, float>, std::vector<int>> by_factor;
            std::vector<std::pair<float, float>> order;
            for (int j = 0; j < NV; j++) {
                const std::pair<float, float> key(kf[2 * j], kf[2 * j + 1]);
                if (!by_factor.count(key)) order.push_back(key);
                by_factor[key].push_back(j);
            }
            for (const auto& key : order) {
                const std::vector<int>& js = by_factor[key];
                o << "{ const v2 fr = " << kvec(js[0], "f.x") << ", fi = " << kvec(js[0], "f.y")
                  << ", fin = " << kvec(js[0], "-f.y") << ";\n";
                for (int j : js)
                    o << "{ const v2 a = r" << j << ", b = i" << j << "; r" << j
                      << " = vfma(fin, b, vmul(fr, a)); i" << j << " = vfma(fi, a, vmul(fr, b)); }\n";
                o << "}\n";
            }
            o << "}\n";
        } else if (neg_in_mul) {
            o << "{ const float ns = negf ? -1.f : 1.f;\n";
            for (int j = 0; j < NV; j++)
                o << "{ const v2 k = " << kvec(j, "ns") << "; r" << j << " = vmul(k, r" << j << "); i" << j
                  << " = vmul(k, i" << j << "); }\n";
            o << "}\n";
        } else if (any_k) {
            for (int j = 0; j < NV; j++) g.rescale(j, kf[2 * j], kf[2 * j + 1]);
        }
        if (lastp) {
            // vector j holds the amplitudes at pidx | (its register bits) and + 1
            for (int form = 0; form < 2; form++) {
                o << (form == 0 ? "if (copy == nullptr) {\n" : "} else {\n");
                for (int j = 0; j < NV; j++) {
                    uint64_t off = 0;
                    for (int b = 1; b < R; b++)
                        if ((j >> (b - 1)) & 1) off |= uint64_t(1) << tile_phys[P.r_local[b]];
                    o << "{ float4 w; vunpack(r" << j << ", w.x, w.z); vunpack(i" << j << ", w.y, w.w); st_amps<"
                      << (form ? "true" : "false") << ">(state, copy, pidx | " << hex64(off) << ", w); }\n";
                }
            }
            o << "}\n}\n";
            continue;
        }
        for (int j = 0; j < NV; j++) {
            uint32_t c = 0;
            for (int b = 1; b < R; b++)
                if ((j >> (b - 1)) & 1) c ^= col[b];
            o << "((ulonglong2*)buf)[(sb" << p << " ^ " << c << "u) >> 1] = make_ulonglong2(r" << j
              << ", i" << j << ");\n";
        }
        // the next phase keeps the warp bits (thread bits 5..): each warp
        // reads back only what it wrote, so a warp sync orders the exchange
        bool warp_local = p + 1 < prog.phases.size() && K - R > 5;
        for (int j = 5; warp_local && j < K - R; j++)
            warp_local = P.g_local[j] == prog.phases[p + 1].g_local[j];
        o << (warp_local ? std::string("__syncwarp();\n") : SYNC) << "}\n";
    }
    if (!direct) {
        // staged write-back; pieces are (re0, re1, im0, im1) after a phase and
        // as loaded when there is none
        o << "const u64 gdst = base + toff;\n";
        for (int form = 0; form < 2; form++) {
            const char* tf = form ? "true" : "false";
            o << (form == 0 ? "if (copy == nullptr) {\n" : "} else {\n");
            for (int m = 0; m < PPT; m++) {
                if (prog.phases.empty())
                    o << "st_amps<" << tf << ">(state, copy, gdst + " << hex64(poff[m]) << ", buf[(tslot ^ "
                      << pslot[m] << "u) >> 1]);\n";
                else
                    o << "{ const ulonglong2 q = ((const ulonglong2*)buf)[(tslot ^ " << pslot[m]
                      << "u) >> 1]; float4 w; vunpack(q.x, w.x, w.z); vunpack(q.y, w.y, w.w); st_amps<" << tf
                      << ">(state, copy, gdst + " << hex64(poff[m]) << ", w); }\n";
            }
        }
        o << "}\n";
        o << SYNC;
        if (ring) o << "if (tile_of(i + 3) < ntiles) load_tile(tile_of(i + 3), bi, i + 3);\n";
    }
    o << "}\n";
    // a thread leaves with none of its copies in flight
    if (ring) o << "asm volatile(\"cp.async.wait_all;\" ::: \"memory\");\n";
    o << "}\n";
    return o.str();
}

// One generated source: compiled once per process.  An entry is pending while
// its first requester compiles it; later requesters of the same source wait
// for it rather than compiling it again.
struct CacheEntry {
    JitKernel k;
    bool ok = false;
    bool pending = true;
    std::string err;
    std::mutex m;
    std::condition_variable cv;
};

std::mutex g_cache_mu;
std::map<std::string, std::shared_ptr<CacheEntry>> g_cache;

JitKernel compile_source(const std::string& src, int threads, size_t smem) {
    Nvrtc& nv = nvrtc();
    HQ_REQUIRE(nv.ok, HQ_ERR_UNSUPPORTED, "NVRTC unavailable: %s", nv.why.c_str());
    nvrtcProgram_t prog = nullptr;
    HQ_REQUIRE(nv.create(&prog, src.c_str(), "hq_oshm_group.cu", 0, nullptr, nullptr) == 0,
               HQ_ERR_UNSUPPORTED, "nvrtcCreateProgram failed");
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17"};
    const int rc = nv.compile(prog, 2, opts);
    if (rc != 0) {
        size_t ls = 0;
        nv.log_size(prog, &ls);
        std::string log(ls, '\0');
        nv.log(prog, &log[0]);
        nv.destroy(&prog);
        fail(HQ_ERR_UNSUPPORTED, "NVRTC compile failed (%d): %.800s", rc, log.c_str());
    }
    size_t cs = 0;
    nv.cubin_size(prog, &cs);
    std::vector<char> cubin(cs);
    nv.cubin(prog, cubin.data());
    nv.destroy(&prog);
    JitKernel k;
    HQ_CHECK_CUDA(cudaLibraryLoadData(&k.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    HQ_CHECK_CUDA(cudaLibraryGetKernel(&k.kern, k.lib, "hq_oshm_group"));
    k.threads = threads;
    k.smem = smem;
    HQ_CHECK_CUDA(cudaFuncSetAttribute((const void*)k.kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    cudaFuncAttributes fa;
    HQ_CHECK_CUDA(cudaFuncGetAttributes(&fa, (const void*)k.kern));
    k.local_bytes = fa.localSizeBytes;
    int bps = 0;
    HQ_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)k.kern, threads, smem));
    HQ_REQUIRE(bps >= 1, HQ_ERR_UNSUPPORTED, "specialised kernel does not fit on an SM");
    k.blocks_per_sm = bps;
    return k;
}

}  // namespace

bool jit_available() { return nvrtc().ok; }

// The first shape tried: RING unless HQ_OSHM_SHAPE names another ("paired",
// "single"), a tuning knob for comparing the shapes on a given GPU.
Shape first_shape() {
    const char* e = getenv("HQ_OSHM_SHAPE");
    if (e && !strcmp(e, "paired")) return Shape::PAIRED;
    if (e && !strcmp(e, "single")) return Shape::SINGLE;
    return Shape::RING;
}

// Generated sources by program (its bytes; phases and ops are zero-filled
// before they are set, so equal programs have equal bytes) and shape: a
// circuit compiled again skips the generator.
struct GenEntry {
    std::string src;
    int threads = 0;
    size_t smem = 0;
};
std::mutex g_gen_mu;
std::map<std::string, GenEntry> g_gen;

std::string generate_cached(const OshmProgram& p, int& threads, size_t& smem, Shape shape) {
    std::string key;
    const int32_t hdr[4] = {p.n, p.k, p.r, (int32_t)shape};
    key.append((const char*)hdr, sizeof(hdr));
    key.append((const char*)&p.tile_mask, sizeof(p.tile_mask));
    key.append((const char*)p.phases.data(), p.phases.size() * sizeof(OshmPhase));
    key.append((const char*)p.ops.data(), p.ops.size() * sizeof(OshmOp));
    {
        std::lock_guard<std::mutex> lk(g_gen_mu);
        auto it = g_gen.find(key);
        if (it != g_gen.end()) {
            threads = it->second.threads;
            smem = it->second.smem;
            return it->second.src;
        }
    }
    GenEntry e;
    e.src = generate(p, e.threads, e.smem, shape);
    threads = e.threads;
    smem = e.smem;
    std::lock_guard<std::mutex> lk(g_gen_mu);
    return g_gen.emplace(std::move(key), std::move(e)).first->second.src;
}

std::vector<JitKernel> jit_compile_groups(const std::vector<const OshmProgram*>& progs) {
    ensure_init();
    const Shape shape0 = first_shape();
    std::vector<std::string> srcs(progs.size());
    std::vector<int> threads(progs.size());
    std::vector<size_t> smem(progs.size());
    for (size_t i = 0; i < progs.size(); i++)
        srcs[i] = generate_cached(*progs[i], threads[i], smem[i], shape0);
    std::vector<std::shared_ptr<CacheEntry>> ents(progs.size());
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        for (size_t i = 0; i < progs.size(); i++) {
            auto it = g_cache.find(srcs[i]);
            if (it != g_cache.end()) {
                ents[i] = it->second;
            } else {
                ents[i] = std::make_shared<CacheEntry>();
                g_cache[srcs[i]] = ents[i];
                todo.push_back(i);
            }
        }
    }
    // NVRTC compiles in parallel; loading (cudaLibraryLoadData) needs the device
    // current in each worker thread
    const int dev = ctx().device;
    std::vector<std::thread> pool;
    std::mutex next_mu;
    size_t next = 0;
    const size_t nthreads = std::min<size_t>(todo.size(), std::max(1u, std::thread::hardware_concurrency()));
    for (size_t w = 0; w < nthreads; w++) {
        pool.emplace_back([&] {
            cudaSetDevice(dev);
            while (true) {
                size_t k;
                {
                    std::lock_guard<std::mutex> lk(next_mu);
                    if (next >= todo.size()) return;
                    k = todo[next++];
                }
                try {
                    JitKernel jk = compile_source(srcs[k], threads[k], smem[k]);
                    // a spill of up to 128 bytes per thread costs less than the 16
                    // warps per SM gain (measured on the 30-qubit grid); beyond that,
                    // one double-buffered CTA of 8 warps per SM
                    // PAIRED needs two CTAs per SM; RING one (narrower RING tiles ask
                    // for more through __launch_bounds__, but one still works)
                    const int need = shape0 == Shape::PAIRED ? 2 : 1;
                    if (shape0 != Shape::SINGLE && (jk.local_bytes > 128 || jk.blocks_per_sm < need)) {
                        cudaLibraryUnload(jk.lib);
                        int t2 = 0;
                        size_t s2 = 0;
                        const std::string src2 = generate(*progs[k], t2, s2, Shape::SINGLE);
                        jk = compile_source(src2, t2, s2);
                    }
                    std::lock_guard<std::mutex> lk(ents[k]->m);
                    ents[k]->k = jk;
                    ents[k]->ok = true;
                } catch (const Failure& f) {
                    std::lock_guard<std::mutex> lk(ents[k]->m);
                    ents[k]->err = f.what();
                }
                {
                    std::lock_guard<std::mutex> lk(ents[k]->m);
                    ents[k]->pending = false;
                }
                ents[k]->cv.notify_all();
            }
        });
    }
    for (auto& th : pool) th.join();
    std::vector<JitKernel> out;
    for (size_t i = 0; i < progs.size(); i++) {
        bool ok;
        std::string err;
        {
            // an entry another caller is compiling: wait for it
            std::unique_lock<std::mutex> lk(ents[i]->m);
            ents[i]->cv.wait(lk, [&] { return !ents[i]->pending; });
            ok = ents[i]->ok;
            err = ents[i]->err;
        }
        if (!ok) {
            {
                std::lock_guard<std::mutex> lk(g_cache_mu);
                auto it = g_cache.find(srcs[i]);
                if (it != g_cache.end() && it->second == ents[i]) g_cache.erase(it);
            }
            fail(HQ_ERR_UNSUPPORTED, "%s", err.empty() ? "specialisation failed" : err.c_str());
        }
        out.push_back(ents[i]->k);
    }
    return out;
}

bool jit_lookup_cached(const std::vector<const OshmProgram*>& progs, std::vector<JitKernel>& out) {
    const Shape shape0 = first_shape();
    std::vector<JitKernel> ks;
    for (const OshmProgram* pr : progs) {
        int t = 0;
        size_t sm = 0;
        const std::string src = generate_cached(*pr, t, sm, shape0);
        std::shared_ptr<CacheEntry> e;
        {
            std::lock_guard<std::mutex> lk(g_cache_mu);
            auto it = g_cache.find(src);
            if (it == g_cache.end()) return false;
            e = it->second;
        }
        std::lock_guard<std::mutex> lk(e->m);
        if (e->pending || !e->ok) return false;
        ks.push_back(e->k);
    }
    out.swap(ks);
    return true;
}

void jit_launch(const JitKernel& k, void* state, uint64_t ntiles, int* err, cudaStream_t st,
                void* copy) {
    const uint64_t slots = uint64_t(compute_sms()) * k.blocks_per_sm;
    const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
    void* args[] = {&state, &ntiles, &err, &copy};
    HQ_CHECK_CUDA(cudaLaunchKernel((const void*)k.kern, dim3(grid), dim3(k.threads), args, k.smem, st));
}

std::string jit_source(const OshmProgram& prog) {
    int t;
    size_t s;
    return generate(prog, t, s, first_shape());
}

}  // namespace hq
