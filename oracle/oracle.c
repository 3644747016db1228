/* CPU oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h for who may call it).
 *
 * FP64 gate-by-gate restatement of the reference's gate semantics, and the same
 * code in complex64 as the timed CPU baseline.  Each block cites the reference
 * lines it follows.  SDG and TDG follow their factory matrices
 * (src/gate.cpp:212-246); the reference's plain path runs them through the S and
 * T kernels (src/kernelSimple.cu:413-424), a known quirk that is not reproduced.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum {
    T_CCX, T_CNOT, T_CY, T_CZ, T_CRX, T_CRY, T_CU1, T_CRZ, T_U1, T_U2, T_U3, T_H, T_X, T_Y,
    T_Z, T_S, T_SDG, T_T, T_TDG, T_RX, T_RY, T_RZ, T_TOTAL, T_ID, T_GII, T_GZZ, T_GOC, T_GCC
};

static void set(double* m, double r00, double i00, double r01, double i01, double r10, double i10,
                double r11, double i11) {
    m[0] = r00; m[1] = i00; m[2] = r01; m[3] = i01;
    m[4] = r10; m[5] = i10; m[6] = r11; m[7] = i11;
}

/* src/gate.cpp:9-342 -- factory matrices, evaluated in double */
int oracle_gate_matrix(int type, const double* p, double* m) {
    const double r2 = 1.0 / sqrt(2.0);
    switch (type) {
        case T_CCX: case T_CNOT: case T_X: set(m, 0, 0, 1, 0, 1, 0, 0, 0); return 0;
        case T_CY: case T_Y: set(m, 0, 0, 0, -1, 0, 1, 0, 0); return 0;
        case T_CZ: case T_Z: set(m, 1, 0, 0, 0, 0, 0, -1, 0); return 0;
        case T_CRX: case T_RX: {
            double c = cos(p[0] / 2.0), s = sin(p[0] / 2.0);
            set(m, c, 0, 0, -s, 0, -s, c, 0); return 0;
        }
        case T_CRY: case T_RY: {
            double c = cos(p[0] / 2.0), s = sin(p[0] / 2.0);
            set(m, c, 0, -s, 0, s, 0, c, 0); return 0;
        }
        case T_CU1: case T_U1: set(m, 1, 0, 0, 0, 0, 0, cos(p[0]), sin(p[0])); return 0;
        case T_CRZ: case T_RZ: {
            double c = cos(p[0] / 2.0), s = sin(p[0] / 2.0);
            set(m, c, -s, 0, 0, 0, 0, c, s); return 0;
        }
        case T_U2: { /* gate.cpp:124-136, params (phi, lambda) */
            double phi = p[0], lam = p[1];
            set(m, r2, 0, -cos(lam) * r2, -sin(lam) * r2, cos(phi) * r2, sin(phi) * r2,
                cos(lam + phi) * r2, sin(lam + phi) * r2);
            return 0;
        }
        case T_U3: { /* gate.cpp:138-150, params (theta, phi, lambda) */
            double th = p[0], phi = p[1], lam = p[2];
            double c = cos(th / 2), s = sin(th / 2);
            set(m, c, 0, -cos(lam) * s, -sin(lam) * s, cos(phi) * s, sin(phi) * s,
                cos(phi + lam) * c, sin(phi + lam) * c);
            return 0;
        }
        case T_H: set(m, r2, 0, r2, 0, r2, 0, -r2, 0); return 0;
        case T_S: set(m, 1, 0, 0, 0, 0, 0, 0, 1); return 0;
        case T_SDG: set(m, 1, 0, 0, 0, 0, 0, 0, -1); return 0;
        case T_T: set(m, 1, 0, 0, 0, 0, 0, r2, r2); return 0;
        case T_TDG: set(m, 1, 0, 0, 0, 0, 0, r2, -r2); return 0;
        case T_ID: set(m, 1, 0, 0, 0, 0, 0, 1, 0); return 0;
        default: return -1;
    }
}

/* Per-pair arithmetic of every gate type, src/kernelSimple.cu:75-332: L and H
 * are the (lo, hi) amplitudes of one pair.  Shared by the flat and the blocked
 * application below, so both run the same operations on every amplitude. */
#define DEFINE_PAIR(NAME, REAL)                                                               \
    static inline __attribute__((always_inline)) void NAME##_pair4(                           \
        int type, const REAL* m, REAL* Lr, REAL* Li, REAL* Hr, REAL* Hi) {                    \
        const REAL r2 = (REAL)0.70710678118654752440084436210485;                             \
        const REAL m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3];                        \
        const REAL m10r = m[4], m10i = m[5], m11r = m[6], m11i = m[7];                        \
        REAL lr = *Lr, li = *Li, hr = *Hr, hv = *Hi;                                          \
        switch (type) {                                                                       \
            case T_CCX: case T_CNOT: case T_X:                                                \
                *Lr = hr; *Li = hv; *Hr = lr; *Hi = li; break;                                \
            case T_CY: case T_Y:                                                              \
                *Lr = hv; *Li = -hr; *Hr = -li; *Hi = lr; break;                              \
            case T_CZ: case T_Z:                                                              \
                *Hr = -hr; *Hi = -hv; break;                                                  \
            case T_CRX: case T_RX: {                                                          \
                REAL al = m00r, be = -m01i;                                                   \
                *Lr = al * lr + be * hv; *Li = al * li - be * hr;                             \
                *Hr = al * hr + be * li; *Hi = al * hv - be * lr; break;                      \
            }                                                                                 \
            case T_CRY: case T_RY: {                                                          \
                REAL al = m00r, be = m10r;                                                    \
                *Lr = al * lr - be * hr; *Li = al * li - be * hv;                             \
                *Hr = be * lr + al * hr; *Hi = be * li + al * hv; break;                      \
            }                                                                                 \
            case T_CRZ: case T_RZ: {                                                          \
                REAL al = m00r, be = -m00i;                                                   \
                *Lr = al * lr + be * li; *Li = al * li - be * lr;                             \
                *Hr = al * hr - be * hv; *Hi = al * hv + be * hr; break;                      \
            }                                                                                 \
            case T_CU1: case T_U1:                                                            \
                *Hr = m11r * hr - m11i * hv; *Hi = m11r * hv + m11i * hr; break;              \
            case T_H:                                                                         \
                *Lr = r2 * (lr + hr); *Li = r2 * (li + hv);                                   \
                *Hr = r2 * (lr - hr); *Hi = r2 * (li - hv); break;                            \
            case T_S: *Hr = -hv; *Hi = hr; break;                                             \
            case T_SDG: *Hr = hv; *Hi = -hr; break;                                           \
            case T_T: *Hr = r2 * (hr - hv); *Hi = r2 * (hr + hv); break;                      \
            case T_TDG: *Hr = r2 * (hr + hv); *Hi = r2 * (hv - hr); break;                    \
            default: /* U2, U3 and anything given by its matrix */                            \
                *Lr = lr * m00r - li * m00i + hr * m01r - hv * m01i;                          \
                *Li = lr * m00i + li * m00r + hr * m01i + hv * m01r;                          \
                *Hr = lr * m10r - li * m10i + hr * m11r - hv * m11i;                          \
                *Hi = lr * m10i + li * m10r + hr * m11i + hv * m11r;                          \
                break;                                                                        \
        }                                                                                     \
    }

#define DEFINE_PAIR2(NAME, REAL)                                                              \
    static inline void NAME##_pair(int type, const REAL* m, REAL* L, REAL* H) {               \
        NAME##_pair4(type, m, L, L + 1, H, H + 1);                                            \
    }

/* Per-gate application over all 2^(n-1) (lo,hi) pairs, src/kernelSimple.cu:40-70
 * (SINGLE/CONTROL/CC_GATE_BEGIN): lo = the target bit inserted as 0, hi = lo with
 * it set, pairs whose control bits are not all set are skipped.  Generated for
 * double and float; `nt` OpenMP threads split the pairs. */
#define DEFINE_APPLY(NAME, REAL)                                                              \
    DEFINE_PAIR(NAME, REAL)                                                                   \
    DEFINE_PAIR2(NAME, REAL)                                                                  \
    static void NAME##_one(int n, REAL* a, const oracle_gate* g, int nt) {                   \
        const int64_t npair = (int64_t)1 << (n - 1);                                         \
        const int t = g->target;                                                              \
        const int64_t tmask = ((int64_t)1 << t) - 1;                                          \
        int64_t cmask = 0;                                                                    \
        if (g->control >= 0) cmask |= (int64_t)1 << g->control;                               \
        if (g->control2 >= 0) cmask |= (int64_t)1 << g->control2;                             \
        const int type = g->type;                                                             \
        REAL m[8];                                                                            \
        for (int k = 0; k < 8; k++) m[k] = (REAL)g->mat[k];                                   \
        int64_t i;                                                                            \
        if (nt <= 1) {                                                                        \
            for (i = 0; i < npair; i++) {                                                     \
                int64_t lo = ((i >> t) << (t + 1)) | (i & tmask);                             \
                if ((lo & cmask) != cmask) continue;                                          \
                NAME##_pair(type, m, a + 2 * lo, a + 2 * (lo | ((int64_t)1 << t)));           \
            }                                                                                 \
            return;                                                                           \
        }                                                                                     \
        _Pragma("omp parallel for schedule(static) num_threads(nt)")                          \
        for (i = 0; i < npair; i++) {                                                         \
            int64_t lo = ((i >> t) << (t + 1)) | (i & tmask);                                 \
            if ((lo & cmask) != cmask) continue;                                              \
            NAME##_pair(type, m, a + 2 * lo, a + 2 * (lo | ((int64_t)1 << t)));               \
        }                                                                                     \
    }                                                                                         \
    static int NAME##_check(int n, const oracle_gate* gates, int ngates) {                    \
        if (n < 1 || n > 40) return -1;                                                       \
        for (int k = 0; k < ngates; k++) {                                                    \
            const oracle_gate* g = &gates[k];                                                 \
            if (g->target < 0 || g->target >= n) return -1;                                   \
            if (g->control >= n || g->control2 >= n) return -1;                               \
            if (g->control == g->target || (g->control2 >= 0 && g->control2 == g->target))    \
                return -1;                                                                    \
        }                                                                                     \
        return 0;                                                                             \
    }                                                                                         \
    int NAME(int n, REAL* a, const oracle_gate* gates, int ngates, int nt) {                  \
        if (NAME##_check(n, gates, ngates) != 0) return -1;                                   \
        if (nt <= 0) nt = 1;                                                                  \
        for (int k = 0; k < ngates; k++) NAME##_one(n, a, &gates[k], nt);                     \
        return 0;                                                                             \
    }

DEFINE_APPLY(oracle_apply_f64, double)
DEFINE_APPLY(oracle_apply_f32, float)

static uint64_t gate_qubits(const oracle_gate* g) {
    uint64_t q = (uint64_t)1 << g->target;
    if (g->control >= 0) q |= (uint64_t)1 << g->control;
    if (g->control2 >= 0) q |= (uint64_t)1 << g->control2;
    return q;
}

static int popcount64(uint64_t x) {
    int c = 0;
    for (; x; x &= x - 1) c++;
    return c;
}

/* One gate on an m-qubit register held as split real / imaginary arrays:
 * the pairs of oracle_apply_f64_one in the same order, with the gate type
 * fixed per loop so the compiler can vectorise it (element-wise operations
 * only: the results do not change). */
#define LOCAL_LOOP(TY)                                                                        \
    if (cmask == 0) {                                                                         \
        for (int64_t b0 = 0; b0 < len; b0 += 2 * T)                                           \
            for (int64_t j = b0; j < b0 + T; j++)                                             \
                oracle_apply_f64_pair4(TY, mm, re + j, im + j, re + j + T, im + j + T);       \
    } else {                                                                                  \
        for (int64_t b0 = 0; b0 < len; b0 += 2 * T)                                           \
            for (int64_t j = b0; j < b0 + T; j++) {                                           \
                if ((j & cmask) != cmask) continue;                                           \
                oracle_apply_f64_pair4(TY, mm, re + j, im + j, re + j + T, im + j + T);       \
            }                                                                                 \
    }
#define LOCAL_CASE(TY) case TY: LOCAL_LOOP(TY) break;

static void local_apply_f64(int m, double* re, double* im, const oracle_gate* g) {
    const int64_t len = (int64_t)1 << m;
    const int64_t T = (int64_t)1 << g->target;
    int64_t cmask = 0;
    if (g->control >= 0) cmask |= (int64_t)1 << g->control;
    if (g->control2 >= 0) cmask |= (int64_t)1 << g->control2;
    double mm[8];
    for (int k = 0; k < 8; k++) mm[k] = g->mat[k];
    switch (g->type) {
        LOCAL_CASE(T_X) LOCAL_CASE(T_Y) LOCAL_CASE(T_Z) LOCAL_CASE(T_CNOT) LOCAL_CASE(T_CZ)
        LOCAL_CASE(T_CCX) LOCAL_CASE(T_CY) LOCAL_CASE(T_RX) LOCAL_CASE(T_CRX) LOCAL_CASE(T_RY)
        LOCAL_CASE(T_CRY) LOCAL_CASE(T_RZ) LOCAL_CASE(T_CRZ) LOCAL_CASE(T_U1) LOCAL_CASE(T_CU1)
        LOCAL_CASE(T_H) LOCAL_CASE(T_S) LOCAL_CASE(T_SDG) LOCAL_CASE(T_T) LOCAL_CASE(T_TDG)
        default: {
            const int ty = g->type;
            LOCAL_LOOP(ty)
        }
    }
}

/* One segment of the blocked application: every gate of `seg` acts on qubits
 * inside the set S (mask `smask`, m qubits).  For each of the 2^(n-m)
 * assignments of the other qubits, the 2^m amplitudes that differ only in S
 * are copied to a thread-local buffer, the gates run on it in order with
 * their qubits renamed to positions inside S, and the buffer is copied back.
 * Each amplitude sees exactly the operations of oracle_apply_f64, in the
 * same order: blocking only changes which amplitudes are in cache. */
static int run_segment_f64(int n, double* a, uint64_t smask, const oracle_gate* seg, int k,
                           int nt) {
    int pos[64], rest[64], m = 0, r = 0;
    for (int b = 0; b < n; b++) {
        if (smask >> b & 1) pos[m++] = b;
        else rest[r++] = b;
    }
    oracle_gate* local = (oracle_gate*)malloc(sizeof(oracle_gate) * (size_t)(k > 0 ? k : 1));
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) << m);
    if (!local || !off) { free(local); free(off); return -1; }
    for (int g = 0; g < k; g++) {
        local[g] = seg[g];
        int* fields[3] = {&local[g].target, &local[g].control, &local[g].control2};
        for (int f = 0; f < 3; f++) {
            if (*fields[f] < 0) continue;
            for (int j = 0; j < m; j++)
                if (pos[j] == *fields[f]) { *fields[f] = j; break; }
        }
    }
    for (int64_t j = 0; j < ((int64_t)1 << m); j++) {
        int64_t o = 0;
        for (int b = 0; b < m; b++)
            if (j >> b & 1) o |= (int64_t)1 << pos[b];
        off[j] = o;
    }
    const int64_t nblk = (int64_t)1 << (n - m);
    const int64_t len = (int64_t)1 << m;
    int rc = 0;
#pragma omp parallel num_threads(nt)
    {
        double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)len);  /* re | im */
        if (!buf) {
#pragma omp atomic write
            rc = -1;
        }
        int64_t blk;
#pragma omp for schedule(static)
        for (blk = 0; blk < nblk; blk++) {
            if (!buf) continue;
            int64_t base = 0;
            for (int b = 0; b < r; b++)
                if (blk >> b & 1) base |= (int64_t)1 << rest[b];
            double* re = buf;
            double* im = buf + len;
            for (int64_t j = 0; j < len; j++) {
                re[j] = a[2 * (base + off[j])];
                im[j] = a[2 * (base + off[j]) + 1];
            }
            for (int g = 0; g < k; g++) local_apply_f64(m, re, im, &local[g]);
            for (int64_t j = 0; j < len; j++) {
                a[2 * (base + off[j])] = re[j];
                a[2 * (base + off[j]) + 1] = im[j];
            }
        }
        free(buf);
    }
    free(local);
    free(off);
    return rc;
}

/* Same result as oracle_apply_f64, bit for bit, with the gates cut into
 * segments whose qubits fit in `width` qubits (padded with the lowest free
 * qubits so the copies run over contiguous memory). */
int oracle_apply_f64_blocked(int n, double* a, const oracle_gate* gates, int ngates, int nt,
                             int width) {
    if (oracle_apply_f64_check(n, gates, ngates) != 0) return -1;
    if (width < 1 || width > 20) return -1;
    if (nt <= 0) nt = 1;
    if (width > n) width = n;
    int start = 0;
    while (start < ngates) {
        uint64_t S = 0;
        int end = start;
        while (end < ngates) {
            const uint64_t q = gate_qubits(&gates[end]);
            if (popcount64(S | q) > width) break;
            S |= q;
            end++;
        }
        for (int b = 0; b < n && popcount64(S) < width; b++) S |= (uint64_t)1 << b;
        if (run_segment_f64(n, a, S, gates + start, end - start, nt) != 0) return -1;
        start = end;
    }
    return 0;
}

/* One pass over an FP64 reference and a complex64 result: out = {max |ref -
 * got|, Re <ref|got>, Im <ref|got>, <ref|ref>, <got|got>}, all in FP64. */
void oracle_compare_c64(int64_t count, const double* ref, const float* got, int nt, double* out) {
    double mx = 0, ore = 0, oim = 0, rr = 0, gg = 0;
    int64_t i;
    if (nt <= 0) nt = 1;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(max : mx) \
    reduction(+ : ore, oim, rr, gg)
    for (i = 0; i < count; i++) {
        const double ar = ref[2 * i], ai = ref[2 * i + 1];
        const double br = got[2 * i], bi = got[2 * i + 1];
        const double dr = ar - br, di = ai - bi;
        const double d = sqrt(dr * dr + di * di);
        if (d > mx) mx = d;
        ore += ar * br + ai * bi;
        oim += ar * bi - ai * br;
        rr += ar * ar + ai * ai;
        gg += br * br + bi * bi;
    }
    out[0] = mx; out[1] = ore; out[2] = oim; out[3] = rr; out[4] = gg;
}

/* src/kernelSimple.cu:9-37 -- memset 0, amp[0] = 1 */
void oracle_init_zero_f64(int n, double* a) {
    memset(a, 0, sizeof(double) * 2 * ((size_t)1 << n));
    a[0] = 1.0;
}
void oracle_init_zero_f32(int n, float* a) {
    memset(a, 0, sizeof(float) * 2 * ((size_t)1 << n));
    a[0] = 1.0f;
}

/* src/kernelSimple.cu:482-516 (measure + reduce): P(q = 0) = sum |a_lo|^2 */
double oracle_prob_zero_f32(int n, const float* a, int q, int nt) {
    const int64_t npair = (int64_t)1 << (n - 1);
    const int64_t qmask = ((int64_t)1 << q) - 1;
    double acc = 0;
    int64_t i;
    if (nt <= 0) nt = 1;
#pragma omp parallel for schedule(static) reduction(+ : acc) num_threads(nt)
    for (i = 0; i < npair; i++) {
        int64_t lo = ((i >> q) << (q + 1)) | (i & qmask);
        double r = a[2 * lo], im = a[2 * lo + 1];
        acc += r * r + im * im;
    }
    return acc;
}

/* src/schedule.cpp:578-702 -- U e_c for every column c, by applying the gates
 * to basis vectors of an m-qubit register (local bit j <-> qubits[j]). */
int oracle_group_unitary(int m, const int* qubits, const oracle_gate* gates, int ngates, double* U) {
    if (m < 1 || m > 12) return -1;
    const int64_t dim = (int64_t)1 << m;
    oracle_gate* local = (oracle_gate*)malloc(sizeof(oracle_gate) * (ngates > 0 ? ngates : 1));
    if (!local) return -1;
    for (int k = 0; k < ngates; k++) {
        local[k] = gates[k];
        int* fields[3] = {&local[k].target, &local[k].control, &local[k].control2};
        for (int f = 0; f < 3; f++) {
            int q = *fields[f];
            if (q < 0) continue;
            int j = -1;
            for (int x = 0; x < m; x++)
                if (qubits[x] == q) j = x;
            if (j < 0) { free(local); return -1; }
            *fields[f] = j;
        }
    }
    int rc = 0;
    for (int64_t c = 0; c < dim && rc == 0; c++) {
        double* col = U + 2 * c * dim;
        memset(col, 0, sizeof(double) * 2 * dim);
        col[2 * c] = 1.0;
        rc = oracle_apply_f64(m, col, local, ngates, 1);
    }
    free(local);
    return rc;
}
