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

/* Per-gate application over all 2^(n-1) (lo,hi) pairs, src/kernelSimple.cu:40-70
 * (SINGLE/CONTROL/CC_GATE_BEGIN) with the per-type arithmetic of
 * src/kernelSimple.cu:75-332.  Generated for double and float. */
#define DEFINE_APPLY(NAME, REAL)                                                              \
    static void NAME##_one(int n, REAL* a, const oracle_gate* g, int nt) {                   \
        const int64_t npair = (int64_t)1 << (n - 1);                                         \
        const int t = g->target;                                                              \
        const int64_t tmask = ((int64_t)1 << t) - 1;                                          \
        int64_t cmask = 0;                                                                    \
        if (g->control >= 0) cmask |= (int64_t)1 << g->control;                               \
        if (g->control2 >= 0) cmask |= (int64_t)1 << g->control2;                             \
        const int type = g->type;                                                             \
        const REAL m00r = (REAL)g->mat[0], m00i = (REAL)g->mat[1];                             \
        const REAL m01r = (REAL)g->mat[2], m01i = (REAL)g->mat[3];                             \
        const REAL m10r = (REAL)g->mat[4], m10i = (REAL)g->mat[5];                             \
        const REAL m11r = (REAL)g->mat[6], m11i = (REAL)g->mat[7];                             \
        const REAL r2 = (REAL)0.70710678118654752440084436210485;                             \
        int64_t i;                                                                            \
        _Pragma("omp parallel for schedule(static) num_threads(nt)")                          \
        for (i = 0; i < npair; i++) {                                                         \
            int64_t lo = ((i >> t) << (t + 1)) | (i & tmask);                                 \
            if ((lo & cmask) != cmask) continue;                                              \
            int64_t hi = lo | ((int64_t)1 << t);                                              \
            REAL* L = a + 2 * lo;                                                             \
            REAL* H = a + 2 * hi;                                                             \
            REAL lr = L[0], li = L[1], hr = H[0], hv = H[1];                                  \
            switch (type) {                                                                   \
                case T_CCX: case T_CNOT: case T_X:                                            \
                    L[0] = hr; L[1] = hv; H[0] = lr; H[1] = li; break;                        \
                case T_CY: case T_Y:                                                          \
                    L[0] = hv; L[1] = -hr; H[0] = -li; H[1] = lr; break;                      \
                case T_CZ: case T_Z:                                                          \
                    H[0] = -hr; H[1] = -hv; break;                                            \
                case T_CRX: case T_RX: {                                                      \
                    REAL al = m00r, be = -m01i;                                               \
                    L[0] = al * lr + be * hv; L[1] = al * li - be * hr;                       \
                    H[0] = al * hr + be * li; H[1] = al * hv - be * lr; break;                \
                }                                                                             \
                case T_CRY: case T_RY: {                                                      \
                    REAL al = m00r, be = m10r;                                                \
                    L[0] = al * lr - be * hr; L[1] = al * li - be * hv;                       \
                    H[0] = be * lr + al * hr; H[1] = be * li + al * hv; break;                \
                }                                                                             \
                case T_CRZ: case T_RZ: {                                                      \
                    REAL al = m00r, be = -m00i;                                               \
                    L[0] = al * lr + be * li; L[1] = al * li - be * lr;                       \
                    H[0] = al * hr - be * hv; H[1] = al * hv + be * hr; break;                \
                }                                                                             \
                case T_CU1: case T_U1:                                                        \
                    H[0] = m11r * hr - m11i * hv; H[1] = m11r * hv + m11i * hr; break;        \
                case T_H:                                                                     \
                    L[0] = r2 * (lr + hr); L[1] = r2 * (li + hv);                             \
                    H[0] = r2 * (lr - hr); H[1] = r2 * (li - hv); break;                      \
                case T_S: H[0] = -hv; H[1] = hr; break;                                       \
                case T_SDG: H[0] = hv; H[1] = -hr; break;                                     \
                case T_T: H[0] = r2 * (hr - hv); H[1] = r2 * (hr + hv); break;                \
                case T_TDG: H[0] = r2 * (hr + hv); H[1] = r2 * (hv - hr); break;              \
                default: /* U2, U3 and anything given by its matrix */                        \
                    L[0] = lr * m00r - li * m00i + hr * m01r - hv * m01i;                     \
                    L[1] = lr * m00i + li * m00r + hr * m01i + hv * m01r;                     \
                    H[0] = lr * m10r - li * m10i + hr * m11r - hv * m11i;                     \
                    H[1] = lr * m10i + li * m10r + hr * m11i + hv * m11r;                     \
                    break;                                                                    \
            }                                                                                 \
        }                                                                                     \
    }                                                                                         \
    int NAME(int n, REAL* a, const oracle_gate* gates, int ngates, int nt) {                  \
        if (n < 1 || n > 40) return -1;                                                       \
        if (nt <= 0) nt = 1;                                                                  \
        for (int k = 0; k < ngates; k++) {                                                    \
            const oracle_gate* g = &gates[k];                                                 \
            if (g->target < 0 || g->target >= n) return -1;                                   \
            if (g->control >= n || g->control2 >= n) return -1;                               \
            if (g->control == g->target || (g->control2 >= 0 && g->control2 == g->target))    \
                return -1;                                                                    \
            NAME##_one(n, a, g, nt);                                                          \
        }                                                                                     \
        return 0;                                                                             \
    }

DEFINE_APPLY(oracle_apply_f64, double)
DEFINE_APPLY(oracle_apply_f32, float)

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
