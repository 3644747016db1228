/* CPU oracle for the state-vector path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
 * the --impl reference arm) load this library, and only as the checker or the
 * CPU baseline; the product library never links or calls it.
 *
 * What it restates from the reference (thu-pacman/HyQuas):
 *   - gate matrices of every factory, src/gate.cpp:9-342 (computed in double);
 *   - gate-by-gate application, src/kernelSimple.cu:40-70 (index macros:
 *     lo = target bit inserted as 0, hi = lo | 1<<t, control predicate
 *     (lo>>c)&1) and the per-type arithmetic of src/kernelSimple.cu:75-332;
 *   - |0..0> initialisation, src/kernelSimple.cu:9-37;
 *   - the qubit-probability reduction P(q=0), src/kernelSimple.cu:482-516;
 *   - fused gate-group unitary, src/schedule.cpp:578-702 (column c = U e_c).
 * Parity pin: tests/golden/ holds outputs of the reference's own CPU code
 * (gate factories, GateGroup::initCPUMatrix) built by oracle/Makefile `ref`;
 * tests/test_oracle.py checks this restatement against them.
 */
#ifndef HQ_ORACLE_H
#define HQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same record as hq_gate in include/hyquas_gb300.h. */
typedef struct {
    int32_t type;      /* reference GateType ordinal (src/gate.h:7-9) */
    int32_t target;
    int32_t control;   /* -1 when absent */
    int32_t control2;  /* -1 when absent */
    double mat[8];     /* row-major 2x2: re00 im00 re01 im01 re10 im10 re11 im11 */
} oracle_gate;

/* Matrix of gate `type` with angles params[0..2]; returns 0 or -1 (unknown type). */
int oracle_gate_matrix(int type, const double* params, double mat[8]);

/* Apply gates in order to an interleaved complex state of 2^n amplitudes. */
int oracle_apply_f64(int n, double* state, const oracle_gate* gates, int ngates, int nthreads);
int oracle_apply_f32(int n, float* state, const oracle_gate* gates, int ngates, int nthreads);

/* Same result as oracle_apply_f64, bit for bit: consecutive gates whose
 * qubits fit in `width` (1..20) qubits run on cache-sized blocks of the state. */
int oracle_apply_f64_blocked(int n, double* state, const oracle_gate* gates, int ngates,
                             int nthreads, int width);

/* out = {max |ref - got|, Re <ref|got>, Im <ref|got>, <ref|ref>, <got|got>}
 * over `count` amplitudes of an FP64 reference and a complex64 result. */
void oracle_compare_c64(int64_t count, const double* ref, const float* got, int nthreads,
                        double* out);

/* |0..0> */
void oracle_init_zero_f64(int n, double* state);
void oracle_init_zero_f32(int n, float* state);

/* sum over amplitudes with bit q clear of |a|^2 (FP64 accumulation) */
double oracle_prob_zero_f32(int n, const float* state, int q, int nthreads);

/* Fused unitary of `ngates` gates whose qubits are all in qubits[0..m-1]:
 * local bit j <-> qubits[j].  U is written column-major (U[c*2^m + r] = <r|U|c>),
 * i.e. the layout the reference hands to cuBLAS as matrix A. */
int oracle_group_unitary(int m, const int* qubits, const oracle_gate* gates, int ngates, double* U);

#ifdef __cplusplus
}
#endif
#endif
