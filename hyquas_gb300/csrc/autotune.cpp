// Autotuner: measures the cost model's constants on the GPU at hand.
//
// The reference calibrates its evaluator offline with a separate program that
// times gate kernels and writes per-GPU parameter files
// (evaluator-preprocess/process.cpp:24-176, read by src/evaluator.cpp:98-107).
// Here one call times single-group circuits on a scratch state with CUDA
// events, through the same compiled path a user's circuit takes, and fits:
//   pass_floor      one OShareMem group with a single Z gate
//   oshm_gate       arithmetic of a group of RX gates on its tile qubits
//   oshm_diag       added arithmetic of T gates interleaved with those RX gates
//   oshm_ctrl_diag  added arithmetic of CU1 gates interleaved with them
// (group time = amps * sqrt(pass_floor^2 + arithmetic^2), compiler.cpp)
//   mm_*            one 6-qubit TransMM group per precision
//   launch          a one-tile group (13 qubits)
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.h"
#include "compiler.h"
#include "executor.h"
#include "gates.h"

namespace hq {

namespace {

// median device seconds of one run of `gates` compiled with `opt` on s
double time_circuit(hq_state_s* s, const std::vector<hq_gate>& gates, const hq_compile_options& opt) {
    hq_circuit_s c;
    c.n = s->n;
    c.gates = gates;
    circuit_compile(&c, opt);
    std::vector<double> t;
    try {
        circuit_run(&c, s, true);  // warm-up
        for (int i = 0; i < 3; i++) t.push_back(circuit_run(&c, s, true) * 1e-6);
    } catch (...) {
        circuit_release(&c);
        throw;
    }
    circuit_release(&c);
    std::sort(t.begin(), t.end());
    return t[1];
}

hq_gate gate(int type, int target, int control = -1, double angle = 0.0) {
    return make_gate(type, target, control, -1, &angle);
}

}  // namespace

hq_cost_params autotune(int n) {
    if (n == 0) n = 26;
    HQ_REQUIRE(n >= 20 && n <= 32, HQ_ERR_INVALID, "autotune: %d qubits outside [20, 32]", n);
    ensure_init();
    hq_compile_options o{};
    o.backend = HQ_BACKEND_OSHM;
    o.specialize = 2;
    const double amps = double(uint64_t(1) << n);
    const int G = 96;
    hq_cost_params p = cost_params();

    hq_state_s* s = state_create(n);
    try {
        launch_init_zero(s->d, n, ctx().stream);
        // every gate on tile qubits 0..12 of a 13-qubit tile: one group
        const double floor = time_circuit(s, {gate(G_Z, 1)}, o);
        // diagonal gates are timed where circuits have them: between
        // non-diagonal gates on the same qubits
        std::vector<hq_gate> nd, dg, cd;
        for (int i = 0; i < G; i++) {
            const hq_gate rx = gate(G_RX, 1 + i % 12, -1, 0.1 + 0.01 * i);
            nd.push_back(rx);
            dg.push_back(rx);
            dg.push_back(gate(G_T, 1 + i % 12));
            cd.push_back(rx);
            cd.push_back(gate(G_CU1, 1 + (i + 1) % 12, 1 + i % 12, 0.2 + 0.01 * i));
        }
        const double t_nd = time_circuit(s, nd, o);
        const double t_dg = time_circuit(s, dg, o);
        const double t_cd = time_circuit(s, cd, o);
        // cost_oshm: t = amps * sqrt(floor^2 + work^2) per group
        auto work = [&](double t) { return std::sqrt(std::max(0.0, t * t - floor * floor)) / amps; };
        p.pass_floor = floor / amps;
        p.oshm_gate = work(t_nd) / (G * oshm_gate_units(nd[0]));  // per unit (RX: 2)
        p.oshm_diag = std::max(0.0, work(t_dg) - work(t_nd)) / G;
        p.oshm_ctrl_diag = std::max(0.0, work(t_cd) - work(t_nd)) / G;
        // TransMM: 6-qubit groups on qubits 0..5
        std::vector<hq_gate> mm;
        for (int i = 0; i < 24; i++) mm.push_back(gate(G_RY, i % 6, -1, 0.3 + 0.05 * i));
        for (int i = 0; i < 5; i++) mm.push_back(gate(G_CZ, i + 1, i));
        hq_compile_options om = o;
        om.backend = HQ_BACKEND_TRANSMM;
        om.mm_qubits = 6;
        om.mm_precision = HQ_MM_BF16X3;
        p.mm_bf16x3 = time_circuit(s, mm, om) / amps;
        om.mm_precision = HQ_MM_TF32;
        p.mm_tf32 = time_circuit(s, mm, om) / amps;
        om.mm_precision = HQ_MM_FP32;
        p.mm_fp32 = time_circuit(s, mm, om) / amps;
    } catch (...) {
        state_destroy(s);
        throw;
    }
    state_destroy(s);
    // launch cost: a one-tile group
    hq_state_s* s13 = state_create(13);
    try {
        launch_init_zero(s13->d, 13, ctx().stream);
        p.launch = time_circuit(s13, {gate(G_Z, 1)}, o);
    } catch (...) {
        state_destroy(s13);
        throw;
    }
    state_destroy(s13);
    set_cost_params(p);
    return p;
}

}  // namespace hq
