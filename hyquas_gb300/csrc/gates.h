// Gate model: type ordinals, factory matrices and the classification the
// compiler and the kernels need.  Follows src/gate.h:7-66 and src/gate.cpp:9-342.
#pragma once

#include <cstdint>
#include <vector>

#include "common.h"

namespace hq {

// Reference GateType ordinals (src/gate.h:7-9) plus the SWAP extension.
enum GateType : int32_t {
    G_CCX = 0, G_CNOT, G_CY, G_CZ, G_CRX, G_CRY, G_CU1, G_CRZ, G_U1, G_U2, G_U3, G_H, G_X, G_Y,
    G_Z, G_S, G_SDG, G_T, G_TDG, G_RX, G_RY, G_RZ, G_TOTAL, G_ID, G_GII, G_GZZ, G_GOC, G_GCC,
    G_SWAP = 28
};

// Build a gate from a factory (Gate::H, Gate::U3, ...).  Throws on bad input.
hq_gate make_gate(int32_t type, int32_t target, int32_t control, int32_t control2,
                  const double* params);

// Validate a caller-supplied gate against an n-qubit register.
void validate_gate(const hq_gate& g, int n);

// The reference's diagonal list (src/gate.h:26-28); used for grouping parity.
bool ref_is_diagonal(int32_t type);
// True when the gate's matrix is diagonal (any type).
bool matrix_is_diagonal(const hq_gate& g);
// Controlled X (X, CNOT, CCX): lo/hi exchange.
bool is_x_like(const hq_gate& g);
inline bool has_control(const hq_gate& g) { return g.control >= 0; }
inline uint64_t gate_qubits(const hq_gate& g) {
    uint64_t m = uint64_t(1) << g.target;
    if (g.control >= 0) m |= uint64_t(1) << g.control;
    if (g.control2 >= 0) m |= uint64_t(1) << g.control2;
    return m;
}
inline uint64_t gate_controls(const hq_gate& g) {
    uint64_t m = 0;
    if (g.control >= 0) m |= uint64_t(1) << g.control;
    if (g.control2 >= 0) m |= uint64_t(1) << g.control2;
    return m;
}

// Fold SWAP extensions into a relabelling (no data movement): returns the
// gates with every SWAP removed and later qubit references relabelled, and
// `perm`, where perm[s] = the qubit whose data the user's qubit s names once
// all swaps are applied (so the readout layout is pos[s] = layout[perm[s]]).
std::vector<hq_gate> fold_swaps(const std::vector<hq_gate>& gates, int n, std::vector<int>& perm);

// Runs of single-qubit gates on one qubit multiplied into one gate each (for
// the interpreted kernels, whose cost is per gate rather than per flop).
// origin (optional): for each output gate, the index of its first input gate.
std::vector<hq_gate> fuse_single_qubit_runs(const std::vector<hq_gate>& gates, int n,
                                            std::vector<int>* origin = nullptr);

// OpenQASM 2 text -> register size and gate list (qasm.cpp).
void parse_qasm(const char* text, int& n, std::vector<hq_gate>& out);

}  // namespace hq
