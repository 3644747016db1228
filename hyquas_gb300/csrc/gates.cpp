#include "gates.h"

#include <cmath>
#include <cstring>

namespace hq {

static void set(hq_gate& g, double r00, double i00, double r01, double i01, double r10, double i10,
                double r11, double i11) {
    double m[8] = {r00, i00, r01, i01, r10, i10, r11, i11};
    std::memcpy(g.mat, m, sizeof(m));
}

// Factory matrices, src/gate.cpp:9-342, evaluated in double.
hq_gate make_gate(int32_t type, int32_t target, int32_t control, int32_t control2,
                  const double* params) {
    hq_gate g;
    g.type = type;
    g.target = target;
    g.control = control;
    g.control2 = control2;
    const double zero[3] = {0, 0, 0};
    const double* p = params ? params : zero;
    const double r2 = 1.0 / std::sqrt(2.0);
    bool needs_c = false, needs_c2 = false;
    switch (type) {
        case G_CCX: needs_c = needs_c2 = true; set(g, 0, 0, 1, 0, 1, 0, 0, 0); break;
        case G_CNOT: needs_c = true; set(g, 0, 0, 1, 0, 1, 0, 0, 0); break;
        case G_CY: needs_c = true; set(g, 0, 0, 0, -1, 0, 1, 0, 0); break;
        case G_CZ: needs_c = true; set(g, 1, 0, 0, 0, 0, 0, -1, 0); break;
        case G_CRX: case G_RX: {
            needs_c = type == G_CRX;
            double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
            set(g, c, 0, 0, -s, 0, -s, c, 0);
            break;
        }
        case G_CRY: case G_RY: {
            needs_c = type == G_CRY;
            double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
            set(g, c, 0, -s, 0, s, 0, c, 0);
            break;
        }
        case G_CU1: case G_U1:
            needs_c = type == G_CU1;
            set(g, 1, 0, 0, 0, 0, 0, std::cos(p[0]), std::sin(p[0]));
            break;
        case G_CRZ: case G_RZ: {
            needs_c = type == G_CRZ;
            double c = std::cos(p[0] / 2.0), s = std::sin(p[0] / 2.0);
            set(g, c, -s, 0, 0, 0, 0, c, s);
            break;
        }
        case G_U2: {  // (phi, lambda), gate.cpp:124-136
            double phi = p[0], lam = p[1];
            set(g, r2, 0, -std::cos(lam) * r2, -std::sin(lam) * r2, std::cos(phi) * r2,
                std::sin(phi) * r2, std::cos(lam + phi) * r2, std::sin(lam + phi) * r2);
            break;
        }
        case G_U3: {  // (theta, phi, lambda), gate.cpp:138-150
            double th = p[0], phi = p[1], lam = p[2];
            double c = std::cos(th / 2), s = std::sin(th / 2);
            set(g, c, 0, -std::cos(lam) * s, -std::sin(lam) * s, std::cos(phi) * s,
                std::sin(phi) * s, std::cos(phi + lam) * c, std::sin(phi + lam) * c);
            break;
        }
        case G_H: set(g, r2, 0, r2, 0, r2, 0, -r2, 0); break;
        case G_X: set(g, 0, 0, 1, 0, 1, 0, 0, 0); break;
        case G_Y: set(g, 0, 0, 0, -1, 0, 1, 0, 0); break;
        case G_Z: set(g, 1, 0, 0, 0, 0, 0, -1, 0); break;
        case G_S: set(g, 1, 0, 0, 0, 0, 0, 0, 1); break;
        case G_SDG: set(g, 1, 0, 0, 0, 0, 0, 0, -1); break;
        case G_T: set(g, 1, 0, 0, 0, 0, 0, r2, r2); break;
        case G_TDG: set(g, 1, 0, 0, 0, 0, 0, r2, -r2); break;
        case G_ID: set(g, 1, 0, 0, 0, 0, 0, 1, 0); break;
        case G_SWAP: needs_c = true; set(g, 1, 0, 0, 0, 0, 0, 1, 0); break;
        default: fail(HQ_ERR_INVALID, "unknown gate type %d", type);
    }
    if (!needs_c) g.control = -1;
    if (!needs_c2) g.control2 = -1;
    HQ_REQUIRE(target >= 0, HQ_ERR_INVALID, "gate type %d: negative target", type);
    HQ_REQUIRE(!needs_c || control >= 0, HQ_ERR_INVALID, "gate type %d needs a control", type);
    HQ_REQUIRE(!needs_c2 || control2 >= 0, HQ_ERR_INVALID, "gate type %d needs two controls", type);
    return g;
}

void validate_gate(const hq_gate& g, int n) {
    HQ_REQUIRE(g.target >= 0 && g.target < n, HQ_ERR_INVALID, "gate target %d out of range [0,%d)",
               g.target, n);
    HQ_REQUIRE(g.control >= -1 && g.control < n, HQ_ERR_INVALID, "gate control %d out of range",
               g.control);
    HQ_REQUIRE(g.control2 >= -1 && g.control2 < n, HQ_ERR_INVALID, "gate control2 %d out of range",
               g.control2);
    HQ_REQUIRE(g.control != g.target && (g.control2 < 0 || g.control2 != g.target) &&
                   (g.control2 < 0 || g.control2 != g.control),
               HQ_ERR_INVALID, "gate qubits must be distinct (t=%d c=%d c2=%d)", g.target, g.control,
               g.control2);
    HQ_REQUIRE(g.control2 < 0 || g.control >= 0, HQ_ERR_INVALID, "control2 without control");
    HQ_REQUIRE(g.type >= 0 && g.type <= G_SWAP && g.type != G_TOTAL, HQ_ERR_INVALID,
               "unknown gate type %d", g.type);
    for (double v : g.mat)
        HQ_REQUIRE(std::isfinite(v), HQ_ERR_INVALID, "non-finite gate matrix entry");
}

bool ref_is_diagonal(int32_t t) {
    return t == G_CZ || t == G_CU1 || t == G_CRZ || t == G_U1 || t == G_Z || t == G_S ||
           t == G_SDG || t == G_T || t == G_TDG || t == G_RZ;
}

bool matrix_is_diagonal(const hq_gate& g) {
    if (g.type == G_SWAP) return false;
    return g.mat[2] == 0 && g.mat[3] == 0 && g.mat[4] == 0 && g.mat[5] == 0;
}

bool is_x_like(const hq_gate& g) {
    return g.mat[0] == 0 && g.mat[1] == 0 && g.mat[2] == 1 && g.mat[3] == 0 && g.mat[4] == 1 &&
           g.mat[5] == 0 && g.mat[6] == 0 && g.mat[7] == 0;
}

std::vector<hq_gate> fold_swaps(const std::vector<hq_gate>& gates, int n, std::vector<int>& perm) {
    // content[s] = the qubit whose data sits in user slot s once the swaps so
    // far are folded; a gate on user qubit u then acts on qubit content[u].
    std::vector<int> content(n);
    for (int q = 0; q < n; q++) content[q] = q;
    std::vector<hq_gate> out;
    out.reserve(gates.size());
    for (const hq_gate& g0 : gates) {
        if (g0.type == G_SWAP) {
            std::swap(content[g0.target], content[g0.control]);
            continue;
        }
        hq_gate g = g0;
        g.target = content[g0.target];
        if (g0.control >= 0) g.control = content[g0.control];
        if (g0.control2 >= 0) g.control2 = content[g0.control2];
        out.push_back(g);
    }
    perm = content;
    return out;
}

// Consecutive single-qubit gates on one qubit (no gate touching that qubit in
// between) multiplied into one 2x2 gate, kept where the first of them stood.
std::vector<hq_gate> fuse_single_qubit_runs(const std::vector<hq_gate>& gates, int n,
                                            std::vector<int>* origin) {
    std::vector<hq_gate> out;
    if (origin) origin->clear();
    std::vector<int> open(n, -1);  // qubit -> index in `out` of a 1q gate still open for fusion
    for (const hq_gate& g : gates) {
        const bool one = g.control < 0 && g.control2 < 0 && g.type != G_SWAP;
        if (one && open[g.target] >= 0) {
            hq_gate& f = out[open[g.target]];
            // f <- g . f (g acts after f)
            double m[8];
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 2; c++) {
                    double re = 0, im = 0;
                    for (int k = 0; k < 2; k++) {
                        const double ar = g.mat[(r * 2 + k) * 2], ai = g.mat[(r * 2 + k) * 2 + 1];
                        const double br = f.mat[(k * 2 + c) * 2], bi = f.mat[(k * 2 + c) * 2 + 1];
                        re += ar * br - ai * bi;
                        im += ar * bi + ai * br;
                    }
                    m[(r * 2 + c) * 2] = re;
                    m[(r * 2 + c) * 2 + 1] = im;
                }
            for (int q = 0; q < 8; q++) f.mat[q] = m[q];
            f.type = G_U3;  // a general single-qubit matrix (the planner reads the matrix)
            continue;
        }
        for (uint64_t qs = gate_qubits(g); qs; qs &= qs - 1) open[__builtin_ctzll(qs)] = -1;
        if (g.type == G_SWAP) open[g.control] = -1;
        out.push_back(g);
        if (origin) origin->push_back(int(&g - gates.data()));
        if (one) open[g.target] = (int)out.size() - 1;
    }
    return out;
}

}  // namespace hq
