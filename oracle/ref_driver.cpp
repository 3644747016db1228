// Golden-data driver for the oracle (test infrastructure only).
//
// Links the reference's own CPU code -- src/gate.cpp (gate factories),
// src/compiler.cpp + src/evaluator.cpp (hybrid partitioner and cost model) and
// src/schedule.cpp (qubit layouts, GateGroup::initCPUMatrix) -- compiled from
// the reference sources by oracle/Makefile, and prints what that code computes
// for a circuit read from stdin.  The outputs become the committed fixtures in
// tests/golden/ that pin the CPU oracle (oracle/oracle.c) and the partitioner.
//
// Input (stdin):
//   n <numQubits>
//   g <type> <target> <control> <control2> <p0> <p1> <p2>   (one per gate;
//       type = reference GateType ordinal, src/gate.h:7-9; -1 = no control)
//   s <re> <im>             (optional: 2^n amplitudes of an input state)
//   cmd matrices|unitary|compile
//
// matrices : one line per gate, the 2x2 matrix from the reference factory.
// unitary  : the whole circuit fused by GateGroup::initCPUMatrix
//            (src/schedule.cpp:578-702) with the identity layout, applied to the
//            input state (or |0..0> when none is given).
// compile  : Compiler::run (src/compiler.cpp:70-165) on a single GPU; per gate
//            group its backend, related qubits, gate indices and layout.
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "compiler.h"
#include "gate.h"
#include "schedule.h"
#include "utils.h"

static Gate make_gate(int type, int t, int c, int c2, double p0, double p1, double p2) {
    switch (GateType(type)) {
        case GateType::CCX: return Gate::CCX(c, c2, t);
        case GateType::CNOT: return Gate::CNOT(c, t);
        case GateType::CY: return Gate::CY(c, t);
        case GateType::CZ: return Gate::CZ(c, t);
        case GateType::CRX: return Gate::CRX(c, t, p0);
        case GateType::CRY: return Gate::CRY(c, t, p0);
        case GateType::CU1: return Gate::CU1(c, t, p0);
        case GateType::CRZ: return Gate::CRZ(c, t, p0);
        case GateType::U1: return Gate::U1(t, p0);
        case GateType::U2: return Gate::U2(t, p0, p1);
        case GateType::U3: return Gate::U3(t, p0, p1, p2);
        case GateType::H: return Gate::H(t);
        case GateType::X: return Gate::X(t);
        case GateType::Y: return Gate::Y(t);
        case GateType::Z: return Gate::Z(t);
        case GateType::S: return Gate::S(t);
        case GateType::SDG: return Gate::SDG(t);
        case GateType::T: return Gate::T(t);
        case GateType::TDG: return Gate::TDG(t);
        case GateType::RX: return Gate::RX(t, p0);
        case GateType::RY: return Gate::RY(t, p0);
        case GateType::RZ: return Gate::RZ(t, p0);
        default: break;
    }
    fprintf(stderr, "unsupported gate type %d\n", type);
    exit(2);
}

static const char* backend_name(Backend b) {
    switch (b) {
        case Backend::PerGate: return "pergate";
        case Backend::BLAS: return "blas";
        default: return "none";
    }
}

int main() {
    MyGlobalVars::numGPUs = 1;
    MyGlobalVars::localGPUs = 1;
    MyGlobalVars::bit = 0;
    MyMPI::rank = 0;
    MyMPI::commSize = 1;
    MyMPI::commBit = 0;

    int n = -1;
    std::vector<Gate> gates;
    std::map<int, int> id_to_index;
    std::vector<double> psi;
    char tag[64];
    std::string cmd;
    while (scanf("%63s", tag) == 1) {
        if (!strcmp(tag, "n")) {
            if (scanf("%d", &n) != 1) return 2;
        } else if (!strcmp(tag, "g")) {
            int type, t, c, c2;
            double p0, p1, p2;
            if (scanf("%d %d %d %d %lf %lf %lf", &type, &t, &c, &c2, &p0, &p1, &p2) != 7) return 2;
            Gate g = make_gate(type, t, c, c2, p0, p1, p2);
            id_to_index[g.gateID] = (int)gates.size();
            gates.push_back(g);
        } else if (!strcmp(tag, "s")) {
            double re, im;
            if (scanf("%lf %lf", &re, &im) != 2) return 2;
            psi.push_back(re);
            psi.push_back(im);
        } else if (!strcmp(tag, "cmd")) {
            char buf[64];
            if (scanf("%63s", buf) != 1) return 2;
            cmd = buf;
        }
    }
    if (n <= 0) return 2;

    if (cmd == "matrices") {
        for (auto& g : gates) {
            printf("m");
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 2; c++) printf(" %.17g %.17g", g.mat[r][c].x, g.mat[r][c].y);
            printf("\n");
        }
    } else if (cmd == "unitary") {
        GateGroup gg;
        gg.gates = gates;
        gg.relatedQubits = (qindex(1) << n) - 1;
        gg.state = State(n);
        gg.matQubit = n;
        gg.backend = Backend::BLAS;
        gg.initCPUMatrix(n);
        const qComplex* mat = gg.matrix[0].get();
        qindex dim = qindex(1) << n;
        if (psi.empty()) {
            psi.assign(2 * dim, 0.0);
            psi[0] = 1.0;
        }
        if ((qindex)psi.size() != 2 * dim) return 3;
        // row c of the reference's matrix holds U e_c (src/schedule.cpp:578-702)
        for (qindex r = 0; r < dim; r++) {
            double re = 0, im = 0;
            for (qindex c = 0; c < dim; c++) {
                qComplex u = mat[c * dim + r];
                re += u.x * psi[2 * c] - u.y * psi[2 * c + 1];
                im += u.x * psi[2 * c + 1] + u.y * psi[2 * c];
            }
            printf("a %.17g %.17g\n", re, im);
        }
    } else if (cmd == "compile") {
        Compiler compiler(n, gates);
        Schedule schedule = compiler.run();
        for (auto& lg : schedule.localGroups) {
            for (auto& gg : lg.fullGroups) {
                printf("group %s related %llu matqubit %d gates %d :", backend_name(gg.backend),
                       (unsigned long long)gg.relatedQubits,
                       gg.backend == Backend::BLAS ? gg.matQubit : 0, (int)gg.gates.size());
                for (auto& g : gg.gates) printf(" %d", id_to_index.at(g.gateID));
                printf(" pos");
                for (int q = 0; q < n; q++) printf(" %d", gg.state.pos[q]);
                printf("\n");
            }
        }
        printf("final");
        for (int q = 0; q < n; q++) printf(" %d", schedule.finalState.pos[q]);
        printf("\n");
    } else {
        fprintf(stderr, "unknown cmd '%s'\n", cmd.c_str());
        return 2;
    }
    return 0;
}
