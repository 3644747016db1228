// Trace driver for the reference's own single-GPU run -- TEST INFRASTRUCTURE ONLY.
//
// Builds the circuit read from stdin with the reference's gate factories
// (src/gate.cpp), then runs the reference's public API exactly as its main.cpp
// does (src/circuit.h:20-46, main.cpp:233-251): MyGlobalVars::init(),
// Circuit(n), addGate, compile(), run(copy_back = false, destroy = false).
// Linked against fake_cuda.cpp instead of the CUDA runtime, so every device
// operation the reference issues lands in the trace given as argv[1]; the
// reference's logical -> physical qubit map is read back through
// Circuit::ampAtGPU (src/circuit.cpp:120-142) and stored in the trace too.
//
// Input (stdin), as oracle/ref_driver.cpp:
//   n <numQubits>
//   g <type> <target> <control> <control2> <p0> <p1> <p2>   (one per gate)
#include <cstdio>
#include <cstring>
#include <vector>

#include "circuit.h"
#include "gate.h"
#include "logger.h"
#include "utils.h"

extern "C" int fake_trace_open(const char* path);
extern "C" void fake_trace_info(int32_t num_qubits);
extern "C" void fake_trace_layout(const int32_t* pos, int32_t n);
extern "C" uint64_t fake_last_d2h_src();
extern "C" uint64_t fake_alloc_base_of(uint64_t addr);
extern "C" void fake_trace_close();

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

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <trace-out> < circuit\n", argv[0]);
        return 2;
    }
    int n = -1;
    std::vector<Gate> gates;
    char tag[64];
    while (scanf("%63s", tag) == 1) {
        if (!strcmp(tag, "n")) {
            if (scanf("%d", &n) != 1) return 2;
        } else if (!strcmp(tag, "g")) {
            int type, t, c, c2;
            double p0, p1, p2;
            if (scanf("%d %d %d %d %lf %lf %lf", &type, &t, &c, &c2, &p0, &p1, &p2) != 7) return 2;
            gates.push_back(make_gate(type, t, c, c2, p0, p1, p2));
        }
    }
    if (n <= 0 || n > 34) return 2;
    if (fake_trace_open(argv[1]) != 0) {
        fprintf(stderr, "cannot write %s\n", argv[1]);
        return 2;
    }
    fake_trace_info(n);
    MyMPI::init();
    MyGlobalVars::init();
    Circuit c(n);
    for (auto& g : gates) c.addGate(g);
    c.compile();
    c.run(false, false);
    // logical qubit q sits at physical position log2(offset of amplitude 1 << q)
    std::vector<int32_t> pos(n, -1);
    for (int q = 0; q < n; q++) {
        c.ampAtGPU(qindex(1) << q);
        const uint64_t src = fake_last_d2h_src();
        const uint64_t off = (src - fake_alloc_base_of(src)) / sizeof(qComplex);
        for (int b = 0; b < n; b++)
            if (off == (uint64_t(1) << b)) pos[q] = b;
        if (pos[q] < 0) {
            fprintf(stderr, "layout of qubit %d not found\n", q);
            return 3;
        }
    }
    fake_trace_layout(pos.data(), n);
    fake_trace_close();
    Logger::print();
    return 0;
}
