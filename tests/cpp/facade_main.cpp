// Drives the header-only C++ facade (hyquas_gb300/circuit.hpp) the way code
// written against the reference's Circuit/Gate API does.
//   facade_main gates        print every factory matrix (no GPU needed)
//   facade_main run N SEED   U3 + CNOT layers on N qubits, print all amplitudes
//   facade_main qasm FILE    parse, print the gate list; with "run" also run
//                            it and print all amplitudes
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../hyquas_gb300/circuit.hpp"

using namespace hyquas;

static void print_gate(const char* name, const Gate& g) {
    std::printf("%s", name);
    for (int r = 0; r < 2; r++)
        for (int c = 0; c < 2; c++) std::printf(" %.17g %.17g", g.re(r, c), g.im(r, c));
    std::printf("\n");
}

static double uni(unsigned long long& s) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return double(s >> 11) * (1.0 / 9007199254740992.0) * 6.283185307179586;
}

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "gates") == 0) {
        print_gate("CNOT", Gate::CNOT(0, 1));
        print_gate("CY", Gate::CY(0, 1));
        print_gate("CZ", Gate::CZ(0, 1));
        print_gate("CRX", Gate::CRX(0, 1, 0.3));
        print_gate("CRY", Gate::CRY(0, 1, 0.4));
        print_gate("CU1", Gate::CU1(0, 1, 0.5));
        print_gate("CRZ", Gate::CRZ(0, 1, 0.6));
        print_gate("U1", Gate::U1(0, 0.7));
        print_gate("U2", Gate::U2(0, 0.8, 0.9));
        print_gate("U3", Gate::U3(0, 1.0, 1.1, 1.2));
        print_gate("H", Gate::H(0));
        print_gate("X", Gate::X(0));
        print_gate("Y", Gate::Y(0));
        print_gate("Z", Gate::Z(0));
        print_gate("S", Gate::S(0));
        print_gate("SDG", Gate::SDG(0));
        print_gate("T", Gate::T(0));
        print_gate("TDG", Gate::TDG(0));
        print_gate("RX", Gate::RX(0, 1.3));
        print_gate("RY", Gate::RY(0, 1.4));
        print_gate("RZ", Gate::RZ(0, 1.5));
        print_gate("ID", Gate::ID(0));
        print_gate("CCX", Gate::CCX(0, 1, 2));
        return 0;
    }
    if (argc >= 4 && std::strcmp(argv[1], "run") == 0) {
        const int n = std::atoi(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10);
        Circuit c(n);
        for (int layer = 0; layer < 4; layer++) {
            for (int q = 0; q < n; q++) {
                const double a = uni(s), b = uni(s), d = uni(s);
                c.addGate(Gate::U3(q, a, b, d));
            }
            for (int q = layer & 1; q + 1 < n; q += 2) c.addGate(Gate::CNOT(q, q + 1));
        }
        c.compile();
        c.run(true, false);
        const qComplex g0 = c.ampAtGPU(0);
        const ResultItem r0 = c.ampAt(0);
        if (g0.x != r0.amp.x || g0.y != r0.amp.y) {
            std::printf("ampAtGPU/ampAt mismatch\n");
            return 2;
        }
        for (qindex i = 0; i < (qindex(1) << n); i++) {
            const ResultItem r = c.ampAt(i);
            std::printf("%.9g %.9g\n", r.amp.x, r.amp.y);
        }
        return 0;
    }
    if (argc >= 4 && std::strcmp(argv[1], "roundtrip") == 0) {
        // compile, serialise, load the bytes into a second Circuit, run both
        const int n = std::atoi(argv[2]);
        unsigned long long s = std::strtoull(argv[3], nullptr, 10);
        Circuit c(n);
        for (int layer = 0; layer < 4; layer++) {
            for (int q = 0; q < n; q++) c.addGate(Gate::U3(q, uni(s), uni(s), uni(s)));
            for (int q = layer & 1; q + 1 < n; q += 2) c.addGate(Gate::CNOT(q, q + 1));
        }
        c.compile();
        const std::vector<unsigned char> bytes = c.serialize();
        std::unique_ptr<Circuit> d = Circuit::deserialize(bytes);
        c.run();
        d->run();
        for (qindex i = 0; i < (qindex(1) << n); i++) {
            const ResultItem a = c.ampAt(i), b = d->ampAt(i);
            if (a.amp.x != b.amp.x || a.amp.y != b.amp.y) {
                std::printf("mismatch at %lld\n", (long long)i);
                return 2;
            }
        }
        std::printf("ok %zu bytes\n", bytes.size());
        return 0;
    }
    if (argc >= 3 && std::strcmp(argv[1], "qasm") == 0) {
        std::unique_ptr<Circuit> c = parse_circuit(argv[2]);
        c->dumpGates();
        if (argc >= 4 && std::strcmp(argv[3], "run") == 0) {
            c->compile();
            c->run();
            for (qindex i = 0; i < (qindex(1) << c->numQubits); i++) {
                const ResultItem r = c->ampAt(i);
                std::printf("%.9g %.9g\n", r.amp.x, r.amp.y);
            }
        }
        return 0;
    }
    std::fprintf(stderr, "usage: facade_main gates | run N SEED | qasm FILE [run]\n");
    return 1;
}
