// Header-only C++ facade over the hyquas_gb300 C ABI with the reference's
// user API: Circuit (src/circuit.h:20-46), Gate and its static factories
// (src/gate.h:11-66), ResultItem (src/circuit.h:9-18).  Method names, argument
// orders (control before target) and return values follow the reference, so
// code written against it compiles after replacing its includes with this
// header and linking libhyquas_gb300.so.
//
// Differences:
//   - amplitudes are complex64 (the reference's FP32 build); matrices are kept
//     in double as the reference factories compute them;
//   - errors throw hyquas::Error (status code + message) instead of exiting;
//   - MyGlobalVars::init() is optional (the library initialises device 0 on
//     first use); hyquas::init(device) selects another device;
//   - Circuit::compile(options) and Circuit::state() expose the backend choice
//     and the device state; Gate::SWAP folds into the qubit layout.
#pragma once

#include <cmath>
#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../include/hyquas_gb300.h"

namespace hyquas {

typedef long long qindex;
typedef double qreal;
struct qComplex {
    float x, y;
};

enum class GateType {
    CCX, CNOT, CY, CZ, CRX, CRY, CU1, CRZ, U1, U2, U3, H, X, Y, Z, S, SDG, T, TDG, RX, RY, RZ,
    TOTAL, ID, SWAP = HQ_SWAP
};

struct Error : std::runtime_error {
    hq_status code;
    Error(hq_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(hq_status s) {
    if (s != HQ_OK) throw Error(s, hq_last_error());
}

inline void init(int device = 0) { check(hq_init(device)); }

struct Gate {
    hq_gate g{};
    GateType type = GateType::ID;
    int targetQubit = 0;
    int controlQubit = -1;   // -1 if no control
    int controlQubit2 = -1;  // -1 if no control

    Gate() = default;
    bool isControlGate() const { return controlQubit != -1; }
    bool isC2Gate() const { return controlQubit2 != -1; }
    bool isDiagonal() const {
        return type == GateType::CZ || type == GateType::CU1 || type == GateType::CRZ ||
               type == GateType::U1 || type == GateType::Z || type == GateType::S ||
               type == GateType::SDG || type == GateType::T || type == GateType::TDG ||
               type == GateType::RZ;
    }
    // mat[r][c] as (re, im), row-major
    double re(int r, int c) const { return g.mat[(r * 2 + c) * 2]; }
    double im(int r, int c) const { return g.mat[(r * 2 + c) * 2 + 1]; }

    static Gate make(GateType t, int target, int control = -1, int control2 = -1,
                     std::vector<double> params = {}) {
        Gate x;
        check(hq_gate_make((int32_t)t, target, control, control2,
                           params.empty() ? nullptr : params.data(), &x.g));
        x.type = t;
        x.targetQubit = target;
        x.controlQubit = control;
        x.controlQubit2 = control2;
        return x;
    }
    static Gate CCX(int c1, int c2, int targetQubit) {
        return make(GateType::CCX, targetQubit, c1, c2);
    }
    static Gate CNOT(int controlQubit, int targetQubit) {
        return make(GateType::CNOT, targetQubit, controlQubit);
    }
    static Gate CY(int controlQubit, int targetQubit) {
        return make(GateType::CY, targetQubit, controlQubit);
    }
    static Gate CZ(int controlQubit, int targetQubit) {
        return make(GateType::CZ, targetQubit, controlQubit);
    }
    static Gate CRX(int controlQubit, int targetQubit, qreal angle) {
        return make(GateType::CRX, targetQubit, controlQubit, -1, {angle});
    }
    static Gate CRY(int controlQubit, int targetQubit, qreal angle) {
        return make(GateType::CRY, targetQubit, controlQubit, -1, {angle});
    }
    static Gate CU1(int controlQubit, int targetQubit, qreal lambda) {
        return make(GateType::CU1, targetQubit, controlQubit, -1, {lambda});
    }
    static Gate CRZ(int controlQubit, int targetQubit, qreal angle) {
        return make(GateType::CRZ, targetQubit, controlQubit, -1, {angle});
    }
    static Gate U1(int targetQubit, qreal lambda) {
        return make(GateType::U1, targetQubit, -1, -1, {lambda});
    }
    static Gate U2(int targetQubit, qreal phi, qreal lambda) {
        return make(GateType::U2, targetQubit, -1, -1, {phi, lambda});
    }
    static Gate U3(int targetQubit, qreal theta, qreal phi, qreal lambda) {
        return make(GateType::U3, targetQubit, -1, -1, {theta, phi, lambda});
    }
    static Gate H(int targetQubit) { return make(GateType::H, targetQubit); }
    static Gate X(int targetQubit) { return make(GateType::X, targetQubit); }
    static Gate Y(int targetQubit) { return make(GateType::Y, targetQubit); }
    static Gate Z(int targetQubit) { return make(GateType::Z, targetQubit); }
    static Gate S(int targetQubit) { return make(GateType::S, targetQubit); }
    static Gate SDG(int targetQubit) { return make(GateType::SDG, targetQubit); }
    static Gate T(int targetQubit) { return make(GateType::T, targetQubit); }
    static Gate TDG(int targetQubit) { return make(GateType::TDG, targetQubit); }
    static Gate RX(int targetQubit, qreal angle) {
        return make(GateType::RX, targetQubit, -1, -1, {angle});
    }
    static Gate RY(int targetQubit, qreal angle) {
        return make(GateType::RY, targetQubit, -1, -1, {angle});
    }
    static Gate RZ(int targetQubit, qreal angle) {
        return make(GateType::RZ, targetQubit, -1, -1, {angle});
    }
    static Gate ID(int targetQubit) { return make(GateType::ID, targetQubit); }
    static Gate SWAP(int a, int b) { return make(GateType::SWAP, a, b); }
};

struct ResultItem {
    ResultItem() = default;
    ResultItem(qindex idx, qComplex amp) : idx(idx), amp(amp) {}
    qindex idx = 0;
    qComplex amp{0.f, 0.f};
    static double zero_wrapper(double x) { return (x > -1e-14 && x < 1e-14) ? 0.0 : x; }
    void print() const {
        std::printf("%lld %.12f: %.12f %.12f\n", idx,
                    double(amp.x) * amp.x + double(amp.y) * amp.y, zero_wrapper(amp.x),
                    zero_wrapper(amp.y));
    }
    bool operator<(const ResultItem& b) const { return idx < b.idx; }
};

class Circuit {
public:
    explicit Circuit(int numQubits) : numQubits(numQubits) {
        check(hq_circuit_create(numQubits, &c_));
    }
    ~Circuit() {
        if (s_) hq_state_destroy(s_);
        if (c_) hq_circuit_destroy(c_);
    }
    Circuit(const Circuit&) = delete;
    Circuit& operator=(const Circuit&) = delete;

    void addGate(const Gate& gate) {
        check(hq_circuit_add_gates(c_, &gate.g, 1));
        gates_.push_back(gate);
    }
    // Circuit::compile, src/circuit.cpp:202-248 (default: OShareMem groups)
    void compile() {
        hq_compile_options o;
        check(hq_compile_options_default(&o));
        compile(o);
    }
    void compile(const hq_compile_options& o) { check(hq_circuit_compile(c_, &o)); }
    // Circuit::run, src/circuit.cpp:16-71: |0..0>, every group, optional
    // copy-back and free; returns the device time in microseconds.
    int run(bool copy_back = true, bool destroy = true) {
        if (!s_) check(hq_state_create(numQubits, &s_));
        check(hq_state_init_zero(s_));
        double us = 0;
        check(hq_circuit_run(c_, s_, &us));
        if (copy_back) {
            result_.resize(size_t(1) << numQubits);
            check(hq_state_store(s_, reinterpret_cast<float*>(result_.data())));
        }
        if (destroy) {
            check(hq_state_destroy(s_));
            s_ = nullptr;
        }
        return int(us);
    }
    // src/circuit.cpp:115-118 (needs run(copy_back = true))
    ResultItem ampAt(qindex idx) const {
        if (result_.empty()) throw Error(HQ_ERR_STATE, "ampAt: run(copy_back=true) first");
        return ResultItem(idx, result_.at(size_t(idx)));
    }
    // src/circuit.cpp:120-142 (needs run(destroy = false))
    qComplex ampAtGPU(qindex idx) const {
        if (!s_) throw Error(HQ_ERR_STATE, "ampAtGPU: run(destroy=false) first");
        uint64_t i = uint64_t(idx);
        qComplex a;
        check(hq_state_amps(s_, &i, 1, reinterpret_cast<float*>(&a)));
        return a;
    }
    // src/circuit.cpp:285-308: amplitudes 0..127, then those with |a|^2 > 0.001
    void printState() const {
        const size_t N = result_.size();
        for (size_t i = 0; i < N && i < 128; i++) ampAt(qindex(i)).print();
        for (size_t i = 128; i < N; i++) {
            const double p = double(result_[i].x) * result_[i].x + double(result_[i].y) * result_[i].y;
            if (p > 0.001) ampAt(qindex(i)).print();
        }
    }
    void dumpGates() const {
        for (const Gate& g : gates_)
            std::printf("type %d target %d control %d control2 %d\n", int(g.type), g.targetQubit,
                        g.controlQubit, g.controlQubit2);
    }
    hq_circuit handle() const { return c_; }
    hq_state state() const { return s_; }  // the device state after run(destroy = false)

    // The compiled schedule as bytes (the reference's Schedule::serialize,
    // src/schedule.cpp:156-325), and a compiled Circuit back from them: the
    // partitioner does not run again.
    std::vector<unsigned char> serialize() const {
        uint64_t len = 0;
        check(hq_circuit_serialize(c_, nullptr, 0, &len));
        std::vector<unsigned char> b(static_cast<size_t>(len));
        check(hq_circuit_serialize(c_, b.data(), len, &len));
        return b;
    }
    static std::unique_ptr<Circuit> deserialize(const std::vector<unsigned char>& b) {
        int32_t n = 0;
        check(hq_schedule_inspect(b.data(), b.size(), &n, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  nullptr));
        hq_circuit h = nullptr;
        check(hq_circuit_deserialize(b.data(), b.size(), &h));
        return std::unique_ptr<Circuit>(new Circuit(n, h));
    }

    const int numQubits;

private:
    Circuit(int n, hq_circuit h) : numQubits(n), c_(h) {}
    hq_circuit c_ = nullptr;
    hq_state s_ = nullptr;
    std::vector<Gate> gates_;
    std::vector<qComplex> result_;
};

// parse_circuit, main.cpp:65-230: an OpenQASM 2 file -> Circuit (the
// reference parser's subset; see hq_qasm_parse).
inline std::unique_ptr<Circuit> parse_circuit(const std::string& filename) {
    std::ifstream f(filename);
    if (!f) throw Error(HQ_ERR_INVALID, "fail to open " + filename);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    int32_t n = 0, count = 0;
    check(hq_qasm_parse(text.c_str(), &n, nullptr, 0, &count));
    std::vector<hq_gate> gs(size_t(count > 0 ? count : 1));
    check(hq_qasm_parse(text.c_str(), &n, gs.data(), count, &count));
    auto c = std::make_unique<Circuit>(n);
    for (int32_t i = 0; i < count; i++) {
        Gate g;
        g.g = gs[i];
        g.type = GateType(gs[i].type);
        g.targetQubit = gs[i].target;
        g.controlQubit = gs[i].control;
        g.controlQubit2 = gs[i].control2;
        c->addGate(g);
    }
    return c;
}

}  // namespace hyquas
