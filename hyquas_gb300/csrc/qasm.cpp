// OpenQASM 2 front-end: the subset the reference's parser reads
// (parse_circuit / parse_gate / parse_qid, main.cpp:12-230).
//
// Grammar, as there: whitespace-separated statements; lines starting with
// `//`, `OPENQASM` or `include` are skipped; `qreg q[n];` sets the register;
// gates `cx ccx cy cz h x y z s sdg t tdg` take an operand token whose
// integers are the qubits in factory order (control(s) first); parameterised
// gates `crx cry crz cu1 u1 u3 rx ry rz` take `name(p1,p2,...)` where a
// parameter is `pi*x` (pi times x), `pi/x` (pi over x) or a decimal number.
// Extensions (each an error or a crash in the reference): `-pi*x` / `-pi/x`,
// `u2(phi,lambda)`, `id`, `swap`, and `creg` / `barrier` / `measure`
// statements, which are skipped.  Errors return HQ_ERR_INVALID with the line
// number instead of exiting.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"
#include "gates.h"

namespace hq {

namespace {

struct Parser {
    const char* s;
    size_t pos = 0, len;
    int line = 1;

    explicit Parser(const char* text) : s(text), len(std::strlen(text)) {}

    void skip_ws() {
        while (pos < len && std::isspace((unsigned char)s[pos])) {
            if (s[pos] == '\n') line++;
            pos++;
        }
    }
    std::string token() {
        skip_ws();
        size_t b = pos;
        while (pos < len && !std::isspace((unsigned char)s[pos])) pos++;
        return std::string(s + b, pos - b);
    }
    void rest_of_line() {
        while (pos < len && s[pos] != '\n') pos++;
    }
    [[noreturn]] void error(const char* what, const std::string& tok) {
        fail(HQ_ERR_INVALID, "qasm line %d: %s '%s'", line, what, tok.c_str());
    }
};

// every decimal integer in the token, in order (main.cpp:12-27)
std::vector<int> qubit_ids(const std::string& t) {
    std::vector<int> out;
    for (size_t i = 0; i < t.size(); i++) {
        if (!std::isdigit((unsigned char)t[i])) continue;
        long v = 0;
        while (i < t.size() && std::isdigit((unsigned char)t[i])) {
            v = v * 10 + (t[i] - '0');
            if (v > 1000000) break;
            i++;
        }
        out.push_back((int)v);
    }
    return out;
}

double parse_param(Parser& p, const std::string& st) {
    std::string x = st;
    double sign = 1.0;
    if (!x.empty() && x[0] == '-' && x.compare(1, 2, "pi") == 0) {
        sign = -1.0;
        x.erase(0, 1);
    }
    const double pi = std::acos(-1.0);
    char* end = nullptr;
    if (x.compare(0, 3, "pi*") == 0) {
        const double v = std::strtod(x.c_str() + 3, &end);
        if (end == x.c_str() + 3 || *end) p.error("bad parameter", st);
        return sign * pi * v;
    }
    if (x.compare(0, 3, "pi/") == 0) {
        const double v = std::strtod(x.c_str() + 3, &end);
        if (end == x.c_str() + 3 || *end || v == 0.0) p.error("bad parameter", st);
        return sign * pi / v;
    }
    if (x == "pi") return sign * pi;
    const double v = std::strtod(x.c_str(), &end);
    if (end == x.c_str() || *end) p.error("bad parameter", st);
    return v;
}

// name(p1,...) -> name, params (main.cpp:29-63)
void split_gate(Parser& p, const std::string& tok, std::string& name, std::vector<double>& params) {
    const size_t open = tok.find('(');
    name = tok.substr(0, open);
    params.clear();
    if (open == std::string::npos) return;
    const size_t close = tok.find(')', open);
    if (close == std::string::npos) p.error("unclosed parameter list", tok);
    std::string body = tok.substr(open + 1, close - open - 1);
    size_t b = 0;
    while (b <= body.size()) {
        size_t e = body.find(',', b);
        if (e == std::string::npos) e = body.size();
        params.push_back(parse_param(p, body.substr(b, e - b)));
        b = e + 1;
    }
}

}  // namespace

void parse_qasm(const char* text, int& n, std::vector<hq_gate>& out) {
    Parser p(text);
    n = -1;
    out.clear();
    struct Fixed {
        const char* name;
        int type, nq;
    };
    static const Fixed fixed[] = {
        {"cx", G_CNOT, 2}, {"ccx", G_CCX, 3}, {"cy", G_CY, 2}, {"cz", G_CZ, 2},
        {"h", G_H, 1},     {"x", G_X, 1},     {"y", G_Y, 1},   {"z", G_Z, 1},
        {"s", G_S, 1},     {"sdg", G_SDG, 1}, {"t", G_T, 1},   {"tdg", G_TDG, 1},
        {"id", G_ID, 1},   {"swap", G_SWAP, 2},
    };
    struct Param {
        const char* name;
        int type, nq, np;
    };
    static const Param param[] = {
        {"crx", G_CRX, 2, 1}, {"cry", G_CRY, 2, 1}, {"crz", G_CRZ, 2, 1}, {"cu1", G_CU1, 2, 1},
        {"u1", G_U1, 1, 1},   {"u2", G_U2, 1, 2},   {"u3", G_U3, 1, 3},   {"rx", G_RX, 1, 1},
        {"ry", G_RY, 1, 1},   {"rz", G_RZ, 1, 1},
    };
    auto add = [&](int type, const std::vector<int>& q, const std::vector<double>& prm,
                   const std::string& tok) {
        if (n < 0) p.error("gate before qreg", tok);
        int target, control = -1, control2 = -1;
        if (type == G_SWAP) {
            target = q[0];
            control = q[1];
        } else if (q.size() == 3) {
            control = q[0];
            control2 = q[1];
            target = q[2];
        } else if (q.size() == 2) {
            control = q[0];
            target = q[1];
        } else {
            target = q[0];
        }
        hq_gate g = make_gate(type, target, control, control2, prm.empty() ? nullptr : prm.data());
        validate_gate(g, n);
        out.push_back(g);
    };
    for (;;) {
        std::string tok = p.token();
        if (tok.empty()) break;
        if (tok.compare(0, 2, "//") == 0 || tok == "OPENQASM" || tok == "include" ||
            tok == "creg" || tok == "barrier" || tok == "measure") {
            p.rest_of_line();
            continue;
        }
        if (tok == "qreg") {
            std::string r = p.token();
            std::vector<int> v = qubit_ids(r);
            if (v.size() != 1 || v[0] < 1 || v[0] > 36) p.error("bad qreg", r);
            if (n >= 0) p.error("second qreg", r);
            n = v[0];
            p.rest_of_line();
            continue;
        }
        bool done = false;
        for (const Fixed& f : fixed) {
            if (tok != f.name) continue;
            std::string ops = p.token();
            std::vector<int> q = qubit_ids(ops);
            if ((int)q.size() != f.nq) p.error("wrong number of qubits", ops);
            add(f.type, q, {}, ops);
            done = true;
            break;
        }
        if (!done) {
            std::string name;
            std::vector<double> prm;
            split_gate(p, tok, name, prm);
            for (const Param& g : param) {
                if (name != g.name) continue;
                if ((int)prm.size() != g.np) p.error("wrong number of parameters", tok);
                std::string ops = p.token();
                std::vector<int> q = qubit_ids(ops);
                if ((int)q.size() != g.nq) p.error("wrong number of qubits", ops);
                add(g.type, q, prm, ops);
                done = true;
                break;
            }
        }
        if (!done) p.error("unrecognized token", tok);
        p.rest_of_line();
    }
    if (n < 0) fail(HQ_ERR_INVALID, "qasm: no qreg declaration");
}

}  // namespace hq
