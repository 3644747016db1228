#include "compiler.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <mutex>
#include <cstring>

namespace hq {

namespace {

// Fixed-capacity bitset over a gate window (<= 2048 gates).
struct WinSet {
    std::vector<uint64_t> w;
    explicit WinSet(int nbits = 0) : w((nbits + 63) / 64, 0) {}
    void set(int i) { w[i >> 6] |= uint64_t(1) << (i & 63); }
    bool test(int i) const { return (w[i >> 6] >> (i & 63)) & 1; }
    int count() const {
        int c = 0;
        for (uint64_t x : w) c += __builtin_popcountll(x);
        return c;
    }
    bool any() const {
        for (uint64_t x : w)
            if (x) return true;
        return false;
    }
    WinSet& operator|=(const WinSet& o) {
        for (size_t i = 0; i < w.size(); i++) w[i] |= o.w[i];
        return *this;
    }
    void andnot(const WinSet& o) {
        for (size_t i = 0; i < w.size(); i++) w[i] &= ~o.w[i];
    }
};

struct GroupingInput {
    int n;
    const std::vector<hq_gate>* gates;
    std::vector<char> diag;   // per gate: counts as diagonal for grouping
    bool ref_semantics;       // reproduce the reference exactly (CCX control2 ignored)
};

// GateGroup::newRelated, src/schedule.cpp:35-50
uint64_t new_related(uint64_t rel, const hq_gate& g, bool diag, uint64_t local_qubits,
                     bool enable_global) {
    if (enable_global) {
        if (!diag) rel |= uint64_t(1) << g.target;
    } else {
        if (!diag || ((local_qubits >> g.target) & 1)) rel |= uint64_t(1) << g.target;
        if (g.control >= 0 && ((local_qubits >> g.control) & 1)) rel |= uint64_t(1) << g.control;
        if (g.control2 >= 0 && ((local_qubits >> g.control2) & 1)) rel |= uint64_t(1) << g.control2;
    }
    return rel;
}

// OneLayerCompiler::getGroupOpt, src/compiler.cpp:322-452.  Returns indices
// (into the gate list) of the selected gates in window order.
std::vector<int> get_group_opt(const GroupingInput& in, const std::vector<int>& remain,
                               int max_gates, std::vector<char>& full, std::vector<uint64_t>& related,
                               bool enable_global, int local_size, uint64_t local_qubits) {
    const int n = in.n;
    const auto& gates = *in.gates;
    const int gate_num = std::min<int>(max_gates, (int)remain.size());
    std::vector<WinSet> cur(n, WinSet(gate_num));
    WinSet selected(gate_num);

    // phase 1: per-qubit dependency chains while the related set fits
    for (int id = 0; id < gate_num; id++) {
        if (id % 100 == 0) {
            bool live = false;
            for (int i = 0; i < n; i++)
                if (!full[i]) live = true;
            if (!live) break;
        }
        const hq_gate& g = gates[remain[id]];
        const bool dg = in.diag[remain[id]];
        if (g.control >= 0) {
            const int c = g.control, t = g.target;
            const int c2 = in.ref_semantics ? -1 : g.control2;
            if (!full[c] && !full[t] && (c2 < 0 || !full[c2])) {
                uint64_t nr = related[c] | related[t] | (c2 >= 0 ? related[c2] : 0);
                nr = new_related(nr, g, dg, local_qubits, enable_global);
                if (__builtin_popcountll(nr) <= local_size) {
                    WinSet nc = cur[c];
                    nc |= cur[t];
                    if (c2 >= 0) nc |= cur[c2];
                    nc.set(id);
                    cur[c] = nc;
                    cur[t] = nc;
                    related[c] = related[t] = nr;
                    if (c2 >= 0) {
                        cur[c2] = nc;
                        related[c2] = nr;
                    }
                    continue;
                }
            }
            full[c] = full[t] = 1;
            if (c2 >= 0) full[c2] = 1;
        } else {
            if (!full[g.target]) {
                cur[g.target].set(id);
                related[g.target] = new_related(related[g.target], g, dg, local_qubits, enable_global);
            }
        }
    }

    // phase 2: greedy union of the largest chains that still fit
    std::vector<char> blocked(n, 0);
    uint64_t selected_related = 0;
    while (true) {
        int mx = 0, id = -1;
        for (int i = 0; i < n; i++) {
            const int count_i = cur[i].count();
            if (!blocked[i] && count_i > mx) {
                if (__builtin_popcountll(selected_related | related[i]) <= local_size) {
                    mx = count_i;
                    id = i;
                } else {
                    blocked[i] = 1;
                }
            }
        }
        if (mx == 0) break;
        selected |= cur[id];
        selected_related |= related[id];
        blocked[id] = 1;
        for (int i = 0; i < n; i++) {
            if (!blocked[i] && cur[i].any()) {
                if ((related[i] | selected_related) == selected_related) {
                    selected |= cur[i];
                    blocked[i] = 1;
                } else {
                    cur[i].andnot(cur[id]);
                }
            }
        }
    }

    if (enable_global) {
        // phase 3: absorb diagonal gates on qubits not blocked by a skipped gate
        std::fill(blocked.begin(), blocked.end(), 0);
        int cnt = 0;
        for (int id = 0; id < gate_num; id++) {
            cnt++;
            if (cnt % 100 == 0) {
                bool live = false;
                for (int i = 0; i < n; i++)
                    if (!blocked[i]) live = true;
                if (!live) break;
            }
            if (selected.test(id)) continue;
            const hq_gate& g = gates[remain[id]];
            const int c2 = in.ref_semantics ? -1 : g.control2;
            if (in.diag[remain[id]]) {
                if (g.control >= 0) {
                    if (!blocked[g.control] && !blocked[g.target] && (c2 < 0 || !blocked[c2])) {
                        selected.set(id);
                    } else {
                        blocked[g.control] = blocked[g.target] = 1;
                        if (c2 >= 0) blocked[c2] = 1;
                    }
                } else if (!blocked[g.target]) {
                    selected.set(id);
                }
            } else {
                if (g.control >= 0) blocked[g.control] = 1;
                if (c2 >= 0) blocked[c2] = 1;
                blocked[g.target] = 1;
            }
        }
    }
    std::vector<int> ret;
    for (int id = 0; id < gate_num; id++)
        if (selected.test(id)) ret.push_back(remain[id]);
    return ret;
}

void remove_selected(std::vector<int>& remain, const std::vector<int>& sel) {
    std::vector<int> out;
    out.reserve(remain.size());
    size_t j = 0;
    for (int x : remain) {
        while (j < sel.size() && sel[j] < x) j++;
        if (j < sel.size() && sel[j] == x) continue;
        out.push_back(x);
    }
    remain.swap(out);
}

// GateGroup::initBlasState, src/schedule.cpp:339-382: bring the group's
// qubits to the lowest physical positions (layout only).
void blas_layout(std::vector<int>& pos, std::vector<int>& layout, uint64_t related, int n) {
    const int nm = __builtin_popcountll(related);
    std::vector<int> to_global, to_local;
    for (int i = 0; i < nm; i++)
        if (!((related >> layout[i]) & 1)) to_global.push_back(layout[i]);
    for (int i = nm; i < n; i++)
        if ((related >> layout[i]) & 1) to_local.push_back(layout[i]);
    for (size_t i = 0; i < to_global.size() && i < to_local.size(); i++) {
        const int x = to_global[i], y = to_local[i];
        std::swap(pos[x], pos[y]);
        layout[pos[x]] = x;
        layout[pos[y]] = y;
    }
}

}  // namespace

uint64_t pad_tile(uint64_t mask, int k, int n) {
    for (int b = 0; b < n && __builtin_popcountll(mask) < k; b++) mask |= uint64_t(1) << b;
    return mask;
}

// Greedy grouping can leave a late group with a handful of gates, which then
// costs a whole pass over the state.  Each gate of such a group moves to the
// end of the latest earlier OShareMem group that can hold it -- its
// non-diagonal target inside that group's tile (diagonal gates fit any tile)
// -- provided every gate it moves past commutes with it (disjoint qubits, or
// both diagonal).  The group is dropped when all of its gates found a place.
void absorb_small_groups(Partition& part, const std::vector<hq_gate>& gates,
                         const std::vector<char>& diag, int n, int max_gates) {
    auto commute = [&](int a, int b) {
        return (gate_qubits(gates[a]) & gate_qubits(gates[b])) == 0 || (diag[a] && diag[b]);
    };
    for (size_t g = part.groups.size(); g-- > 1;) {
        const GroupPlan& src = part.groups[g];
        if ((int)src.gates.size() > max_gates || src.backend != HQ_BACKEND_OSHM) continue;
        std::vector<std::vector<int>> add(g);
        std::vector<int> placed(src.gates.size(), -1);
        bool ok = true;
        for (size_t xi = 0; xi < src.gates.size() && ok; xi++) {
            const int x = src.gates[xi];
            int lb = 0;
            for (size_t yi = 0; yi < xi; yi++)
                if (!commute(src.gates[yi], x)) lb = std::max(lb, placed[yi]);
            int where = -1;
            for (int p = (int)g - 1; p >= lb; p--) {
                const GroupPlan& gp = part.groups[p];
                if (gp.backend == HQ_BACKEND_OSHM) {
                    const uint64_t tile = pad_tile(gp.related | 1, gp.width, n);
                    if (diag[x] || ((tile >> gates[x].target) & 1)) {
                        where = p;
                        break;
                    }
                }
                bool pass = true;
                for (int y : gp.gates) pass = pass && commute(y, x);
                for (int y : add[p]) pass = pass && commute(y, x);
                if (!pass) break;
            }
            if (where < 0) {
                ok = false;
                break;
            }
            placed[xi] = where;
            add[where].push_back(x);
        }
        if (!ok) continue;
        for (size_t p = 0; p < g; p++) {
            GroupPlan& gp = part.groups[p];
            for (int x : add[p]) {
                gp.gates.push_back(x);
                if (!diag[x]) gp.related |= uint64_t(1) << gates[x].target;
            }
        }
        part.groups.erase(part.groups.begin() + g);
    }
}

namespace {
Partition partition_greedy(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                           const CompileConfig& cfg);
}  // namespace

// The greedy grouping in gate order, and (GB300 widths) the same greedy over
// the gates in reverse order with its groups played back in reverse (the
// dependencies of a reversed circuit are the reversed ones, so the played-back
// groups are a valid schedule); the one with fewer passes is kept, the
// forward one on a tie.  The reference's grouping is only the forward greedy.
namespace {
Partition partition_width(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                          const CompileConfig& cfg);
}  // namespace

// The cost model's device time of a partition (seconds).
double predicted_time(int n, const std::vector<hq_gate>& gates, const Partition& part,
                      const CompileConfig& cfg) {
    double t = 0;
    for (const GroupPlan& gp : part.groups) {
        if (gp.backend == HQ_BACKEND_OSHM) {
            std::vector<hq_gate> gs;
            for (int x : gp.gates) gs.push_back(gates[x]);
            t += cost_oshm(n, 0, gs, gp.width);
        } else {
            t += cost_transmm(n, gp.width, cfg.mm_precision);
        }
    }
    return t;
}

// With tile_auto the OShareMem tile width is chosen per circuit: the circuit
// is partitioned at 13, 12 and 11 tile qubits and a narrower tile is kept
// only when the cost model predicts it at least 15 % faster than the widest
// so far: the model prices passes and arithmetic, not the narrower kernels'
// lower efficiency per pass (measured on GB300: the 30-qubit grid 60.6 ms at
// 13, 69.9 at 12, 67.2 at 11; QFT-28 5.1 ms at 13).  The reference reads
// per-qubit-count parameter files for its choices instead
// (src/evaluator.cpp:60-109).
//
// The hybrid's per-group choice (the reference's, by predicted time per gate)
// can miss a schedule that is faster as a whole: deep dense blocks that all
// fuse into TransMM groups, say.  So the hybrid also partitions the circuit
// OShareMem-only and TransMM-only and keeps whichever of the three the cost
// model predicts fastest.
Partition partition(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                    const CompileConfig& cfg) {
    auto one = [&](const CompileConfig& c) {
        Partition p = partition_width(n, gates, pos0, c);
        if (c.backend != HQ_BACKEND_HYBRID || c.reference) return p;
        double bt = predicted_time(n, gates, p, c);
        for (int alt : {HQ_BACKEND_OSHM, HQ_BACKEND_TRANSMM}) {
            CompileConfig a = c;
            a.backend = alt;
            Partition q = partition_width(n, gates, pos0, a);
            const double qt = predicted_time(n, gates, q, a);
            if (qt < bt) {
                p = std::move(q);
                bt = qt;
            }
        }
        return p;
    };
    if (!cfg.tile_auto || cfg.reference || cfg.backend == HQ_BACKEND_TRANSMM) return one(cfg);
    Partition best;
    double best_t = 0;
    bool have = false;
    for (int t = 13; t >= 11; t--) {
        if (t > n && have) continue;
        CompileConfig c = cfg;
        c.tile = std::min(t, n);
        Partition p = one(c);
        const double pt = predicted_time(n, gates, p, c);
        if (!have || pt < best_t * 0.85) {
            best = std::move(p);
            best_t = pt;
            have = true;
        }
        if (t > n) break;
    }
    return best;
}

namespace {
Partition partition_width(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                          const CompileConfig& cfg) {
    Partition fwd = partition_greedy(n, gates, pos0, cfg);
    if (cfg.reference || gates.size() < 2) return fwd;
    const int N = (int)gates.size();
    std::vector<hq_gate> rev(gates.rbegin(), gates.rend());
    Partition back = partition_greedy(n, rev, pos0, cfg);
    if (back.groups.size() >= fwd.groups.size()) return fwd;
    Partition out;
    for (auto it = back.groups.rbegin(); it != back.groups.rend(); ++it) {
        GroupPlan gp = *it;
        for (int& x : gp.gates) x = N - 1 - x;
        std::sort(gp.gates.begin(), gp.gates.end());
        out.groups.push_back(std::move(gp));
    }
    out.final_pos = fwd.final_pos;  // layouts stay the identity outside reference grouping
    return out;
}
}  // namespace

namespace {
Partition partition_greedy(int n, const std::vector<hq_gate>& gates, const std::vector<int>& pos0,
                           const CompileConfig& cfg) {
    Partition out;
    GroupingInput in;
    in.n = n;
    in.gates = &gates;
    in.ref_semantics = cfg.reference;
    in.diag.resize(gates.size());
    for (size_t i = 0; i < gates.size(); i++)
        in.diag[i] = cfg.reference ? ref_is_diagonal(gates[i].type) : matrix_is_diagonal(gates[i]);

    std::vector<int> pos = pos0, layout(n);
    for (int q = 0; q < n; q++) layout[pos[q]] = q;
    std::vector<int> remain(gates.size());
    for (size_t i = 0; i < gates.size(); i++) remain[i] = (int)i;
    const uint64_t all = n >= 64 ? ~uint64_t(0) : ((uint64_t(1) << n) - 1);
    const int tile = cfg.reference ? 10 : std::min(cfg.tile, n);
    const int coalesce = cfg.reference ? 3 : std::max(1, std::min(cfg.coalesce, tile));
    const int mat = cfg.reference ? 6 : std::min(cfg.mm_qubits, n);

    auto oshm_candidate = [&](uint64_t& rel_out) {
        std::vector<char> full(n, 0);
        uint64_t seed = 0;
        for (int j = 0; j < coalesce && j < n; j++) seed |= uint64_t(1) << layout[j];
        std::vector<uint64_t> related(n, seed);
        std::vector<int> idx = get_group_opt(in, remain, 512, full, related, true, tile, all);
        uint64_t rel = 0;
        for (int x : idx) rel = new_related(rel, gates[x], in.diag[x], all, true);
        rel_out = rel | seed;
        return idx;
    };
    auto mm_candidate = [&](int m, uint64_t& rel_out) {
        std::vector<char> full(n, 0);
        std::vector<uint64_t> related(n, 0);
        std::vector<int> idx = get_group_opt(in, remain, 512, full, related, false, m, all);
        uint64_t rel = 0;
        for (int x : idx) rel = new_related(rel, gates[x], in.diag[x], all, false);
        rel_out = rel;
        return idx;
    };

    int guard = 0;
    while (!remain.empty()) {
        HQ_REQUIRE(++guard < 1000000, HQ_ERR_INVALID, "partition did not converge");
        GroupPlan gp;
        gp.pos = pos;
        uint64_t rel = 0;
        std::vector<int> idx;
        int backend = cfg.backend == HQ_BACKEND_TRANSMM ? HQ_BACKEND_TRANSMM : HQ_BACKEND_OSHM;
        if (cfg.backend == HQ_BACKEND_HYBRID && !cfg.reference) {
            // per-group choice by predicted time per gate (src/compiler.cpp:248-280)
            uint64_t r_o = 0;
            std::vector<int> io = oshm_candidate(r_o);
            double best = 1e30;
            if (!io.empty()) {
                std::vector<hq_gate> gs;
                for (int x : io) gs.push_back(gates[x]);
                best = cost_oshm(n, 0, gs, tile) / io.size();
            }
            idx = io;
            rel = r_o;
            backend = HQ_BACKEND_OSHM;
            for (int m = 4; m <= std::min(mat, 8); m++) {
                uint64_t r_m = 0;
                std::vector<int> im = mm_candidate(m, r_m);
                if (im.empty()) continue;
                const double eff = cost_transmm(n, std::max(m, __builtin_popcountll(r_m)),
                                                cfg.mm_precision) / im.size();
                if (eff < best) {
                    best = eff;
                    idx = im;
                    rel = r_m;
                    backend = HQ_BACKEND_TRANSMM;
                }
            }
        } else if (backend == HQ_BACKEND_OSHM) {
            idx = oshm_candidate(rel);
        } else {
            idx = mm_candidate(mat, rel);
        }
        if (idx.empty()) {  // cannot happen for valid widths; keep progress anyway
            idx.push_back(remain.front());
            rel = gate_qubits(gates[remain.front()]);
        }
        gp.backend = backend;
        gp.gates = idx;
        gp.related = rel;
        if (backend == HQ_BACKEND_OSHM) {
            gp.width = tile;
        } else {
            gp.width = std::max(__builtin_popcountll(rel), cfg.reference ? 4 : 1);
            if (cfg.reference) blas_layout(pos, layout, rel, n);
        }
        gp.pos_after = pos;
        remove_selected(remain, idx);
        out.groups.push_back(std::move(gp));
    }
    out.final_pos = pos;
    if (!cfg.reference) absorb_small_groups(out, gates, in.diag, n, 16);
    return out;
}
}  // namespace

// ---- OShareMem lowering ---------------------------------------------------------

namespace {

// smem slot class of a local tile bit: which of slot bits 0..3 it moves
// (see the swizzle in k_oshm.cu)
int slot_class(int b) { return b <= 3 ? b : 1 + (b - 4) % 3; }

}  // namespace

namespace {

bool close(double a, double b) { return std::fabs(a - b) < 1e-12; }

// Hadamard-like 2x2 matrices that the kernel runs as adds with a deferred
// 1/sqrt(2): H, RY(pi/2) (sqrt(Y)), RX(pi/2) (sqrt(X)).
int hadamard_like(const hq_gate& g) {
    const double c = 1.0 / std::sqrt(2.0);
    const double* m = g.mat;
    auto is = [&](double r00, double i00, double r01, double i01, double r10, double i10, double r11,
                  double i11) {
        return close(m[0], r00) && close(m[1], i00) && close(m[2], r01) && close(m[3], i01) &&
               close(m[4], r10) && close(m[5], i10) && close(m[6], r11) && close(m[7], i11);
    };
    if (is(c, 0, c, 0, c, 0, -c, 0)) return OP_H;
    if (is(c, 0, -c, 0, c, 0, c, 0)) return OP_SY;
    if (is(c, 0, 0, -c, 0, -c, c, 0)) return OP_SX;
    return -1;
}

}  // namespace

namespace {

// values within 1e-14 of 0 or +-1 are those exactly (so that RZ(pi) becomes a sign flip)
double snap(double x) {
    for (double v : {0.0, 1.0, -1.0})
        if (std::fabs(x - v) < 1e-14) return v;
    return x;
}

// the shear form of a rotation by phi: phi reduced to [-pi/2, pi/2] (a rotation
// by pi is a negation), a = -tan(phi/2), b = sin(phi)
// a real 2x2 [[c, -s], [s, c]] with c^2 + s^2 = 1 (RY and its powers)
bool is_rotation(const hq_gate& g) {
    const double c = g.mat[0], s = g.mat[4];
    return std::fabs(g.mat[6] - c) < 1e-12 && std::fabs(g.mat[2] + s) < 1e-12 &&
           std::fabs(c * c + s * s - 1.0) < 1e-12;
}

void shear(double phi, OshmOp& o) {
    const double pi = std::acos(-1.0);
    if (phi > pi / 2) {
        phi -= pi;
        o.flags |= OPF_NEG;
    } else if (phi < -pi / 2) {
        phi += pi;
        o.flags |= OPF_NEG;
    }
    o.m[0] = (float)(-std::tan(phi / 2));
    o.m[1] = (float)std::sin(phi);
}

}  // namespace

OshmProgram plan_oshm(int n, const std::vector<hq_gate>& gates, uint64_t tile_mask) {
    OshmProgram prog;
    const int k = __builtin_popcountll(tile_mask);
    HQ_REQUIRE(k >= 6 && k <= OSHM_MAX_K && k <= n, HQ_ERR_INVALID, "oshm: tile width %d", k);
    HQ_REQUIRE(tile_mask & 1, HQ_ERR_INVALID, "oshm: tile must contain physical qubit 0");
    const int r = oshm_reg_bits(k);
    prog.n = n;
    prog.k = k;
    prog.r = r;
    prog.tile_mask = tile_mask;
    int loc[64];
    int phys_of[OSHM_MAX_K];
    for (int b = 0, j = 0; b < 64; b++) {
        loc[b] = -1;
        if ((tile_mask >> b) & 1) {
            loc[b] = j;
            phys_of[j] = b;
            j++;
        }
    }
    std::vector<char> diag(gates.size());
    for (size_t i = 0; i < gates.size(); i++) {
        diag[i] = matrix_is_diagonal(gates[i]);
        HQ_REQUIRE(diag[i] || loc[gates[i].target] >= 0, HQ_ERR_INVALID,
                   "oshm: non-diagonal gate on qubit %d outside the tile", gates[i].target);
    }

    const double rsqrt2 = 1.0 / std::sqrt(2.0);
    std::complex<double> gfac(1.0, 0.0);  // factors taken out of uncontrolled diagonal gates
    double pending_scale = 1.0;  // deferred 1/sqrt2 factors not applied yet
    int pending_count = 0;
    std::vector<char> done(gates.size(), 0);
    size_t ndone = 0;
    // The gates of the next phase given the gates done so far, and its register
    // qubits: local qubit 0 always (the f32x2 lane), plus up to r-1 targets
    // chosen greedily in gate order, padded with the tile qubits fewest of the
    // phase's diagonal gates target (a diagonal gate off the register set is a
    // per-thread scalar instead of a multiply per amplitude).
    auto choose = [&](const std::vector<char>& dn, std::vector<int>& members, uint32_t& rset) {
        rset = 1u;
        members.clear();
        uint64_t blocked = 0;
        for (size_t i = 0; i < gates.size(); i++) {
            if (dn[i]) continue;
            const hq_gate& g = gates[i];
            const uint64_t q = gate_qubits(g);
            if (q & blocked) {
                blocked |= q;
                continue;
            }
            if (!diag[i]) {
                const uint32_t tl = 1u << loc[g.target];
                if (!(rset & tl)) {
                    if (__builtin_popcount(rset) >= r) {
                        blocked |= q;
                        continue;
                    }
                    rset |= tl;
                }
            }
            members.push_back((int)i);
        }
        std::vector<int> score(k, 0);
        for (int i : members)
            if (diag[i] && loc[gates[i].target] >= 0) score[loc[gates[i].target]]++;
        // ties go to the highest tile qubits: the low ones stay thread bits, where
        // they give whole 32-byte sectors to the stores of neighbouring threads
        std::vector<int> cand;
        for (int b = k - 1; b >= 1; b--)
            if (!((rset >> b) & 1)) cand.push_back(b);
        std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return score[a] < score[b]; });
        for (int b : cand) {
            if (__builtin_popcount(rset) >= r) break;
            rset |= 1u << b;
        }
    };
    // a diagonal gate that the kernels run as a per-thread complex factor when
    // its target is a thread bit (not a pure sign, no register control)
    auto thread_factor = [&](int i, uint32_t rset) {
        const hq_gate& g = gates[i];
        if (!diag[i]) return false;
        const int lt = loc[g.target];
        if (lt >= 0 && ((rset >> lt) & 1)) return false;
        for (int c : {g.control, g.control2})
            if (c >= 0 && loc[c] >= 0 && ((rset >> loc[c]) & 1)) return false;
        const bool sign = g.mat[0] == 1.0 && g.mat[1] == 0.0 && g.mat[6] == -1.0 && g.mat[7] == 0.0;
        return !sign;
    };
    while (ndone < gates.size()) {
        std::vector<int> members;
        uint32_t rset;
        choose(done, members, rset);
        HQ_REQUIRE(!members.empty(), HQ_ERR_INVALID, "oshm: planner made no progress");
        // A single-qubit diagonal gate on a register qubit (other than the lane)
        // that no later non-diagonal gate of the phase targets can wait for the
        // next phase (it commutes with everything between).  Where its qubit is
        // a thread bit there, it is a per-thread factor instead of arithmetic on
        // every amplitude (about 16 packed operations per thread), but a phase
        // with such factors pays a complex multiply of its amplitudes (about 32
        // more): the gates wait when the next phase, planned ahead, gains.
        {
            std::vector<int> keep, later;
            for (size_t a = 0; a < members.size(); a++) {
                const int i = members[a];
                const hq_gate& g = gates[i];
                const int lt = loc[g.target];
                bool wait = diag[i] && g.control < 0 && g.control2 < 0 && lt > 0 && ((rset >> lt) & 1);
                for (size_t b = a + 1; wait && b < members.size(); b++)
                    if (!diag[members[b]] && gates[members[b]].target == g.target) wait = false;
                (wait ? later : keep).push_back(i);
            }
            if (!later.empty() && !keep.empty() && ndone + members.size() < gates.size()) {
                std::vector<char> dn = done;
                for (int i : keep) dn[i] = 1;
                std::vector<int> next;
                uint32_t nrset;
                choose(dn, next, nrset);
                std::vector<char> is_later(gates.size(), 0);
                for (int i : later) is_later[i] = 1;
                bool acc = false;
                for (int i : next)
                    if (!is_later[i] && thread_factor(i, nrset)) acc = true;
                std::vector<int> moved;
                for (int i : later)
                    if (thread_factor(i, nrset)) moved.push_back(i);
                if (moved.size() * 16 > (acc ? 0u : 32u)) {
                    std::vector<char> is_moved(gates.size(), 0);
                    for (int i : moved) is_moved[i] = 1;
                    std::vector<int> m2;
                    for (int i : members)
                        if (!is_moved[i]) m2.push_back(i);
                    members.swap(m2);
                }
            }
        }
        // The phase's per-thread factors wait for the next phase when all of them
        // can: their qubits are thread bits there too (so they stay per-thread
        // factors), and this phase saves the complex multiply that applies them.
        {
            std::vector<int> fac, rest;
            for (int i : members) (thread_factor(i, rset) ? fac : rest).push_back(i);
            if (!fac.empty() && !rest.empty() && ndone + members.size() < gates.size()) {
                std::vector<char> dn = done;
                for (int i : rest) dn[i] = 1;
                std::vector<int> next;
                uint32_t nrset;
                choose(dn, next, nrset);
                std::vector<char> in_next(gates.size(), 0);
                for (int i : next) in_next[i] = 1;
                bool all = true;
                for (int i : fac) all = all && in_next[i] && thread_factor(i, nrset);
                if (all) members.swap(rest);
            }
        }

        OshmPhase ph;
        std::memset(&ph, 0, sizeof(ph));
        int r_local[OSHM_MAX_R];
        int nr = 0;
        r_local[nr++] = 0;
        for (int b = 1; b < k; b++)
            if ((rset >> b) & 1) r_local[nr++] = b;
        for (int j = 0; j < r; j++) ph.r_local[j] = (uint8_t)r_local[j];
        int reg_of_local[OSHM_MAX_K];
        for (int b = 0; b < k; b++) reg_of_local[b] = -1;
        for (int j = 0; j < r; j++) reg_of_local[r_local[j]] = j;

        // thread-index bits: the first three give conflict-free 16-byte smem
        // accesses within a quarter warp (distinct swizzle classes 1, 2, 3)
        std::vector<int> gfree;
        for (int b = 0; b < k; b++)
            if (!((rset >> b) & 1)) gfree.push_back(b);
        std::vector<int> order;
        auto take_class = [&](int cls) {
            for (size_t i = 0; i < gfree.size(); i++)
                if (slot_class(gfree[i]) == cls) {
                    order.push_back(gfree[i]);
                    gfree.erase(gfree.begin() + i);
                    return;
                }
        };
        take_class(1);
        take_class(2);
        take_class(3);
        for (int b : gfree) order.push_back(b);
        for (size_t j = 0; j < order.size(); j++) {
            ph.g_local[j] = (uint8_t)order[j];
            ph.g_phys[j] = (uint8_t)phys_of[order[j]];
        }

        ph.op_begin = (uint32_t)prog.ops.size();
        for (int i : members) {
            const hq_gate& g = gates[i];
            OshmOp o;
            std::memset(&o, 0, sizeof(o));
            for (int q = 0; q < 8; q++) o.m[q] = (float)g.mat[q];
            auto add_ctrl = [&](int c) {
                if (c < 0) return;
                const int lc = loc[c];
                if (lc >= 0 && reg_of_local[lc] >= 0)
                    o.creg |= 1u << reg_of_local[lc];
                else
                    o.cout |= uint64_t(1) << c;
            };
            add_ctrl(g.control);
            add_ctrl(g.control2);
            if (o.creg) o.flags |= OPF_CREG;
            if (o.cout) o.flags |= OPF_COUT;
            const int lt = loc[g.target];
            const int rt = lt >= 0 ? reg_of_local[lt] : -1;
            if (diag[i]) {
                double d0r = g.mat[0], d0i = g.mat[1], d1r = g.mat[6], d1i = g.mat[7];
                if (g.control < 0 && g.control2 < 0 && !(d0r == 1.0 && d0i == 0.0)) {
                    // diag(d0, d1) = d0 diag(1, d1 / d0): d0 multiplies the whole state
                    // and is applied once, at the end of the group
                    const std::complex<double> d0(d0r, d0i), q = std::complex<double>(d1r, d1i) / d0;
                    gfac *= d0;
                    d0r = 1.0;
                    d0i = 0.0;
                    d1r = snap(q.real());
                    d1i = snap(q.imag());
                    o.m[0] = 1.f;
                    o.m[1] = 0.f;
                    o.m[6] = (float)d1r;
                    o.m[7] = (float)d1i;
                }
                const bool d0one = d0r == 1.0 && d0i == 0.0;
                if (d0one) o.flags |= OPF_D0_ONE;
                if (d0one && d1r == 1.0 && d1i == 0.0) continue;  // identity
                if (rt >= 0) {
                    o.tbit = (uint8_t)rt;
                    o.kind = (d0one && d1r == -1.0 && d1i == 0.0) ? OP_NEGHI : OP_DREG;
                    if (o.kind == OP_DREG && d0one && rt >= 1 && o.creg == 0 &&
                        std::fabs(std::hypot(d1r, d1i) - 1.0) < 1e-12) {
                        o.kind = OP_DROT;
                        shear(std::atan2(d1i, d1r), o);
                    }
                } else {
                    o.kind = OP_DOUT;
                    o.tout = uint64_t(1) << g.target;
                    if (o.creg == 0) ph.flags |= PHF_ACC;
                }
            } else {
                o.tbit = (uint8_t)rt;
                const bool real = g.mat[1] == 0 && g.mat[3] == 0 && g.mat[5] == 0 && g.mat[7] == 0;
                const bool imoff = g.mat[1] == 0 && g.mat[7] == 0 && g.mat[2] == 0 && g.mat[4] == 0;
                const int had = hadamard_like(g);
                if (is_x_like(g)) {
                    o.kind = OP_X;
                } else if (o.creg == 0 && o.cout == 0 && had >= 0) {
                    o.kind = (uint8_t)had;  // runs without its 1/sqrt2: deferred
                    pending_scale *= rsqrt2;
                    pending_count++;
                } else if (rt >= 1 && o.creg == 0 && real && is_rotation(g)) {
                    o.kind = OP_RROT;  // three shears per plane instead of a 2x2 product
                    shear(std::atan2(g.mat[4], g.mat[0]), o);
                } else if (o.creg == 0 && real) {
                    o.kind = OP_REAL;
                } else if (o.creg == 0 && imoff) {
                    o.kind = OP_IMOFF;
                } else {
                    o.kind = OP_U;
                }
            }
            prog.ops.push_back(o);
        }
        for (int i : members) done[i] = 1;
        ndone += members.size();
        if (ndone == gates.size() && gfac != std::complex<double>(1.0, 0.0)) {
            // the factors taken out of diagonal gates, once, as a per-thread phase
            OshmOp o;
            std::memset(&o, 0, sizeof(o));
            o.kind = OP_DOUT;
            o.m[0] = o.m[6] = (float)gfac.real();
            o.m[1] = o.m[7] = (float)gfac.imag();
            prog.ops.push_back(o);
            ph.flags |= PHF_ACC;
        }
        ph.op_end = (uint32_t)prog.ops.size();
        // apply the deferred factors before they could leave FP32 range
        // (2^(count/2) growth), and always at the last phase
        const bool last = ndone == gates.size();
        ph.scale = 1.0f;
        if (pending_count > 0 && (last || pending_count >= 48)) {
            ph.scale = (float)pending_scale;
            pending_scale = 1.0;
            pending_count = 0;
        }
        prog.phases.push_back(ph);
    }
    return prog;
}

OshmLaunch make_oshm_launch(const OshmProgram& prog, void* state, const OshmPhase* d_phases,
                            const OshmOp* d_ops, int* d_err) {
    OshmLaunch p;
    std::memset(&p, 0, sizeof(p));
    const int n = prog.n, k = prog.k, r = prog.r;
    p.state = state;
    p.phases = d_phases;
    p.ops = d_ops;
    p.err = d_err;
    p.n = n;
    p.k = k;
    p.nphases = (int)prog.phases.size();
    p.ntiles = uint64_t(1) << (n - k);
    for (int b = 0, j = 0; b < n; b++)
        if ((prog.tile_mask >> b) & 1) p.tile_phys[j++] = (uint8_t)b;
    // runs of block bits: tile index bit i -> physical bit
    int src = 0, nruns = 0;
    for (int b = 0; b < n;) {
        if ((prog.tile_mask >> b) & 1) {
            b++;
            continue;
        }
        int len = 0;
        while (b + len < n && !((prog.tile_mask >> (b + len)) & 1)) len++;
        HQ_REQUIRE(nruns < 32, HQ_ERR_INVALID, "oshm: too many block-bit runs");
        p.run_src[nruns] = (uint8_t)src;
        p.run_dst[nruns] = (uint8_t)b;
        p.run_len[nruns] = (uint8_t)len;
        nruns++;
        src += len;
        b += len;
    }
    p.nruns = nruns;
    // pieces: thread t handles piece t + m*T (local index 2*(t + m*T))
    const int T = oshm_threads(k, r);
    const int ppt = (1 << (k - 1)) / T;
    HQ_REQUIRE(ppt <= 32, HQ_ERR_INVALID, "oshm: piece table");
    for (int m = 0; m < ppt; m++) {
        const uint32_t local = uint32_t(2 * m * T);
        uint64_t off = 0;
        for (int j = 0; j < k; j++)
            if ((local >> j) & 1) off |= uint64_t(1) << p.tile_phys[j];
        p.piece_off[m] = off;
        p.piece_slot[m] = oshm_swizzle(local);
    }
    return p;
}

// ---- GB300 cost model --------------------------------------------------------
// Seconds per pass over 2^n amplitudes: a pass costs its HBM floor (16 B per
// amplitude at the copy bandwidth) plus, for OShareMem, FP32 work per gate.
// The defaults are fitted to CUDA-event times of the kernels on a GB300
// (30-qubit grid circuit, 28-qubit QFT); hq_autotune measures them on the GPU
// at hand (autotune.cpp).  Replaces the reference's V100 tables and their
// calibrator (src/evaluator.h:18-127, src/evaluator.cpp:111-229,
// evaluator-preprocess/process.cpp:24-176).
namespace {
std::mutex g_cost_mu;
// fitted to 63 measured groups of seven 26-30 qubit circuits (grid, QFT,
// RY/RZ+CZ, U3+CNOT) on GB300 with the RING kernels
hq_cost_params g_cost = {2.5e-12, 6.2e-14, 4.1e-14, 4.2e-14,
                         5.4e-12, 4.6e-12, 1.5e-11, 1e-6};
}  // namespace

hq_cost_params cost_params() {
    std::lock_guard<std::mutex> lk(g_cost_mu);
    return g_cost;
}

void set_cost_params(const hq_cost_params& p) {
    const double v[] = {p.pass_floor, p.oshm_gate, p.oshm_diag, p.oshm_ctrl_diag,
                        p.mm_bf16x3,  p.mm_tf32,   p.mm_fp32,   p.launch};
    for (double x : v)
        HQ_REQUIRE(std::isfinite(x) && x >= 0.0 && x < 1.0, HQ_ERR_INVALID, "cost parameter %g out of range", x);
    std::lock_guard<std::mutex> lk(g_cost_mu);
    g_cost = p;
}

// A generated OShareMem kernel overlaps its tile loads and stores with the
// arithmetic (RING shape), so a group costs about the larger of its memory
// pass (pass_floor per amplitude) and its arithmetic (the gates' weights per
// amplitude); the two combine as sqrt(floor^2 + work^2), which follows the
// measured groups through the change-over between the two regimes.
double cost_oshm(int n, int nphases, const std::vector<hq_gate>& gates, int k) {
    (void)k;
    (void)nphases;
    const hq_cost_params c = cost_params();
    const double amps = double(uint64_t(1) << n);
    double w = 0;
    for (const auto& g : gates) {
        if (!matrix_is_diagonal(g))
            w += c.oshm_gate * oshm_gate_units(g);
        else
            w += g.control >= 0 ? c.oshm_ctrl_diag : c.oshm_diag;
    }
    return amps * std::hypot(c.pass_floor, w) + c.launch;
}

// Arithmetic of a non-diagonal gate in the register phases, in units of one
// packed add per amplitude (the sqrt(X) / sqrt(Y) / H gates): an exchange is
// register renaming, a real rotation three shears per plane, another real or
// imaginary-off-diagonal 2x2 one multiply and one fused multiply-add per
// component, a general complex 2x2 four.
double oshm_gate_units(const hq_gate& g) {
    if (is_x_like(g)) return 0.25;
    if (hadamard_like(g) >= 0) return 1.0;
    const bool real = g.mat[1] == 0 && g.mat[3] == 0 && g.mat[5] == 0 && g.mat[7] == 0;
    if (real && is_rotation(g)) return 1.5;
    const bool imoff = g.mat[1] == 0 && g.mat[7] == 0 && g.mat[2] == 0 && g.mat[4] == 0;
    return (real || imoff) ? 2.0 : 4.0;
}

double cost_transmm(int n, int m, int precision) {
    const hq_cost_params c = cost_params();
    const double amps = double(uint64_t(1) << n);
    double per = precision == HQ_MM_FP32 ? c.mm_fp32 : (precision == HQ_MM_TF32 ? c.mm_tf32 : c.mm_bf16x3);
    if (precision == HQ_MM_FP32 && m > 6) per *= double(1 << (m - 6));  // SIMT flops grow with 2^m
    // tensor cores: 6 and 7 qubits cost the same per pass; 8 streams its 512 KB
    // unitary through shared memory per tile (measured 3.1x the 7-qubit pass)
    if (precision != HQ_MM_FP32 && m > 7) per *= 3.1;
    return amps * per + c.launch;
}

}  // namespace hq
