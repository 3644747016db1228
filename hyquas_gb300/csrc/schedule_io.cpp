// Compiled-schedule serialisation.
//
// The reference turns its compiled Schedule into bytes so that rank 0 can
// broadcast it (Schedule / LocalGroup / GateGroup / State::serialize,
// src/schedule.cpp:156-325; Gate::serialize, src/gate.cpp:558-589).  Here the
// bytes hold everything compile decided on the host -- the options, the gate
// list, the SWAP-folded list with its index map and permutation, and the
// partition (per group: backend, width, related qubits, layouts and gate
// indices) -- so that a process which loads them skips the partitioner and
// only lowers and uploads the groups (generated kernels come from the
// source-keyed kernel cache when the process has built them before).
//
// Layout, little-endian, fixed-width fields:
//   "HQSC" u32 version
//   i32 n, 7 x i32 compile options
//   u32 count + gates            (gate = 4 x i32 type target control control2, 8 x f64 mat)
//   u32 count + folded gates
//   u32 count + i32 orig_index, u32 count + i32 swap_perm
//   u32 groups; per group i32 backend, i32 width, u64 related,
//       u32 count + i32 gate indices, u32 count + i32 pos, u32 count + i32 pos_after
//   u32 count + i32 final_pos
//   u64 FNV-1a of all the bytes before it
// Loading checks the magic, version, checksum, every size and index, and the
// gates themselves; lowering then re-checks each group against its tile.
#include <cstring>

#include "common.h"
#include "executor.h"
#include "gates.h"

namespace hq {

namespace {

constexpr uint32_t kVersion = 1;
constexpr int kMaxQubits = 36;

uint64_t fnv1a(const uint8_t* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

struct Writer {
    std::vector<uint8_t> b;
    template <class T>
    void put(T v) {
        uint8_t tmp[sizeof(T)];
        std::memcpy(tmp, &v, sizeof(T));
        b.insert(b.end(), tmp, tmp + sizeof(T));
    }
    void gate(const hq_gate& g) {
        put<int32_t>(g.type);
        put<int32_t>(g.target);
        put<int32_t>(g.control);
        put<int32_t>(g.control2);
        for (double m : g.mat) put<double>(m);
    }
    void ints(const std::vector<int>& v) {
        put<uint32_t>((uint32_t)v.size());
        for (int x : v) put<int32_t>(x);
    }
};

struct Reader {
    const uint8_t* p;
    size_t n, at = 0;
    template <class T>
    T get() {
        HQ_REQUIRE(n - at >= sizeof(T), HQ_ERR_INVALID, "schedule bytes: truncated at offset %zu", at);
        T v;
        std::memcpy(&v, p + at, sizeof(T));
        at += sizeof(T);
        return v;
    }
    uint32_t count(size_t max, const char* what) {
        const uint32_t c = get<uint32_t>();
        HQ_REQUIRE(c <= max, HQ_ERR_INVALID, "schedule bytes: %s count %u exceeds %zu", what, c, max);
        return c;
    }
    hq_gate gate() {
        hq_gate g;
        g.type = get<int32_t>();
        g.target = get<int32_t>();
        g.control = get<int32_t>();
        g.control2 = get<int32_t>();
        for (double& m : g.mat) m = get<double>();
        return g;
    }
    std::vector<int> ints(size_t max, const char* what) {
        const uint32_t c = count(max, what);
        std::vector<int> v(c);
        for (auto& x : v) x = get<int32_t>();
        return v;
    }
};

void require_perm(const std::vector<int>& v, int n, const char* what) {
    HQ_REQUIRE((int)v.size() == n, HQ_ERR_INVALID, "schedule bytes: %s has %zu entries, not %d", what,
               v.size(), n);
    std::vector<char> seen(n, 0);
    for (int x : v) {
        HQ_REQUIRE(x >= 0 && x < n && !seen[x], HQ_ERR_INVALID, "schedule bytes: %s is not a permutation",
                   what);
        seen[x] = 1;
    }
}

}  // namespace

std::vector<uint8_t> schedule_serialize(const hq_circuit_s* c) {
    HQ_REQUIRE(c->compiled, HQ_ERR_STATE, "circuit not compiled");
    Writer w;
    w.b.insert(w.b.end(), {'H', 'Q', 'S', 'C'});
    w.put<uint32_t>(kVersion);
    w.put<int32_t>(c->n);
    const hq_compile_options& o = c->opt;
    for (int32_t v : {o.backend, o.tile_qubits, o.coalesce, o.mm_qubits, o.mm_precision,
                      o.reference_grouping, o.specialize})
        w.put<int32_t>(v);
    w.put<uint32_t>((uint32_t)c->gates.size());
    for (const hq_gate& g : c->gates) w.gate(g);
    w.put<uint32_t>((uint32_t)c->folded.size());
    for (const hq_gate& g : c->folded) w.gate(g);
    w.ints(c->orig_index);
    w.ints(c->swap_perm);
    w.put<uint32_t>((uint32_t)c->part.groups.size());
    for (const GroupPlan& gp : c->part.groups) {
        w.put<int32_t>(gp.backend);
        w.put<int32_t>(gp.width);
        w.put<uint64_t>(gp.related);
        w.ints(gp.gates);
        w.ints(gp.pos);
        w.ints(gp.pos_after);
    }
    w.ints(c->part.final_pos);
    w.put<uint64_t>(fnv1a(w.b.data(), w.b.size()));
    return w.b;
}

void schedule_deserialize(const uint8_t* buf, size_t len, hq_circuit_s* c) {
    HQ_REQUIRE(buf != nullptr || len == 0, HQ_ERR_INVALID, "schedule bytes: null buffer");
    HQ_REQUIRE(len >= 16 && std::memcmp(buf, "HQSC", 4) == 0, HQ_ERR_INVALID,
               "schedule bytes: not a serialised schedule");
    uint64_t stored;
    std::memcpy(&stored, buf + len - 8, 8);
    HQ_REQUIRE(stored == fnv1a(buf, len - 8), HQ_ERR_INVALID, "schedule bytes: checksum mismatch");
    Reader r{buf, len - 8};
    r.at = 4;
    const uint32_t version = r.get<uint32_t>();
    HQ_REQUIRE(version == kVersion, HQ_ERR_UNSUPPORTED, "schedule bytes: version %u (this build reads %u)",
               version, kVersion);
    const int n = r.get<int32_t>();
    HQ_REQUIRE(n >= 1 && n <= kMaxQubits, HQ_ERR_INVALID, "schedule bytes: %d qubits", n);
    hq_compile_options o;
    o.backend = r.get<int32_t>();
    o.tile_qubits = r.get<int32_t>();
    o.coalesce = r.get<int32_t>();
    o.mm_qubits = r.get<int32_t>();
    o.mm_precision = r.get<int32_t>();
    o.reference_grouping = r.get<int32_t>();
    o.specialize = r.get<int32_t>();
    HQ_REQUIRE(o.specialize >= 0 && o.specialize <= 3, HQ_ERR_INVALID, "schedule bytes: specialize %d",
               o.specialize);
    config_from_options(o, n);  // checks the options
    const size_t max_gates = (len - r.at) / (16 + 64);
    std::vector<hq_gate> gates(r.count(max_gates, "gate"));
    for (auto& g : gates) {
        g = r.gate();
        validate_gate(g, n);
    }
    std::vector<hq_gate> folded(r.count(gates.size(), "folded gate"));
    for (auto& g : folded) {
        g = r.gate();
        validate_gate(g, n);
        HQ_REQUIRE(g.type != G_SWAP, HQ_ERR_INVALID, "schedule bytes: SWAP in the folded gate list");
    }
    std::vector<int> orig = r.ints(folded.size(), "index map");
    HQ_REQUIRE(orig.size() == folded.size(), HQ_ERR_INVALID, "schedule bytes: index map size");
    for (int x : orig)
        HQ_REQUIRE(x >= 0 && (size_t)x < gates.size(), HQ_ERR_INVALID, "schedule bytes: index map entry %d",
                   x);
    std::vector<int> perm = r.ints(kMaxQubits, "permutation");
    require_perm(perm, n, "SWAP permutation");
    Partition part;
    const uint32_t ng = r.count(folded.size() + 1, "group");
    std::vector<char> used(folded.size(), 0);
    for (uint32_t g = 0; g < ng; g++) {
        GroupPlan gp;
        gp.backend = r.get<int32_t>();
        gp.width = r.get<int32_t>();
        gp.related = r.get<uint64_t>();
        HQ_REQUIRE(gp.backend == HQ_BACKEND_OSHM || gp.backend == HQ_BACKEND_TRANSMM, HQ_ERR_INVALID,
                   "schedule bytes: group %u backend %d", g, gp.backend);
        HQ_REQUIRE(gp.width >= 1 && gp.width <= std::min(n, OSHM_MAX_K), HQ_ERR_INVALID,
                   "schedule bytes: group %u width %d", g, gp.width);
        HQ_REQUIRE(n == 64 || (gp.related >> n) == 0, HQ_ERR_INVALID,
                   "schedule bytes: group %u related qubits outside the register", g);
        gp.gates = r.ints(folded.size(), "group gate");
        for (int x : gp.gates) {
            HQ_REQUIRE(x >= 0 && (size_t)x < folded.size() && !used[x], HQ_ERR_INVALID,
                       "schedule bytes: group %u gate index %d", g, x);
            used[x] = 1;
        }
        gp.pos = r.ints(kMaxQubits, "layout");
        gp.pos_after = r.ints(kMaxQubits, "layout");
        require_perm(gp.pos, n, "group layout");
        require_perm(gp.pos_after, n, "group layout");
        part.groups.push_back(std::move(gp));
    }
    part.final_pos = r.ints(kMaxQubits, "final layout");
    require_perm(part.final_pos, n, "final layout");
    HQ_REQUIRE(r.at == r.n, HQ_ERR_INVALID, "schedule bytes: %zu trailing bytes", r.n - r.at);
    const bool grouped = !(o.backend == HQ_BACKEND_PLAIN || n < 6);
    for (size_t x = 0; x < used.size() && grouped; x++)
        HQ_REQUIRE(used[x], HQ_ERR_INVALID, "schedule bytes: folded gate %zu in no group", x);
    HQ_REQUIRE(grouped || ng == 0, HQ_ERR_INVALID, "schedule bytes: groups for a gate-by-gate circuit");

    c->n = n;
    c->opt = o;
    c->gates = std::move(gates);
    c->folded = std::move(folded);
    c->orig_index = std::move(orig);
    c->swap_perm = std::move(perm);
    c->part = std::move(part);
}

}  // namespace hq
