// Patterns, DFS codes, rightmost extension and the minimum-DFS-code check.
//
// The mined pattern set is defined by three host algorithms of the reference, so they are kept
// alike step for step (their order of operations is the specification):
//   * Pattern::add_edge / buildRMPath / extend   (parallel/graph.h:919-980, serial/graph.h:782-860)
//   * GraMi::extend, the rightmost-path children (parallel/grami.h:172-294)
//   * GraMi::isCan + project_is_min              (parallel/grami.h:840-872, parallel/canonical.h)
// The canonical check reproduces the reference's ForwardEdge ordering (parallel/canonical.h:40-44),
// which is not a strict weak ordering once there is more than one edge label.  It feeds a
// std::map, so the same std::map operations are issued in the same sequence to obtain the same
// "smallest" forward extension; with one edge label the ordering is an ordinary label order.
// With that ordering libstdc++'s hinted insertion can overwrite a child link and orphan a subtree
// (the reference leaks those nodes); here every container of one check lives in a monotonic
// arena released when the check ends, which keeps the tree algorithm unchanged.
#pragma once

#include <algorithm>
#include <cstdint>
#include <map>
#include <memory_resource>
#include <set>
#include <string>
#include <tuple>
#include <vector>

namespace tfsm {

constexpr int kMaxPatternVertices = 32;  // parallel/global.h:36 (MAX_PATTERN_SIZE)

struct DfsCode {
    int from = 0, to = 0, from_label = 0, edge_label = 0, to_label = 0;
    bool operator==(const DfsCode &o) const {
        return from == o.from && to == o.to && from_label == o.from_label && edge_label == o.edge_label &&
               to_label == o.to_label;
    }
    bool operator!=(const DfsCode &o) const { return !(*this == o); }
    bool operator<(const DfsCode &o) const {
        if (from != o.from) return from < o.from;
        if (to != o.to) return to < o.to;
        if (from_label != o.from_label) return from_label < o.from_label;
        if (edge_label != o.edge_label) return edge_label < o.edge_label;
        return to_label < o.to_label;
    }
};

struct PEdge {
    int from, label, to, id;
};

struct PVertex {
    int label = 0;
    std::vector<PEdge> edges;  // ascending by `to`
};

// Insert keeping `edges` sorted by `to`, after any equal keys (Pattern::insert, parallel/graph.h:905).
inline void insert_sorted(std::vector<PEdge> &edges, const PEdge &e) {
    auto it = edges.begin();
    for (; it != edges.end(); ++it)
        if (it->to > e.to) break;
    edges.insert(it, e);
}

struct Pattern {
    std::vector<PVertex> vertices;
    std::vector<DfsCode> codes;
    std::vector<int> rmpath;  // indices into codes, rightmost edge first
    int n_edges = 0;

    int size() const { return (int)vertices.size(); }

    void add_edge(const DfsCode &c) {
        if (vertices.empty()) {
            vertices.resize(2);
            vertices[0].label = c.from_label;
            vertices[1].label = c.to_label;
            vertices[0].edges.push_back({0, c.edge_label, 1, 0});
            vertices[1].edges.push_back({1, c.edge_label, 0, 0});
            n_edges = 1;
            return;
        }
        if (!(c.from < size() && c.to < size())) {  // forward edge: a new vertex
            PVertex nv;
            nv.label = c.to_label;
            vertices.push_back(nv);
        }
        insert_sorted(vertices[c.from].edges, {c.from, c.edge_label, c.to, n_edges});
        insert_sorted(vertices[c.to].edges, {c.to, c.edge_label, c.from, n_edges});
        n_edges++;
    }

    void build_rmpath() {
        rmpath.clear();
        int prev = -1;
        for (int i = (int)codes.size(); i > 0; --i) {
            const DfsCode &c = codes[i - 1];
            if (c.from < c.to && (rmpath.empty() || prev == c.to)) {
                prev = c.from;
                rmpath.push_back(i - 1);
            }
        }
    }

    void push(const DfsCode &c) {
        add_edge(c);
        codes.push_back(c);
        build_rmpath();
    }

    static Pattern from_codes(const std::vector<DfsCode> &cs) {
        Pattern p;
        for (auto &c : cs) p.push(c);
        return p;
    }

    int label(int v) const { return vertices[v].label; }
    int degree(int v) const { return (int)vertices[v].edges.size(); }
    bool adjacent(int a, int b) const {
        for (auto &e : vertices[a].edges)
            if (e.to == b) return true;
        return false;
    }
    int edge_label(int a, int b) const {
        for (auto &e : vertices[a].edges)
            if (e.to == b) return e.label;
        return -1;
    }
    bool distinct_labels() const {
        std::set<int> s;
        for (auto &v : vertices)
            if (!s.insert(v.label).second) return false;
        return true;
    }
    bool acyclic() const { return n_edges == size() - 1; }  // connected by construction

    // "v id label" / "e from to elabel" block in DFS-code order (serial/grami.h:622-635).
    std::string to_results_block() const {
        std::string s = "=====================================\n";
        for (int i = 0; i < size(); ++i) s += "v " + std::to_string(i) + " " + std::to_string(label(i)) + "\n";
        for (auto &c : codes)
            s += "e " + std::to_string(c.from) + " " + std::to_string(c.to) + " " + std::to_string(c.edge_label) + "\n";
        return s;
    }
    // Compact key "from,to,fl,el,tl ..." used for set comparisons.
    std::string key() const {
        std::string s;
        for (size_t i = 0; i < codes.size(); ++i) {
            const DfsCode &c = codes[i];
            if (i) s += ' ';
            s += std::to_string(c.from) + "," + std::to_string(c.to) + "," + std::to_string(c.from_label) + "," +
                 std::to_string(c.edge_label) + "," + std::to_string(c.to_label);
        }
        return s;
    }
};

// ------------------------------------------------------------------------------------------
// Minimum DFS code check (parallel/canonical.h:1-346, parallel/grami.h:840-872)
// ------------------------------------------------------------------------------------------
namespace canon {

struct RootKey {
    int from_label, elabel, to_label;
    bool operator<(const RootKey &o) const {
        if (from_label != o.from_label) return from_label < o.from_label;
        if (elabel != o.elabel) return elabel < o.elabel;
        return to_label < o.to_label;
    }
};

// The reference's ForwardEdge ordering (canonical.h:40-44), kept as is: it decides which forward
// extension std::map::begin() yields when edge labels differ.
struct FwdKey {
    int elabel, to_label;
    bool operator<(const FwdKey &o) const {
        if (elabel < o.elabel) return true;
        return to_label < o.to_label;
    }
};

using Trans = std::pmr::vector<const PEdge *>;  // edges of one projection, in MIN code order
using ProjDB = std::pmr::vector<Trans>;

// root[k] of a map ordered by FwdKey, done as std::map::operator[] does it (lower_bound, then
// emplace_hint when the key is not found) so that the tree sees the same operations in the same
// order as the reference's map.  Because FwdKey is not a strict weak ordering, that sequence can
// end at end() (the hint step finds an "equal" key at the end): std::map::operator[] then hands out
// the map's header as if it were an element — undefined behaviour, in the reference's program too,
// whose push into it lands in the map object's own memory and is never seen again by begin().
// Here that case returns nullptr and the caller drops the projection: the defined form of what the
// reference observes, without writing outside the map.
inline ProjDB *fwd_slot(std::pmr::map<FwdKey, ProjDB> &root, const FwdKey &k) {
    auto it = root.lower_bound(k);
    if (it == root.end() || root.key_comp()(k, it->first))
        it = root.emplace_hint(it, std::piecewise_construct, std::forward_as_tuple(k), std::forward_as_tuple());
    return it == root.end() ? nullptr : &it->second;
}

struct History {
    std::vector<const PEdge *> edges;
    std::vector<char> has_edge, has_vertex;
    History(int n_vertices, int n_edges, const Trans &t)
        : edges(t.begin(), t.end()), has_edge((size_t)n_edges, 0), has_vertex((size_t)n_vertices, 0) {
        for (const PEdge *e : t) {
            has_edge[(size_t)e->id] = 1;
            has_vertex[(size_t)e->from] = 1;
            has_vertex[(size_t)e->to] = 1;
        }
    }
};

struct Checker {
    const Pattern &pat;      // the pattern whose code is checked
    const Pattern &g;        // the same pattern viewed as a graph (MIN_GRAPH)
    std::vector<DfsCode> min_codes;
    std::pmr::monotonic_buffer_resource arena;  // owns every map node and projection of the check

    explicit Checker(const Pattern &p) : pat(p), g(p) {}

    int lab(int v) const { return g.vertices[v].label; }

    const PEdge *get_backward(const PEdge *e1, const PEdge *e2, const History &h) const {
        if (e1 == e2) return nullptr;
        for (const PEdge &it : g.vertices[e2->to].edges) {
            if (h.has_edge[(size_t)it.id]) continue;
            if (it.to == e1->from &&
                (e1->label < it.label || (e1->label == it.label && lab(e1->to) <= lab(e2->to))))
                return &it;
        }
        return nullptr;
    }

    bool get_forward_pure(const PEdge *e, int minlabel, const History &h, std::vector<const PEdge *> &out) const {
        out.clear();
        for (const PEdge &it : g.vertices[e->to].edges) {
            if (minlabel > lab(it.to) || h.has_vertex[(size_t)it.to]) continue;
            out.push_back(&it);
        }
        return !out.empty();
    }

    bool get_forward_rmpath(const PEdge *e, int minlabel, const History &h, std::vector<const PEdge *> &out) const {
        out.clear();
        const int tolabel = lab(e->to);
        for (const PEdge &it : g.vertices[e->from].edges) {
            const int tolabel2 = lab(it.to);
            if (e->to == it.to || minlabel > tolabel2 || h.has_vertex[(size_t)it.to]) continue;
            if (e->label < it.label || (e->label == it.label && tolabel <= tolabel2)) out.push_back(&it);
        }
        return !out.empty();
    }

    static std::vector<int> rmpath_of(const std::vector<DfsCode> &codes) {
        std::vector<int> rm;
        int prev = -1;
        for (int i = (int)codes.size(); i > 0; --i) {
            const DfsCode &c = codes[i - 1];
            if (c.from < c.to && (rm.empty() || prev == c.to)) {
                prev = c.from;
                rm.push_back(i - 1);
            }
        }
        return rm;
    }

    bool project_is_min(const ProjDB &projected) {
        const std::vector<int> rmpath = rmpath_of(min_codes);
        const int minlabel = min_codes[0].from_label;
        const int maxtoc = min_codes[(size_t)rmpath[0]].to;
        const int nv = g.size(), ne = g.n_edges;

        // backward extensions from the rightmost vertex
        {
            std::pmr::map<int, ProjDB> root(&arena);
            bool flg = false;
            int new_to = 0, new_tolabel = 0;
            // `i` is unsigned in the reference: with a single-edge rightmost path the loop is empty.
            for (size_t i = rmpath.size() - 1; !flg && i >= 1 && rmpath.size() >= 2; --i) {
                for (const Trans &cur : projected) {
                    History h(nv, ne, cur);
                    const PEdge *e = get_backward(h.edges[(size_t)rmpath[i]], h.edges[(size_t)rmpath[0]], h);
                    if (e) {
                        Trans t(cur, &arena);
                        t.push_back(e);
                        root[e->label].push_back(std::move(t));
                        new_to = min_codes[(size_t)rmpath[i]].from;
                        new_tolabel = min_codes[(size_t)rmpath[i]].from_label;
                        flg = true;
                    }
                }
            }
            if (flg) {
                auto to = root.begin();
                DfsCode c;
                c.from = maxtoc;
                c.to = new_to;
                c.from_label = min_codes[(size_t)rmpath[0]].to_label;
                c.edge_label = to->first;
                c.to_label = new_tolabel;
                min_codes.push_back(c);
                if (pat.codes[min_codes.size() - 1] != min_codes.back()) return false;
                ProjDB next = std::move(to->second);
                return project_is_min(next);
            }
        }
        // forward extensions
        {
            bool flg = false;
            int new_from = 0, new_fromlabel = 0;
            std::pmr::map<FwdKey, ProjDB> root(&arena);
            std::vector<const PEdge *> edges;
            for (const Trans &cur : projected) {
                History h(nv, ne, cur);
                if (get_forward_pure(h.edges[(size_t)rmpath[0]], minlabel, h, edges)) {
                    flg = true;
                    for (const PEdge *it : edges) {
                        FwdKey k{it->label, lab(it->to)};
                        new_from = maxtoc;
                        new_fromlabel = lab(it->from);
                        Trans t(cur, &arena);
                        t.push_back(it);
                        if (ProjDB *db = fwd_slot(root, k)) db->push_back(std::move(t));
                    }
                }
            }
            for (size_t i = 0; !flg && i < rmpath.size(); ++i) {
                for (const Trans &cur : projected) {
                    History h(nv, ne, cur);
                    if (get_forward_rmpath(h.edges[(size_t)rmpath[i]], minlabel, h, edges)) {
                        flg = true;
                        for (const PEdge *it : edges) {
                            FwdKey k{it->label, lab(it->to)};
                            new_from = min_codes[(size_t)rmpath[i]].from;
                            new_fromlabel = lab(it->from);
                            Trans t(cur, &arena);
                            t.push_back(it);
                            if (ProjDB *db = fwd_slot(root, k)) db->push_back(std::move(t));
                        }
                    }
                }
            }
            if (flg) {
                auto from = root.begin();
                DfsCode c;
                c.from = new_from;
                c.to = maxtoc + 1;
                c.from_label = new_fromlabel;
                c.edge_label = from->first.elabel;
                c.to_label = from->first.to_label;
                min_codes.push_back(c);
                if (pat.codes[min_codes.size() - 1] != min_codes.back()) return false;
                ProjDB next = std::move(from->second);
                return project_is_min(next);
            }
        }
        return true;
    }

    bool run() {
        if (pat.codes.size() == 1) return true;
        std::pmr::map<RootKey, ProjDB> root(&arena);
        for (int from = 0; from < g.size(); ++from) {
            const PVertex &v = g.vertices[from];
            for (const PEdge &e : v.edges) {
                if (v.label <= lab(e.to)) {
                    RootKey k{v.label, e.label, lab(e.to)};
                    Trans t(&arena);
                    t.push_back(&e);
                    root[k].push_back(std::move(t));
                }
            }
        }
        auto first = root.begin();
        DfsCode c;
        c.from = 0;
        c.to = 1;
        c.from_label = first->first.from_label;
        c.edge_label = first->first.elabel;
        c.to_label = first->first.to_label;
        min_codes.assign(1, c);
        return project_is_min(first->second);
    }
};

}  // namespace canon

inline bool is_canonical(const Pattern &p) {
    canon::Checker ck(p);
    return ck.run();
}

// ------------------------------------------------------------------------------------------
// Rightmost extension (parallel/grami.h:172-294).  `neighbor_labels[l]` holds the labels that
// form a frequent 1-edge pattern with l; `freq_elabels` are the frequent edge labels.
// Children that fail the canonical check are dropped, as the parallel build does.
// ------------------------------------------------------------------------------------------
struct ExtendContext {
    std::map<int, std::set<int>> neighbor_labels;
    std::vector<int> freq_elabels;
    int max_nodes = -1;  // -1: unbounded
    const std::set<int> &nbrs(int l) const {
        static const std::set<int> empty;
        auto it = neighbor_labels.find(l);
        return it == neighbor_labels.end() ? empty : it->second;
    }
};

inline void extend_pattern(const Pattern &p, const ExtendContext &ctx, std::vector<Pattern> &out,
                           bool check_canonical = true) {
    const int last_id = p.size() - 1;
    const int last_label = p.label(last_id);
    const int min_label = p.codes[0].from_label;
    auto emit = [&](const DfsCode &c) {
        Pattern child = p;
        child.push(c);
        if (!check_canonical || is_canonical(child)) out.push_back(std::move(child));
    };
    // unbounded growth stops at the reference's MAX_PATTERN_SIZE
    const bool grow = (ctx.max_nodes == -1 || p.size() < ctx.max_nodes) && p.size() < kMaxPatternVertices;
    // forward from the rightmost vertex
    if (grow) {
        for (int nl : ctx.nbrs(last_label))
            for (int el : ctx.freq_elabels)
                if (nl >= min_label) emit(DfsCode{last_id, last_id + 1, last_label, el, nl});
    }
    // backward from the rightmost vertex to rightmost-path vertices (not its parent)
    for (size_t i = p.rmpath.size(); i > 1; --i) {
        const DfsCode &rc = p.codes[(size_t)p.rmpath[i - 1]];
        const int cur_id = rc.from;
        const int cur_label = p.label(cur_id);
        if (!ctx.nbrs(last_label).count(cur_label)) continue;
        if (p.adjacent(last_id, cur_id)) continue;
        for (int el : ctx.freq_elabels)
            if (el > rc.edge_label || (el == rc.edge_label && last_label >= rc.to_label))
                emit(DfsCode{last_id, cur_id, last_label, el, cur_label});
    }
    // forward from every rightmost-path vertex
    if (grow) {
        for (size_t i = 0; i < p.rmpath.size(); ++i) {
            const DfsCode &rc = p.codes[(size_t)p.rmpath[i]];
            const int cur_id = rc.from;
            const int cur_label = p.label(cur_id);
            for (int nl : ctx.nbrs(cur_label))
                for (int el : ctx.freq_elabels)
                    if (rc.edge_label < el || (rc.edge_label == el && rc.to_label <= nl))
                        emit(DfsCode{cur_id, last_id + 1, cur_label, el, nl});
        }
    }
}

// Automorphism orbits of a pattern (label- and edge-label-preserving permutations), used to
// share MNI domains between equivalent pattern vertices as serial/grami.h:379-392 does.
inline std::vector<int> automorphism_orbits(const Pattern &p) {
    const int n = p.size();
    std::vector<int> orbit(n);
    for (int i = 0; i < n; ++i) orbit[i] = i;
    std::vector<int> map(n, -1), used(n, 0);
    // union-find over images
    std::vector<int> parent(n);
    for (int i = 0; i < n; ++i) parent[i] = i;
    auto find = [&](int x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    auto unite = [&](int a, int b) {
        a = find(a);
        b = find(b);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
    };
    // search limited to a fixed number of nodes; patterns here have few vertices.
    long budget = 2000000;
    std::vector<int> images_found(n * n, 0);
    auto rec = [&](auto &&self, int d) -> void {
        if (--budget < 0) return;
        if (d == n) {
            for (int i = 0; i < n; ++i) unite(i, map[i]);
            return;
        }
        for (int c = 0; c < n; ++c) {
            if (used[c] || p.label(c) != p.label(d) || p.degree(c) != p.degree(d)) continue;
            bool ok = true;
            for (const PEdge &e : p.vertices[d].edges) {
                if (e.to < d) {
                    if (p.edge_label(c, map[e.to]) != e.label) {
                        ok = false;
                        break;
                    }
                }
            }
            if (!ok) continue;
            used[c] = 1;
            map[d] = c;
            self(self, d + 1);
            used[c] = 0;
            map[d] = -1;
        }
    };
    rec(rec, 0);
    if (budget < 0) {  // give up sharing: every vertex is its own orbit
        for (int i = 0; i < n; ++i) orbit[i] = i;
        return orbit;
    }
    for (int i = 0; i < n; ++i) orbit[i] = find(i);
    return orbit;
}

}  // namespace tfsm
