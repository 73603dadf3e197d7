// Sub-pattern (Apriori) pruning for the miner.
//
// MNI support is anti-monotone: an embedding of a pattern P contains an embedding of every
// connected sub-pattern S of P, with the vertices of S mapped to the same data vertices, so
// MNI(P) <= MNI(S).  Rightmost extension with the canonical check generates every frequent pattern
// exactly once, level by level, so when one of P's connected sub-patterns with one edge less is not
// among the previous level's frequent patterns, P is infrequent and needs no search (the miner
// applies this only with a single frequent edge label: with several, the reference's canonical
// check does not generate every frequent pattern, see miner.cpp).  The
// reference reaches the same decision through its search and its push-down cache of per-vertex
// non-candidates (parallel/decompose.h, parallel/comper.h:1582-1612); the mined set is unchanged.
//
// Sub-patterns are matched by an isomorphism-invariant key: vertices are ordered by an invariant
// (label, degree, sorted (edge label, neighbour label) pairs), every ordering that keeps that
// order is tried, and the smallest edge list wins.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "pattern.hpp"

namespace tfsm {

struct SmallGraph {
    std::vector<int> label;                 // by vertex
    std::vector<std::array<int, 3>> edges;  // (a, b, edge label)
};

// Orderings a canonical key may try; a graph that needs more gets no key (see canonical_key).
constexpr uint64_t kMaxKeyOrderings = 50000;

// Isomorphism-invariant key (bytes of int32 values).  Vertices are ranked by an invariant
// (label, degree, sorted (edge label, neighbour label) pairs), the ranks are refined by the ranks
// of the neighbours until stable (colour refinement: ranks are assigned by sorting signatures, so
// isomorphic graphs get the same ranks), every ordering that keeps the rank order is tried, and the
// smallest edge list wins.  With `order`, also the vertex at each position of the canonical form:
// for two isomorphic graphs, order_a[i] <-> order_b[i] is an isomorphism.  A graph whose classes
// of equal rank allow more than kMaxKeyOrderings orderings (long symmetric paths or cycles) gets
// the empty key, which callers treat as unknown; whether a graph gets one depends only on its
// isomorphism class.
inline std::string canonical_key(const SmallGraph &g, std::vector<int> *order_out = nullptr) {
    const int n = (int)g.label.size();
    std::vector<std::vector<int>> inv((size_t)n);
    for (int v = 0; v < n; ++v) inv[(size_t)v] = {g.label[(size_t)v], 0};
    for (auto &e : g.edges) {
        inv[(size_t)e[0]][1]++;
        inv[(size_t)e[1]][1]++;
    }
    std::vector<std::vector<std::pair<int, int>>> nb((size_t)n);
    for (auto &e : g.edges) {
        nb[(size_t)e[0]].push_back({e[2], g.label[(size_t)e[1]]});
        nb[(size_t)e[1]].push_back({e[2], g.label[(size_t)e[0]]});
    }
    for (int v = 0; v < n; ++v) {
        std::sort(nb[(size_t)v].begin(), nb[(size_t)v].end());
        for (auto &p : nb[(size_t)v]) {
            inv[(size_t)v].push_back(p.first);
            inv[(size_t)v].push_back(p.second);
        }
    }
    // initial ranks from the invariants, then refinement by (rank, sorted (edge label, neighbour rank))
    std::vector<int> rank((size_t)n);
    auto rank_by = [&](const std::vector<std::vector<int>> &sig) {
        std::vector<int> idx((size_t)n);
        for (int v = 0; v < n; ++v) idx[(size_t)v] = v;
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return sig[(size_t)a] < sig[(size_t)b]; });
        int r = 0;
        for (int i = 0; i < n; ++i) {
            if (i > 0 && sig[(size_t)idx[(size_t)i]] != sig[(size_t)idx[(size_t)i - 1]]) ++r;
            rank[(size_t)idx[(size_t)i]] = r;
        }
        return n ? r + 1 : 0;
    };
    int classes = rank_by(inv);
    std::vector<std::vector<std::array<int, 2>>> adj((size_t)n);
    for (auto &e : g.edges) {
        adj[(size_t)e[0]].push_back({e[2], e[1]});
        adj[(size_t)e[1]].push_back({e[2], e[0]});
    }
    for (int round = 0; round < n; ++round) {
        std::vector<std::vector<int>> sig((size_t)n);
        for (int v = 0; v < n; ++v) {
            std::vector<std::pair<int, int>> ns;
            for (auto &a : adj[(size_t)v]) ns.push_back({a[0], rank[(size_t)a[1]]});
            std::sort(ns.begin(), ns.end());
            sig[(size_t)v].push_back(rank[(size_t)v]);
            for (auto &x : ns) {
                sig[(size_t)v].push_back(x.first);
                sig[(size_t)v].push_back(x.second);
            }
        }
        const int before = classes;
        classes = rank_by(sig);
        if (classes == before) break;
    }
    std::vector<int> order((size_t)n);
    for (int v = 0; v < n; ++v) order[(size_t)v] = v;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rank[(size_t)a] < rank[(size_t)b]; });
    // classes of equal rank: [begin, end) ranges of `order` (ascending vertex ids inside)
    std::vector<std::pair<int, int>> cls;
    uint64_t orderings = 1;
    for (int i = 0; i < n;) {
        int j = i + 1;
        while (j < n && rank[(size_t)order[(size_t)j]] == rank[(size_t)order[(size_t)i]]) ++j;
        cls.push_back({i, j});
        for (int f = 2; f <= j - i && orderings <= kMaxKeyOrderings; ++f) orderings *= (uint64_t)f;
        i = j;
    }
    if (orderings > kMaxKeyOrderings) {
        if (order_out) order_out->clear();
        return std::string();
    }
    std::vector<int> pos((size_t)n);
    std::vector<std::array<int, 3>> cur, best;
    bool have = false;
    for (;;) {
        for (int i = 0; i < n; ++i) pos[(size_t)order[(size_t)i]] = i;
        cur.clear();
        for (auto &e : g.edges) {
            const int a = pos[(size_t)e[0]], b = pos[(size_t)e[1]];
            cur.push_back({std::min(a, b), std::max(a, b), e[2]});
        }
        std::sort(cur.begin(), cur.end());
        if (!have || cur < best) {
            best = cur;
            have = true;
            if (order_out) *order_out = order;
        }
        // next ordering: odometer over the classes' permutations
        size_t k = 0;
        for (; k < cls.size(); ++k) {
            auto b = order.begin() + cls[k].first, e = order.begin() + cls[k].second;
            if (std::next_permutation(b, e)) break;  // wrapped classes are back in ascending order
        }
        if (k == cls.size()) break;
    }
    std::vector<int32_t> key;
    key.push_back(n);
    for (int i = 0; i < n; ++i)
        for (int x : inv[(size_t)order[(size_t)i]]) key.push_back(x);  // classes are in sorted order again
    key.push_back(-1);
    for (auto &e : best) key.insert(key.end(), {e[0], e[1], e[2]});
    return std::string(reinterpret_cast<const char *>(key.data()), key.size() * sizeof(int32_t));
}

inline SmallGraph small_graph(const Pattern &p) {
    SmallGraph g;
    for (auto &v : p.vertices) g.label.push_back(v.label);
    for (auto &c : p.codes) g.edges.push_back({c.from, c.to, c.edge_label});
    return g;
}

// A connected sub-pattern of P with one edge less: its key and, for every vertex of P, the
// position of its image in the sub-pattern's canonical order (-1 for the dropped vertex; all -1
// when the key is unknown, i.e. empty).
struct SubPattern {
    std::string key;
    std::vector<int> pos_of;  // by P vertex
};

// P's connected sub-patterns with one edge less (an edge to a degree-1 vertex goes with that
// vertex; an edge whose removal disconnects the rest gives no connected sub-pattern).
inline void one_edge_smaller(const Pattern &p, std::vector<SubPattern> &subs) {
    subs.clear();
    const SmallGraph g = small_graph(p);
    const int n = (int)g.label.size(), m = (int)g.edges.size();
    if (m < 2) return;
    std::vector<int> deg((size_t)n, 0);
    for (auto &e : g.edges) {
        deg[(size_t)e[0]]++;
        deg[(size_t)e[1]]++;
    }
    for (int i = 0; i < m; ++i) {
        const int a = g.edges[(size_t)i][0], b = g.edges[(size_t)i][1];
        int drop = -1;
        if (deg[(size_t)a] == 1) drop = a;
        else if (deg[(size_t)b] == 1) drop = b;
        SmallGraph s;
        std::vector<int> remap((size_t)n, -1);
        for (int v = 0; v < n; ++v)
            if (v != drop) {
                remap[(size_t)v] = (int)s.label.size();
                s.label.push_back(g.label[(size_t)v]);
            }
        for (int j = 0; j < m; ++j)
            if (j != i)
                s.edges.push_back({remap[(size_t)g.edges[(size_t)j][0]], remap[(size_t)g.edges[(size_t)j][1]],
                                   g.edges[(size_t)j][2]});
        // connected?
        const int ns = (int)s.label.size();
        std::vector<int> comp((size_t)ns);
        for (int v = 0; v < ns; ++v) comp[(size_t)v] = v;
        auto find = [&](int x) {
            while (comp[(size_t)x] != x) x = comp[(size_t)x] = comp[(size_t)comp[(size_t)x]];
            return x;
        };
        for (auto &e : s.edges) comp[(size_t)find(e[0])] = find(e[1]);
        bool connected = true;
        for (int v = 1; v < ns && connected; ++v) connected = find(v) == find(0);
        if (!connected) continue;
        SubPattern sp;
        std::vector<int> order;
        sp.key = canonical_key(s, &order);
        sp.pos_of.assign((size_t)n, -1);
        if (!sp.key.empty()) {
            std::vector<int> pos_in_s((size_t)ns);
            for (int i = 0; i < ns; ++i) pos_in_s[(size_t)order[(size_t)i]] = i;
            for (int v = 0; v < n; ++v)
                if (remap[(size_t)v] >= 0) sp.pos_of[(size_t)v] = pos_in_s[(size_t)remap[(size_t)v]];
        }
        subs.push_back(std::move(sp));
    }
}

inline void one_edge_smaller_keys(const Pattern &p, std::vector<std::string> &keys) {
    std::vector<SubPattern> subs;
    one_edge_smaller(p, subs);
    keys.clear();
    for (auto &s : subs) keys.push_back(std::move(s.key));
}

}  // namespace tfsm
