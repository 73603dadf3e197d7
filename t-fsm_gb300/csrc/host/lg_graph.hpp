// Host-side `.lg` loader with the reference's label pruning and id remapping.
//
// Semantics follow the reference loader exactly, because the mined pattern set depends on them:
//   * serial/graph.h:485-494, parallel/graph.h:557-570 (load_graph): read, count labels, prune;
//   * parallel/graph.h:603-660 (construct_graph): edge-label frequency counts every input edge;
//   * parallel/graph.h:662-683 (find_frequent_labels): a vertex label is frequent when at least tau
//     vertices carry it; an edge label when at least tau edges carry it (freq/2 >= tau, where freq
//     counts both directions);
//   * parallel/graph.h:685-803 (construct_freq_graph): vertices with frequent labels get new ids in
//     the order of their `v` lines; an edge survives when both end labels and its edge label are
//     frequent; adjacency is sorted by neighbour id; the 1-edge pattern table ("hashedEdges") keeps
//     a (min label, edge label, max label) triple only when both endpoint sets have >= tau vertices.
//
// The loader is plain C++17 (no intrinsics) and is shared by the miner, the C-ABI and the CPU
// checker.  Errors never exit the process: they are reported through LgError.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace tfsm {

struct LgError : std::runtime_error {
    int code;
    LgError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// A frequent 1-edge pattern (min label, edge label, max label) with its two endpoint-set sizes.
struct EdgePair {
    int la, el, lb;
    uint32_t cand_a, cand_b;
};

struct LgGraph {
    // ---- pruned graph, vertex ids in the reference's pruned order ----
    uint32_t n = 0;                  // vertices after pruning
    uint64_t m = 0;                  // undirected edges after pruning
    std::vector<int> vlabel;         // [n]
    std::vector<uint64_t> offs;      // [n+1] CSR offsets into nbr / elab
    std::vector<uint32_t> nbr;       // [2m] neighbour ids, ascending per vertex
    std::vector<int> elab;           // [2m] edge labels
    std::vector<int> freq_vlabels;   // ascending
    std::vector<int> freq_elabels;   // ascending
    std::vector<EdgePair> edge_pairs;  // frequent 1-edge patterns, ascending (la, el, lb)
    uint32_t max_label_freq = 0;     // largest label class after pruning
    uint32_t max_degree = 0;         // largest degree after pruning
    // ---- input statistics ----
    uint64_t input_vertices = 0, input_edges = 0;

    uint32_t degree(uint32_t v) const { return (uint32_t)(offs[v + 1] - offs[v]); }
};

namespace detail {

inline bool read_file(const std::string &path, std::vector<char> &buf) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize((size_t)sz + 1);
    size_t got = sz > 0 ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
    std::fclose(f);
    buf.resize(got);
    buf.push_back('\n');
    return true;
}

// atoi-like parse of one space-separated token (the reference tokenises on ' ' and uses atoi).
inline long parse_int(const char *&p, const char *end, bool &ok) {
    while (p < end && *p == ' ') ++p;
    if (p >= end || *p == '\n') {
        ok = false;
        return 0;
    }
    const char *tok = p;
    while (p < end && *p != ' ' && *p != '\n') ++p;
    ok = true;
    return std::strtol(tok, nullptr, 10);
}

}  // namespace detail

struct RawLg {
    std::vector<int> vlabel;                           // by input id
    std::vector<std::tuple<uint32_t, uint32_t, int>> edges;  // (a, b, label) in file order
};

inline RawLg parse_lg_text(const char *data, size_t size) {
    RawLg raw;
    const char *p = data, *end = data + size;
    size_t line_no = 0;
    std::vector<std::pair<long, int>> vlines;
    while (p < end) {
        const char *line_end = (const char *)std::memchr(p, '\n', (size_t)(end - p));
        if (!line_end) line_end = end;
        ++line_no;
        const char *q = p;
        while (q < line_end && *q == ' ') ++q;
        if (q < line_end && *q != '\r') {
            char kind = *q;
            const char *r = q + 1;
            bool ok1 = false, ok2 = false, ok3 = false;
            if (kind == 't' || kind == '#') {
                // header / comment: skipped like the reference
            } else if (kind == 'v') {
                long id = detail::parse_int(r, line_end, ok1);
                long lab = detail::parse_int(r, line_end, ok2);
                if (!ok1 || !ok2 || id < 0)
                    throw LgError(3, "malformed vertex line " + std::to_string(line_no));
                vlines.emplace_back(id, (int)lab);
            } else if (kind == 'e') {
                long a = detail::parse_int(r, line_end, ok1);
                long b = detail::parse_int(r, line_end, ok2);
                long l = detail::parse_int(r, line_end, ok3);
                if (!ok1 || !ok2 || !ok3 || a < 0 || b < 0)
                    throw LgError(3, "malformed edge line " + std::to_string(line_no));
                raw.edges.emplace_back((uint32_t)a, (uint32_t)b, (int)l);
            } else {
                throw LgError(3, "unknown line kind at line " + std::to_string(line_no));
            }
        }
        p = line_end + 1;
    }
    // The reference requires ids 0..N-1 given in order (parallel/graph.h:609-616).
    raw.vlabel.assign(vlines.size(), 0);
    for (size_t i = 0; i < vlines.size(); ++i) {
        if (vlines[i].first != (long)i)
            throw LgError(3, "vertex ids must be 0..N-1 in order (line for id " + std::to_string(vlines[i].first) + ")");
        raw.vlabel[i] = vlines[i].second;
    }
    for (auto &e : raw.edges) {
        if (std::get<0>(e) >= raw.vlabel.size() || std::get<1>(e) >= raw.vlabel.size())
            throw LgError(3, "edge endpoint out of range");
    }
    return raw;
}

// Label pruning, remap and 1-edge supports (parallel/graph.h:662-803).
inline LgGraph build_pruned(const RawLg &raw, int tau) {
    LgGraph g;
    g.input_vertices = raw.vlabel.size();
    g.input_edges = raw.edges.size();
    std::map<int, uint64_t> vcount, ecount;
    for (int l : raw.vlabel) vcount[l]++;
    for (auto &e : raw.edges) ecount[std::get<2>(e)]++;
    std::map<int, bool> vfreq, efreq;
    for (auto &kv : vcount)
        if (kv.second >= (uint64_t)std::max(tau, 0)) {
            vfreq[kv.first] = true;
            g.freq_vlabels.push_back(kv.first);
        }
    for (auto &kv : ecount)
        if (kv.second >= (uint64_t)std::max(tau, 0)) {
            efreq[kv.first] = true;
            g.freq_elabels.push_back(kv.first);
        }
    auto is_vf = [&](int l) { return vfreq.count(l) != 0; };
    auto is_ef = [&](int l) { return efreq.count(l) != 0; };

    const size_t N = raw.vlabel.size();
    std::vector<uint32_t> id_map(N, UINT32_MAX);
    for (size_t i = 0; i < N; ++i) {
        if (is_vf(raw.vlabel[i])) {
            id_map[i] = g.n++;
            g.vlabel.push_back(raw.vlabel[i]);
        }
    }
    // Count kept edges per vertex, then fill.
    std::vector<uint64_t> deg(g.n + 1, 0);
    for (auto &e : raw.edges) {
        uint32_t a, b;
        int l;
        std::tie(a, b, l) = e;
        if (is_vf(raw.vlabel[a]) && is_vf(raw.vlabel[b]) && is_ef(l)) {
            deg[id_map[a]]++;
            deg[id_map[b]]++;
            g.m++;
        }
    }
    g.offs.assign(g.n + 1, 0);
    for (uint32_t v = 0; v < g.n; ++v) g.offs[v + 1] = g.offs[v] + deg[v];
    g.nbr.assign(g.offs[g.n], 0);
    g.elab.assign(g.offs[g.n], 0);
    std::vector<uint64_t> fill(g.offs.begin(), g.offs.end() - 1);
    // 1-edge pattern endpoint sets: key (la, el, lb) with la <= lb
    std::map<std::tuple<int, int, int>, std::pair<std::vector<uint32_t>, std::vector<uint32_t>>> pairs;
    for (auto &e : raw.edges) {
        uint32_t a, b;
        int l;
        std::tie(a, b, l) = e;
        const int la = raw.vlabel[a], lb = raw.vlabel[b];
        if (!(is_vf(la) && is_vf(lb) && is_ef(l))) continue;  // never frequent for tau >= 1
        const uint32_t x = id_map[a], y = id_map[b];
        g.nbr[fill[x]] = y;
        g.elab[fill[x]++] = l;
        g.nbr[fill[y]] = x;
        g.elab[fill[y]++] = l;
        if (la < lb) {
            auto &s = pairs[std::make_tuple(la, l, lb)];
            s.first.push_back(x);
            s.second.push_back(y);
        } else if (la == lb) {
            auto &s = pairs[std::make_tuple(la, l, lb)];
            s.first.push_back(x);
            s.first.push_back(y);
        } else {
            auto &s = pairs[std::make_tuple(lb, l, la)];
            s.first.push_back(y);
            s.second.push_back(x);
        }
    }
    // Sort adjacency by neighbour id (stable, so parallel edges keep input order).
    std::vector<std::pair<uint32_t, int>> tmp;
    for (uint32_t v = 0; v < g.n; ++v) {
        const uint64_t b = g.offs[v], e = g.offs[v + 1];
        tmp.clear();
        for (uint64_t i = b; i < e; ++i) tmp.emplace_back(g.nbr[i], g.elab[i]);
        std::stable_sort(tmp.begin(), tmp.end(),
                         [](const std::pair<uint32_t, int> &p, const std::pair<uint32_t, int> &q) { return p.first < q.first; });
        for (uint64_t i = b; i < e; ++i) {
            g.nbr[i] = tmp[i - b].first;
            g.elab[i] = tmp[i - b].second;
        }
    }
    for (uint32_t v = 0; v < g.n; ++v) g.max_degree = std::max(g.max_degree, g.degree(v));
    std::map<int, uint32_t> lcount;
    for (int l : g.vlabel) lcount[l]++;
    for (auto &kv : lcount) g.max_label_freq = std::max(g.max_label_freq, kv.second);
    for (auto &kv : pairs) {
        auto &A = kv.second.first;
        auto &B = kv.second.second;
        std::sort(A.begin(), A.end());
        A.erase(std::unique(A.begin(), A.end()), A.end());
        std::sort(B.begin(), B.end());
        B.erase(std::unique(B.begin(), B.end()), B.end());
        int la, el, lb;
        std::tie(la, el, lb) = kv.first;
        // candB of a same-label pair equals candA (both endpoints go into both sets).
        const uint32_t ca = (uint32_t)A.size();
        const uint32_t cb = la == lb ? ca : (uint32_t)B.size();
        if ((int64_t)ca >= tau && (int64_t)cb >= tau) g.edge_pairs.push_back({la, el, lb, ca, cb});
    }
    return g;
}

inline LgGraph load_lg(const std::string &path, int tau) {
    std::vector<char> buf;
    if (!detail::read_file(path, buf)) throw LgError(2, "cannot open graph file " + path);
    RawLg raw = parse_lg_text(buf.data(), buf.size());
    return build_pruned(raw, tau);
}

}  // namespace tfsm
