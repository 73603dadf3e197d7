// Test driver: the multi-threaded loader (host/lg_fast.hpp) must build exactly the graph of the
// plain restatement of the reference loader (host/lg_graph.hpp), field for field.
//   loader_check FILE TAU [THREADS]      -> prints "same" or the first difference; exit 0 when same
//   loader_check --random SEED TAU       -> the same on a random multigraph (parallel edges,
//                                           self-loops, negative and wide-range labels)
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>

#include "host/lg_fast.hpp"
#include "host/lg_graph.hpp"

using namespace tfsm;

static int compare(const LgGraph &a, const LgGraph &b) {
#define SAME(f)                                                   \
    if (!(a.f == b.f)) {                                          \
        std::printf("differ: %s\n", #f);                          \
        return 1;                                                 \
    }
    SAME(n) SAME(m) SAME(vlabel) SAME(offs) SAME(nbr) SAME(elab) SAME(freq_vlabels) SAME(freq_elabels)
    SAME(max_label_freq) SAME(max_degree) SAME(input_vertices) SAME(input_edges)
    if (a.edge_pairs.size() != b.edge_pairs.size()) {
        std::printf("differ: edge_pairs size %zu vs %zu\n", a.edge_pairs.size(), b.edge_pairs.size());
        return 1;
    }
    for (size_t i = 0; i < a.edge_pairs.size(); ++i) {
        const EdgePair &x = a.edge_pairs[i], &y = b.edge_pairs[i];
        if (x.la != y.la || x.el != y.el || x.lb != y.lb || x.cand_a != y.cand_a || x.cand_b != y.cand_b) {
            std::printf("differ: edge_pairs[%zu]\n", i);
            return 1;
        }
    }
    std::printf("same (n=%u m=%llu pairs=%zu)\n", a.n, (unsigned long long)a.m, a.edge_pairs.size());
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 4 && std::string(argv[1]) == "--random") {
        std::mt19937_64 rng(std::strtoull(argv[2], nullptr, 10));
        const int tau = std::atoi(argv[3]);
        RawLg raw;
        const uint32_t n = 2000 + (uint32_t)(rng() % 20000);
        const bool wide = rng() % 2;
        for (uint32_t i = 0; i < n; ++i) {
            const int l = (int)(rng() % 12) - 3;
            raw.vlabel.push_back(wide ? l * 1000003 : l);
        }
        const uint64_t m = n * (2 + rng() % 8);
        for (uint64_t k = 0; k < m; ++k) {
            const uint32_t a = (uint32_t)(rng() % n);
            const uint32_t b = rng() % 50 == 0 ? a : (uint32_t)(rng() % n);
            const int el = (int)(rng() % 5) - 1;
            raw.edges.emplace_back(a, b, wide ? el * 7919 : el);
            if (rng() % 20 == 0) raw.edges.emplace_back(b, a, wide ? (el + 1) * 7919 : el + 1);  // parallel edge
        }
        const LgGraph ref = build_pruned(raw, tau);
        for (int threads : {1, 3, 16})
            if (compare(ref, build_pruned_fast(raw, tau, threads))) return 1;
        // the host-array form (tfsm_graph_from_edges) reads the caller's arrays in place
        std::vector<uint32_t> src, dst;
        std::vector<int32_t> lab;
        for (auto &e : raw.edges) {
            src.push_back(std::get<0>(e));
            dst.push_back(std::get<1>(e));
            lab.push_back(std::get<2>(e));
        }
        for (int threads : {1, 16})
            if (compare(ref, build_pruned_edges(raw.vlabel, EdgeArrays{src.data(), dst.data(), lab.data(), src.size()},
                                                tau, threads)))
                return 1;
        return 0;
    }
    if (argc < 3) {
        std::fprintf(stderr, "usage: loader_check FILE TAU [THREADS] | --random SEED TAU\n");
        return 2;
    }
    const int tau = std::atoi(argv[2]);
    const int threads = argc > 3 ? std::atoi(argv[3]) : 8;
    std::string e1, e2;
    LgGraph a, b;
    try {
        a = load_lg(argv[1], tau);
    } catch (const LgError &e) {
        e1 = std::to_string(e.code) + " " + e.what();
    }
    try {
        b = load_lg_fast(argv[1], tau, threads);
    } catch (const LgError &e) {
        e2 = std::to_string(e.code) + " " + e.what();
    }
    if (!e1.empty() || !e2.empty()) {
        std::printf("errors: [%s] [%s]\n", e1.c_str(), e2.c_str());
        return e1 == e2 ? 0 : 1;
    }
    return compare(a, b);
}
