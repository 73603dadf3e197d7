// Breadth-first rightmost extension of every canonical pattern over a few vertex labels and three
// edge labels (up to 5 vertices), as the miner grows levels, with each child's canonical check and
// one-edge-smaller sub-patterns.  Built with AddressSanitizer / UndefinedBehaviorSanitizer by
// tests/test_canonical.py: the reference's forward-extension ordering is not a strict weak
// ordering, and the check must still never touch memory outside its containers.  Test
// infrastructure only.
//
// usage: canonical_enum THREADS VERTEX_LABELS MAX_EDGES
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "host/pattern.hpp"
#include "host/subpattern.hpp"

using namespace tfsm;

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    const int threads = std::atoi(argv[1]), nl = std::atoi(argv[2]), max_edges = std::atoi(argv[3]);
    ExtendContext ctx;
    ctx.freq_elabels = {1, 2, 3};
    ctx.max_nodes = 5;
    for (int a = 0; a < nl; ++a)
        for (int b = 0; b < nl; ++b) ctx.neighbor_labels[a].insert(b);
    std::vector<Pattern> level;
    for (int a = 0; a < nl; ++a)
        for (int b = a; b < nl; ++b)
            for (int e = 1; e <= 3; ++e) {
                Pattern p;
                p.push(DfsCode{0, 1, a, e, b});
                level.push_back(p);
            }
    size_t total = level.size();
    for (int edges = 1; edges < max_edges && !level.empty(); ++edges) {
        std::vector<std::vector<Pattern>> kids(level.size());
        std::atomic<size_t> next(0);
        std::atomic<int> bad(0);
        std::vector<std::thread> th;
        for (int t = 0; t < threads; ++t)
            th.emplace_back([&]() {
                for (size_t i; (i = next.fetch_add(1)) < level.size();) {
                    extend_pattern(level[i], ctx, kids[i]);
                    for (auto &k : kids[i]) {
                        if (!is_canonical(k)) bad++;  // every child returned passed the check: stable
                        std::vector<SubPattern> subs;
                        one_edge_smaller(k, subs);
                    }
                }
            });
        for (auto &x : th) x.join();
        if (bad) {
            std::printf("FAIL %d children not canonical on a second check\n", bad.load());
            return 1;
        }
        std::vector<Pattern> nxt;
        for (auto &k : kids)
            for (auto &p : k) nxt.push_back(std::move(p));
        level = std::move(nxt);
        total += level.size();
    }
    std::printf("ok %zu patterns\n", total);
    return 0;
}
