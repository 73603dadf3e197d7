// Test driver: canonical_key (host/subpattern.hpp) is invariant under vertex relabelling and
// separates non-isomorphic small graphs (checked against brute force over all permutations).
#include <algorithm>
#include <cstdio>
#include <random>
#include <set>

#include "host/subpattern.hpp"

using namespace tfsm;

static std::vector<std::array<int, 3>> brute_min(const SmallGraph &g) {
    const int n = (int)g.label.size();
    std::vector<int> perm((size_t)n);
    for (int i = 0; i < n; ++i) perm[(size_t)i] = i;
    std::vector<std::array<int, 3>> best;
    std::vector<int> best_lab;
    bool have = false;
    do {
        std::vector<int> lab((size_t)n);
        for (int v = 0; v < n; ++v) lab[(size_t)perm[(size_t)v]] = g.label[(size_t)v];
        std::vector<std::array<int, 3>> e;
        for (auto &x : g.edges)
            e.push_back({std::min(perm[(size_t)x[0]], perm[(size_t)x[1]]), std::max(perm[(size_t)x[0]], perm[(size_t)x[1]]), x[2]});
        std::sort(e.begin(), e.end());
        if (!have || std::make_pair(lab, e) < std::make_pair(best_lab, best)) {
            best = e;
            best_lab = lab;
            have = true;
        }
    } while (std::next_permutation(perm.begin(), perm.end()));
    std::vector<std::array<int, 3>> out = best;
    out.push_back({-1, -1, -1});
    for (int l : best_lab) out.push_back({l, 0, 0});
    return out;
}

int main() {
    std::mt19937 rng(11);
    int fails = 0;
    std::set<std::vector<std::array<int, 3>>> classes;
    std::set<std::string> keys;
    for (int t = 0; t < 3000; ++t) {
        const int n = 2 + (int)(rng() % 5);
        SmallGraph g;
        for (int v = 0; v < n; ++v) g.label.push_back((int)(rng() % 2));
        for (int v = 1; v < n; ++v) g.edges.push_back({(int)(rng() % v), v, (int)(rng() % 2)});  // a tree
        for (int k = 0; k < 2; ++k) {
            const int a = (int)(rng() % n), b = (int)(rng() % n);
            bool dup = a == b;
            for (auto &e : g.edges) dup = dup || (std::min(e[0], e[1]) == std::min(a, b) && std::max(e[0], e[1]) == std::max(a, b));
            if (!dup) g.edges.push_back({a, b, (int)(rng() % 2)});
        }
        const std::string k0 = canonical_key(g);
        // relabelled copy
        std::vector<int> p((size_t)n);
        for (int i = 0; i < n; ++i) p[(size_t)i] = i;
        std::shuffle(p.begin(), p.end(), rng);
        SmallGraph h;
        h.label.resize((size_t)n);
        for (int v = 0; v < n; ++v) h.label[(size_t)p[(size_t)v]] = g.label[(size_t)v];
        for (auto &e : g.edges) h.edges.push_back({p[(size_t)e[1]], p[(size_t)e[0]], e[2]});
        std::shuffle(h.edges.begin(), h.edges.end(), rng);
        if (canonical_key(h) != k0) ++fails;
        classes.insert(brute_min(g));
        keys.insert(k0);
    }
    std::printf("relabelling mismatches %d, isomorphism classes %zu, distinct keys %zu\n", fails, classes.size(),
                keys.size());
    return fails == 0 && classes.size() == keys.size() ? 0 : 1;
}
