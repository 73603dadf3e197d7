// ORACLE — test infrastructure only.  Exact per-vertex MNI domains by plain backtracking, written
// from the definition alone: v is in D(u) when some injective, label-preserving map of the
// pattern into the data graph sends u to v and every pattern edge (a, b, l) to a data edge
// between the images that carries label l (with parallel edges, any one of them).  No filter, no
// candidate table, no intersection algorithm, no timeout: a second, independent checker for
// patterns where the reference's own engine (oracle/mni_harness.cpp) deviates from the
// definition.  Searches that the reference's engine resumes after a timeout
// (GMatchEngine::resumeSearch, serial/gmatch.h:231-244) can return an embedding that breaks a
// pattern edge, and every vertex of a returned embedding joins the domains.
//
// The graph is read by the repository's restatement of the reference loader (same pruning and
// vertex numbering as the reference).  Every found embedding adds all its vertices to their
// pattern vertices' domains; the remaining candidates are searched exhaustively, in parallel.
//
// usage: mni_brute -file G.lg -freq TAU -patterns P.txt [-threads T] [-decide 1]
//   P.txt and the output use the format of mni_harness: "<codes> | c0 c1 ... c(n-1)".  With
//   -decide 1 the counts are lower bounds that reach TAU everywhere exactly when the pattern is
//   frequent (the search stops early both ways).
#include <algorithm>
#include <array>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../t-fsm_gb300/csrc/host/lg_graph.hpp"

namespace {

struct Pat {
    int n = 0;
    std::vector<int> lab;
    std::vector<std::vector<std::pair<int, int>>> adj;  // (neighbour, edge label)
};

bool parse_pattern(const std::string &line, Pat &p) {
    std::istringstream ss(line);
    std::string tok;
    std::vector<std::array<int, 5>> codes;
    while (ss >> tok) {
        std::array<int, 5> c{};
        if (sscanf(tok.c_str(), "%d,%d,%d,%d,%d", &c[0], &c[1], &c[2], &c[3], &c[4]) != 5) return false;
        codes.push_back(c);
    }
    int n = 0;
    for (auto &c : codes) n = std::max(n, std::max(c[0], c[1]) + 1);
    if (n == 0 || n > 32) return false;
    p.n = n;
    p.lab.assign(n, -1);
    p.adj.assign(n, {});
    for (auto &c : codes) {
        for (int k : {0, 1}) {  // a vertex keeps one label across its codes
            const int x = c[k], l = c[k == 0 ? 2 : 4];
            if (p.lab[x] >= 0 && p.lab[x] != l) return false;
            p.lab[x] = l;
        }
        p.adj[c[0]].push_back({c[1], c[3]});
        p.adj[c[1]].push_back({c[0], c[3]});
    }
    for (int x : p.lab)
        if (x < 0) return false;
    return true;
}

struct Search {
    const tfsm::LgGraph &g;
    const Pat &p;
    std::vector<int> order;                 // BFS order from the start vertex
    std::vector<std::vector<std::pair<int, int>>> back;  // per depth: (earlier depth, edge label)
    std::vector<uint32_t> emb;              // by pattern vertex

    Search(const tfsm::LgGraph &g_, const Pat &p_, int start) : g(g_), p(p_), emb(p_.n) {
        std::vector<int> depth(p.n, -1);
        order.push_back(start);
        depth[start] = 0;
        for (size_t i = 0; i < order.size(); ++i)
            for (auto &e : p.adj[order[i]])
                if (depth[e.first] < 0) {
                    depth[e.first] = (int)order.size();
                    order.push_back(e.first);
                }
        back.assign(order.size(), {});
        for (size_t d = 0; d < order.size(); ++d)
            for (auto &e : p.adj[order[d]])
                if (depth[e.first] >= 0 && depth[e.first] < (int)d) back[d].push_back({depth[e.first], e.second});
    }

    // some x-y edge with label l
    bool edge(uint32_t x, uint32_t y, int l) const {
        auto b = g.nbr.begin() + g.offs[x], e = g.nbr.begin() + g.offs[x + 1];
        for (auto it = std::lower_bound(b, e, y); it != e && *it == y; ++it)
            if (g.elab[it - g.nbr.begin()] == l) return true;
        return false;
    }

    bool used(uint32_t x, size_t d) const {
        for (size_t k = 0; k < d; ++k)
            if (emb[order[k]] == x) return true;
        return false;
    }

    bool dfs(size_t d) {
        if (d == order.size()) return true;
        const int w = order[d];
        // enumerate the neighbours of the backward neighbour with the smallest degree
        size_t best = 0;
        for (size_t k = 1; k < back[d].size(); ++k)
            if (g.degree(emb[order[back[d][k].first]]) < g.degree(emb[order[back[d][best].first]])) best = k;
        const uint32_t a = emb[order[back[d][best].first]];
        const int al = back[d][best].second;
        uint32_t prev = UINT32_MAX;
        for (uint64_t i = g.offs[a]; i < g.offs[a + 1]; ++i) {
            const uint32_t x = g.nbr[i];
            if (x == prev || g.vlabel[x] != p.lab[w]) continue;  // parallel entries: x once
            prev = x;
            if (!edge(a, x, al) || used(x, d)) continue;
            bool ok = true;
            for (size_t k = 0; k < back[d].size() && ok; ++k)
                if (k != best) ok = edge(emb[order[back[d][k].first]], x, back[d][k].second);
            if (!ok) continue;
            emb[w] = x;
            if (dfs(d + 1)) return true;
        }
        return false;
    }
};

}  // namespace

int main(int argc, char **argv) {
    const char *file = nullptr, *pats = nullptr;
    int tau = -1, threads = (int)std::max(1u, std::thread::hardware_concurrency());
    bool decide = false;
    for (int i = 1; i + 1 < argc; i += 2) {
        if (!strcmp(argv[i], "-file")) file = argv[i + 1];
        else if (!strcmp(argv[i], "-freq")) tau = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "-patterns")) pats = argv[i + 1];
        else if (!strcmp(argv[i], "-threads")) threads = std::max(1, atoi(argv[i + 1]));
        else if (!strcmp(argv[i], "-decide")) decide = atoi(argv[i + 1]) != 0;
    }
    if (!file || !pats || tau < 0) {
        std::cerr << "usage: mni_brute -file G.lg -freq TAU -patterns P.txt [-threads T] [-decide 1]" << std::endl;
        return 2;
    }
    const tfsm::LgGraph g = tfsm::load_lg(file, tau);
    std::ifstream in(pats);
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        Pat p;
        if (!parse_pattern(line, p)) {
            std::cerr << "bad pattern: " << line << std::endl;
            return 2;
        }
        // found[u][v]: v proven in D(u) by an embedding
        std::vector<std::vector<std::atomic<uint8_t>>> found(p.n);
        for (auto &f : found) {
            std::vector<std::atomic<uint8_t>> z(g.n);
            f.swap(z);
        }
        // -decide: stop a vertex once tau of its candidates are found, and the pattern once a
        // vertex cannot reach tau; the counts printed are then lower bounds, and the pattern is
        // frequent exactly when every count reaches tau
        std::vector<std::atomic<uint64_t>> nfound(p.n);
        for (int u = 0; u < p.n; ++u) {
            uint64_t cands = 0;
            for (uint32_t v = 0; v < g.n; ++v) cands += g.vlabel[v] == p.lab[u];
            std::atomic<uint32_t> next{0};
            std::atomic<uint64_t> nfail{0};
            auto settled = [&] {
                return decide && (nfound[u].load() >= (uint64_t)tau || cands - nfail.load() < (uint64_t)tau);
            };
            std::vector<std::thread> th;
            for (int t = 0; t < threads; ++t)
                th.emplace_back([&, u] {
                    Search s(g, p, u);
                    for (;;) {
                        const uint32_t v0 = next.fetch_add(64);
                        if (v0 >= g.n || settled()) break;
                        for (uint32_t v = v0; v < std::min<uint32_t>(g.n, v0 + 64); ++v) {
                            if (g.vlabel[v] != p.lab[u] || found[u][v].load()) continue;
                            s.emb[u] = v;
                            if (s.dfs(1)) {
                                for (int w = 0; w < p.n; ++w)
                                    if (found[w][s.emb[w]].exchange(1) == 0) nfound[w].fetch_add(1);
                            } else {
                                nfail.fetch_add(1);
                            }
                        }
                    }
                });
            for (auto &t : th) t.join();
            if (decide && cands - nfail.load() < (uint64_t)tau) break;  // infrequent
        }
        std::cout << line << " |";
        for (int u = 0; u < p.n; ++u) {
            uint64_t c = 0;
            for (uint32_t v = 0; v < g.n; ++v) c += found[u][v].load();
            std::cout << ' ' << c;
        }
        std::cout << std::endl;
    }
    return 0;
}
