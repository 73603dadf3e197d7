// ORACLE — test infrastructure only.  CPU restatement of the reference's per-pattern MNI support
// evaluation, used (a) by the tests as the parity checker of the CUDA path, and (b) by bench.py's
// CPU-baseline leg and reference arm, where the reference's own build is not available (the GPU
// host is aarch64 and the reference's intersection code is AVX2-only).  Nothing in the product
// includes or links this file.
//
// Pinned against the reference itself: tests/golden/ holds pattern sets produced by the
// reference serial and parallel builds and exact per-vertex MNI domains produced by
// oracle/mni_harness.cpp (the reference's own GMatchEngine), all made by tests/golden/make_golden.py.
//
// What is restated, step by step:
//   LDF + NLF candidate filter ........ parallel/gmatch.h:301-415
//   DPiso refinement to a fixpoint .... parallel/gmatch.h:417-472, pruneCandidates 600-658,
//                                       plan (start vertex, BFS tree) 511-599
//   arc consistency for distinct-label acyclic patterns (no search) .. parallel/gmatch.h:474-509,
//                                       parallel/comper.h:1619-1653, serial/grami.h:362-377
//   candidate-edge tables ............. serial/gmatch.h:687-823 (parallel/gmatch.h:995-1130)
//   GQL matching order + backward nbrs  serial/gmatch.h:584-685
//   LFTJ backtracking (one embedding) . serial/gmatch.h:906-987
//   local candidates by intersection .. serial/gmatch.h:1238-1276 with the hybrid
//                                       merge / galloping switch at ratio 50
//                                       (intersection/computesetintersection.cpp:9-44)
//   lazy per-vertex loop with early exit and non-candidate removal ... serial/grami.h:379-599,
//                                       parallel/comper.h:288-297, 1001-1018
// The wall-clock timeout of the reference (0.1 s, then resume) changes only when a search
// finishes, never its answer, so searches here simply run to completion.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <map>
#include <queue>
#include <vector>

#include "../t-fsm_gb300/csrc/host/lg_graph.hpp"
#include "../t-fsm_gb300/csrc/host/pattern.hpp"

namespace oracle {

using tfsm::LgGraph;
using tfsm::Pattern;
using u32 = uint32_t;

constexpr u32 kInvalid = 0xffffffffu;

struct PortGraph {
    const LgGraph *g = nullptr;
    std::map<int, std::vector<u32>> by_label;     // nodesByLabel, ascending ids
    std::vector<std::vector<std::pair<int, u32>>> nlf;  // per vertex: (label, count), ascending label

    explicit PortGraph(const LgGraph &graph) : g(&graph) {
        for (u32 v = 0; v < g->n; ++v) by_label[g->vlabel[v]].push_back(v);
        nlf.resize(g->n);
        std::map<int, u32> cnt;
        for (u32 v = 0; v < g->n; ++v) {
            cnt.clear();
            for (uint64_t i = g->offs[v]; i < g->offs[v + 1]; ++i) cnt[g->vlabel[g->nbr[i]]]++;
            nlf[v].assign(cnt.begin(), cnt.end());
        }
    }
    u32 nlf_count(u32 v, int label) const {
        for (auto &p : nlf[v])
            if (p.first == label) return p.second;
        return 0;
    }
};

// Sorted-set intersection, hybrid as in computesetintersection.cpp:9-44 (scalar forms).
inline void intersect(const u32 *a, u32 na, const u32 *b, u32 nb, u32 *out, u32 &nout) {
    nout = 0;
    if (na == 0 || nb == 0) return;
    if (na / 50 > nb || nb / 50 > na) {
        // galloping: walk the shorter list, exponential + binary search in the longer one
        const u32 *s = na < nb ? a : b, *l = na < nb ? b : a;
        const u32 ns = na < nb ? na : nb, nl = na < nb ? nb : na;
        u32 lo = 0;
        for (u32 i = 0; i < ns && lo < nl; ++i) {
            const u32 x = s[i];
            u32 step = 1, hi = lo;
            while (hi < nl && l[hi] < x) {
                lo = hi + 1;
                hi += step;
                step <<= 1;
            }
            if (hi > nl) hi = nl;
            while (lo < hi) {
                u32 mid = lo + (hi - lo) / 2;
                if (l[mid] < x) lo = mid + 1;
                else hi = mid;
            }
            if (lo < nl && l[lo] == x) out[nout++] = x;
        }
        return;
    }
    u32 i = 0, j = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else {
            out[nout++] = a[i];
            ++i;
            ++j;
        }
    }
}

struct Table {  // Edges (types.h:67-90): CSR over candidate indices
    std::vector<u32> offset, edge;
};

// Per-thread matching engine; scratch sized once per graph (GMatchEngine::initialize_space).
struct Engine {
    const PortGraph &pg;
    const LgGraph &g;
    std::vector<u32> flag, updated;   // |V| scratch for the filters
    std::vector<char> visited;        // |V| scratch for the search
    std::vector<std::vector<u32>> valid;  // per depth, local candidate indices
    std::vector<u32> tmp;
    uint64_t intersections = 0;

    explicit Engine(const PortGraph &p) : pg(p), g(*p.g) {
        flag.assign(g.n, 0);
        updated.assign(g.n, 0);
        visited.assign(g.n, 0);
        const u32 cap = std::max<u32>(g.max_label_freq, 1);
        valid.assign(tfsm::kMaxPatternVertices, std::vector<u32>(cap));
        tmp.assign(cap, 0);
    }

    // ---------------- filters ----------------
    // LDF + NLF (parallel/gmatch.h:301-415); `parent` domains are inherited for vertices the
    // parent has; `non_cand` holds vertices proven not to match (push-down pruning).
    bool ldf(const Pattern &p, const std::vector<std::vector<u32>> *parent, std::vector<std::vector<u32>> &D) {
        const int n = p.size();
        D.assign(n, {});
        for (int i = 0; i < n; ++i) {
            std::map<int, u32> need;
            for (auto &e : p.vertices[i].edges) need[p.label(e.to)]++;
            const u32 deg = (u32)p.degree(i);
            auto pass = [&](u32 v) {
                if (g.degree(v) < deg) return false;
                for (auto &kv : need)
                    if (pg.nlf_count(v, kv.first) < kv.second) return false;
                return true;
            };
            if (parent && i < (int)parent->size()) {
                for (u32 v : (*parent)[i])
                    if (pass(v)) D[i].push_back(v);
            } else {
                auto it = pg.by_label.find(p.label(i));
                if (it != pg.by_label.end())
                    for (u32 v : it->second)
                        if (pass(v)) D[i].push_back(v);
            }
            if (D[i].empty()) return false;
        }
        return true;
    }

    // BFS plan (selectDPisoStartVertex + bfsTraversal + generateDPisoFilterPlan)
    void dpiso_plan(const Pattern &p, const std::vector<std::vector<u32>> &D, std::vector<int> &bfs,
                    std::vector<std::vector<int>> &bn, std::vector<std::vector<int>> &fn) {
        const int n = p.size();
        double min_score = (double)g.n;
        int start = 0;
        for (int i = 0; i < n; ++i) {
            const int d = p.degree(i);
            if (d <= 1) continue;
            const double s = (double)D[i].size() / (double)d;
            if (s < min_score) {
                min_score = s;
                start = i;
            }
        }
        bfs.clear();
        std::vector<char> seen(n, 0);
        std::queue<int> q;
        q.push(start);
        seen[start] = 1;
        while (!q.empty()) {
            int u = q.front();
            q.pop();
            bfs.push_back(u);
            for (auto &e : p.vertices[u].edges)
                if (!seen[e.to]) {
                    seen[e.to] = 1;
                    q.push(e.to);
                }
        }
        std::vector<int> pos(n);
        for (int i = 0; i < n; ++i) pos[bfs[i]] = i;
        bn.assign(n, {});
        fn.assign(n, {});
        for (int u : bfs)
            for (auto &e : p.vertices[u].edges) (pos[e.to] < pos[u] ? bn[u] : fn[u]).push_back(e.to);
    }

    // pruneCandidates (parallel/gmatch.h:600-658)
    bool prune(const Pattern &p, int u, const std::vector<int> &pivots, std::vector<std::vector<u32>> &D) {
        bool shrunk = false;
        const int ulabel = p.label(u);
        const u32 udeg = (u32)p.degree(u);
        u32 count = 0, nupd = 0;
        for (int pv : pivots) {
            const int el = p.edge_label(u, pv);
            for (u32 v : D[pv]) {
                if (v == kInvalid) continue;
                for (uint64_t k = g.offs[v]; k < g.offs[v + 1]; ++k) {
                    const u32 w = g.nbr[k];
                    if (flag[w] == count && g.elab[k] == el && g.vlabel[w] == ulabel && g.degree(w) >= udeg) {
                        flag[w] += 1;
                        if (count == 0) updated[nupd++] = w;
                    }
                }
            }
            count += 1;
        }
        for (u32 &v : D[u]) {
            if (v == kInvalid) continue;
            if (flag[v] != count) {
                v = kInvalid;
                shrunk = true;
            }
        }
        for (u32 i = 0; i < nupd; ++i) flag[updated[i]] = 0;
        return shrunk;
    }

    // DPisoFilter / filterToConsistency: refine until a full pass changes nothing, compact, and
    // require |D(u)| >= support (isCandidateSetValid(support), parallel/gmatch.h:684-690).
    bool refine(const Pattern &p, std::vector<std::vector<u32>> &D, u32 support) {
        std::vector<int> bfs;
        std::vector<std::vector<int>> bn, fn;
        dpiso_plan(p, D, bfs, bn, fn);
        const int n = p.size();
        bool shrunk = true;
        while (shrunk) {
            for (int i = 1; i < n; ++i) shrunk = prune(p, bfs[i], bn[bfs[i]], D);
            for (int i = n - 2; i >= 0; --i) shrunk = prune(p, bfs[i], fn[bfs[i]], D) | shrunk;
        }
        for (auto &d : D) d.erase(std::remove(d.begin(), d.end(), kInvalid), d.end());
        for (auto &d : D)
            if (d.size() < support) return false;
        return true;
    }

    // ---------------- candidate-edge tables (buildTable) ----------------
    void build_tables(const Pattern &p, const std::vector<std::vector<u32>> &D, std::vector<std::vector<Table>> &T) {
        const int n = p.size();
        T.assign(n, std::vector<Table>(n));
        std::vector<std::vector<char>> built(n, std::vector<char>(n, 0));
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int l, int r) {
            if (p.degree(l) == p.degree(r)) return l < r;
            return p.degree(l) > p.degree(r);
        });
        std::vector<u32> tmp_edges;
        for (int u : order) {
            for (auto &pe : p.vertices[u].edges) {
                const int w = pe.to;
                if (built[u][w]) continue;
                built[u][w] = built[w][u] = 1;
                const int el = pe.label;
                for (u32 j = 0; j < D[u].size(); ++j) flag[D[u][j]] = j + 1;
                Table &tw = T[w][u];  // for each candidate of w: indices in D[u]
                Table &tu = T[u][w];
                tw.offset.assign(D[w].size() + 1, 0);
                tu.offset.assign(D[u].size() + 1, 0);
                tmp_edges.clear();
                for (u32 j = 0; j < D[w].size(); ++j) {
                    const u32 v = D[w][j];
                    tw.offset[j] = (u32)tmp_edges.size();
                    for (uint64_t k = g.offs[v]; k < g.offs[v + 1]; ++k) {
                        const u32 x = g.nbr[k];
                        if (flag[x] != 0 && g.elab[k] == el) {
                            const u32 pos = flag[x] - 1;
                            tmp_edges.push_back(pos);
                            tu.offset[pos + 1] += 1;
                        }
                    }
                }
                tw.offset[D[w].size()] = (u32)tmp_edges.size();
                tw.edge = tmp_edges;
                for (u32 j = 1; j <= D[u].size(); ++j) tu.offset[j] += tu.offset[j - 1];
                tu.edge.assign(tmp_edges.size(), 0);
                std::vector<u32> fill(tu.offset.begin(), tu.offset.end() - 1);
                for (u32 j = 0; j < D[w].size(); ++j)
                    for (u32 k = tw.offset[j]; k < tw.offset[j + 1]; ++k) tu.edge[fill[tw.edge[k]]++] = j;
                for (u32 j = 0; j < D[u].size(); ++j) flag[D[u][j]] = 0;
            }
        }
    }

    // GQL order from `start` and backward neighbours (generateGQLQueryPlan + generateBN)
    static void gql_order(const Pattern &p, const std::vector<std::vector<u32>> &D, int start, std::vector<int> &order,
                          std::vector<std::vector<int>> &bn) {
        const int n = p.size();
        std::vector<char> vis(n, 0), adj(n, 0);
        order.assign(1, start);
        vis[start] = 1;
        for (auto &e : p.vertices[start].edges) adj[e.to] = 1;
        for (int i = 1; i < n; ++i) {
            int next = -1;
            size_t best = SIZE_MAX;
            for (int j = 0; j < n; ++j) {
                if (vis[j] || !adj[j]) continue;
                if (D[j].size() < best || (D[j].size() == best && p.degree(j) > p.degree(next))) {
                    best = D[j].size();
                    next = j;
                }
            }
            vis[next] = 1;
            for (auto &e : p.vertices[next].edges) adj[e.to] = 1;
            order.push_back(next);
        }
        bn.assign(n, {});
        std::vector<char> done(n, 0);
        done[order[0]] = 1;
        for (int i = 1; i < n; ++i) {
            for (auto &e : p.vertices[order[i]].edges)
                if (done[e.to]) bn[i].push_back(e.to);
            done[order[i]] = 1;
        }
    }

    // ---------------- LFTJ: does an embedding with order[0] -> D[order[0]][v_idx] exist? ----------------
    bool search(const Pattern &p, const std::vector<std::vector<u32>> &D, const std::vector<std::vector<Table>> &T,
                const std::vector<int> &order, const std::vector<std::vector<int>> &bn, u32 v_idx,
                std::vector<u32> &emb, std::vector<u32> &idx) {
        const int n = p.size();
        std::vector<u32> cnt(n, 0), counter(n, 0);
        const int u0 = order[0];
        idx[u0] = v_idx;
        emb[u0] = D[u0][v_idx];
        visited[emb[u0]] = 1;
        auto gen = [&](int d) {
            const int u = order[d];
            const int b0 = bn[d][0];
            const Table &t0 = T[b0][u];
            u32 c = t0.offset[idx[b0] + 1] - t0.offset[idx[b0]];
            std::copy(t0.edge.begin() + t0.offset[idx[b0]], t0.edge.begin() + t0.offset[idx[b0] + 1], valid[d].begin());
            for (size_t i = 1; i < bn[d].size(); ++i) {
                const int b = bn[d][i];
                const Table &t = T[b][u];
                const u32 *cur = t.edge.data() + t.offset[idx[b]];
                const u32 nc = t.offset[idx[b] + 1] - t.offset[idx[b]];
                u32 out = 0;
                if (nc < c) intersect(cur, nc, valid[d].data(), c, tmp.data(), out);
                else intersect(valid[d].data(), c, cur, nc, tmp.data(), out);
                ++intersections;
                std::copy(tmp.begin(), tmp.begin() + out, valid[d].begin());
                c = out;
            }
            cnt[d] = c;
        };
        int d = 1;
        counter[1] = 0;
        gen(1);
        bool found = false;
        while (true) {
            while (counter[d] < cnt[d]) {
                const u32 vi = valid[d][counter[d]];
                const int u = order[d];
                const u32 v = D[u][vi];
                counter[d]++;
                if (visited[v]) continue;
                emb[u] = v;
                idx[u] = vi;
                if (d == n - 1) {
                    found = true;
                    break;
                }
                visited[v] = 1;
                ++d;
                counter[d] = 0;
                gen(d);
            }
            if (found) break;
            --d;
            if (d < 1) break;
            visited[emb[order[d]]] = 0;
        }
        // clear visited marks of the partial embedding
        for (int i = 0; i < d && i < n; ++i) visited[emb[order[i]]] = 0;
        visited[emb[u0]] = 0;
        return found;
    }
};

// Result of one support evaluation.
struct Eval {
    bool frequent = false;
    std::vector<u32> mni;                    // per vertex: |found|, exact when `exact`
    std::vector<std::vector<u32>> domains;   // final domains (candidates minus non-candidates)
    uint64_t searches = 0;
};

// One pattern: GraMi-style lazy decision (exact == false) or exact MNI domains (exact == true).
inline Eval evaluate(Engine &eng, const Pattern &p, const std::vector<std::vector<u32>> *parent, u32 tau, bool exact) {
    Eval r;
    const int n = p.size();
    r.mni.assign(n, 0);
    std::vector<std::vector<u32>> D;
    const u32 support = exact ? 1 : tau;
    if (!eng.ldf(p, parent, D)) return r;  // an empty domain: no embedding at all
    const bool express = p.distinct_labels() && p.acyclic();
    const bool ok = eng.refine(p, D, support);
    if (express) {
        // arc-consistent domains are the exact MNI domains of a distinct-label tree
        u32 mn = UINT32_MAX;
        for (int i = 0; i < n; ++i) {
            r.mni[i] = (u32)D[i].size();
            mn = std::min(mn, r.mni[i]);
        }
        r.frequent = mn >= tau;
        r.domains = D;
        return r;
    }
    // Lazy mode: some |D(u)| < tau decides "infrequent".  Exact mode: an empty domain means
    // no embedding exists, so every MNI domain is empty.
    if (!ok) return r;
    std::vector<std::vector<Table>> T;
    eng.build_tables(p, D, T);
    std::vector<std::vector<char>> found(n), failed(n);
    std::vector<std::vector<u32>> pos(n);  // vertex id -> index in D[u] via binary search
    for (int i = 0; i < n; ++i) {
        found[i].assign(D[i].size(), 0);
        failed[i].assign(D[i].size(), 0);
    }
    auto index_of = [&](int u, u32 v) -> long {
        auto it = std::lower_bound(D[u].begin(), D[u].end(), v);
        return (it != D[u].end() && *it == v) ? (long)(it - D[u].begin()) : -1;
    };
    std::vector<u32> nfound(n, 0);
    std::vector<u32> emb(n), idx(n);
    std::vector<int> order;
    std::vector<std::vector<int>> bn;
    bool dead = false;
    for (int u = 0; u < n && !dead; ++u) {
        if (!exact && nfound[u] >= tau) continue;
        Engine::gql_order(p, D, u, order, bn);
        u32 nfail = 0;
        for (u32 vi = 0; vi < D[u].size(); ++vi) {
            if (!exact && nfound[u] >= tau) break;
            if (found[u][vi]) continue;
            ++r.searches;
            if (eng.search(p, D, T, order, bn, vi, emb, idx)) {
                for (int j = 0; j < n; ++j) {
                    long k = index_of(j, emb[j]);
                    if (k >= 0 && !found[j][(size_t)k]) {
                        found[j][(size_t)k] = 1;
                        nfound[j]++;
                    }
                }
            } else {
                failed[u][vi] = 1;
                ++nfail;
                if (!exact && D[u].size() - nfail < tau) {
                    dead = true;
                    break;
                }
            }
        }
        if (!exact && nfound[u] < tau) dead = true;
    }
    for (int i = 0; i < n; ++i) r.mni[i] = nfound[i];
    if (dead && !exact) return r;
    u32 mn = UINT32_MAX;
    for (int i = 0; i < n; ++i) mn = std::min(mn, nfound[i]);
    r.frequent = mn >= tau;
    r.domains.assign(n, {});
    for (int i = 0; i < n; ++i)
        for (u32 k = 0; k < D[i].size(); ++k)
            if (!failed[i][k]) r.domains[i].push_back(D[i][k]);
    return r;
}

}  // namespace oracle
