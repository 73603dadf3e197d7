// Multi-threaded `.lg` loader for the product path: same LgGraph as load_lg / build_pruned in
// lg_graph.hpp (field for field, including the order of every adjacency list and of the 1-edge
// pattern table), without their per-edge ordered-map lookups.
//
//   * labels map to dense indices through a direct table (or a hash map for wide label ranges),
//     computed once per vertex and once per distinct edge label;
//   * the 1-edge pattern endpoint sets (parallel/graph.h:759-803 keeps a (la, el, lb) triple when
//     both sets reach tau) are counted per vertex from its sorted adjacency: a vertex is in the
//     endpoint set of (la, el, lb) when one of its edges with label el leads to label lb;
//   * parsing, adjacency sorting and the endpoint counts run on all host threads.
#pragma once

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "lg_graph.hpp"

namespace tfsm {

namespace fast {

// Host threads for parallel host work: TFSM_HOST_THREADS when set (1..64), else the cores (<= 64).
inline int default_threads() {
    static const int n = []() {
        const char *env = std::getenv("TFSM_HOST_THREADS");
        const int want = env ? std::atoi(env) : 0;
        if (want >= 1) return std::min(64, want);
        return (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    }();
    return n;
}

// Process-wide workers for the host's parallel passes (creating a thread per core for each pass
// costs about as much as a pass on a 1 M-edge graph).  One job at a time: callers are serialised
// on `job_mu`; a job runs `tasks` calls of `fn(task)` spread over the workers and the caller.
// Each job's state (function, task count, claim and completion counters) lives in its own record,
// and a job ends only when every task is done and no worker is still inside it, so a worker
// leaving one job can never claim a task of the next.  A task that throws still counts as done;
// the job keeps the first exception and run() rethrows it once the job has ended.
class Workers {
  public:
    static Workers &get() {
        static Workers w(default_threads() - 1);
        return w;
    }
    void run(size_t tasks, const std::function<void(size_t)> &fn) {
        std::lock_guard<std::mutex> job(job_mu_);
        Job j(&fn, tasks);
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &j;
            ++gen_;
        }
        cv_.notify_all();
        drain(j);
        {
            std::unique_lock<std::mutex> lk(mu_);
            done_cv_.wait(lk, [&]() { return j.done.load() == j.tasks && active_ == 0; });
            job_ = nullptr;
        }
        if (j.error) std::rethrow_exception(j.error);
    }
    ~Workers() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }

  private:
    struct Job {
        Job(const std::function<void(size_t)> *f, size_t n) : fn(f), tasks(n) {}
        const std::function<void(size_t)> *fn;
        const size_t tasks;
        std::atomic<size_t> next{0}, done{0};
        std::mutex err_mu;
        std::exception_ptr error;  // the first exception a task threw
    };
    explicit Workers(int n) {
        for (int i = 0; i < n; ++i) th_.emplace_back([this]() { loop(); });
    }
    void drain(Job &j) {
        for (size_t k; (k = j.next.fetch_add(1)) < j.tasks;) {
            try {
                (*j.fn)(k);
            } catch (...) {
                std::lock_guard<std::mutex> lk(j.err_mu);
                if (!j.error) j.error = std::current_exception();
            }
            if (j.done.fetch_add(1) + 1 == j.tasks) {
                std::lock_guard<std::mutex> lk(mu_);
                done_cv_.notify_all();
            }
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            Job *j = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&]() { return quit_ || (job_ != nullptr && gen_ != seen); });
                if (quit_) return;
                seen = gen_;
                j = job_;
                ++active_;
            }
            drain(*j);
            std::lock_guard<std::mutex> lk(mu_);
            if (--active_ == 0) done_cv_.notify_all();
        }
    }
    std::vector<std::thread> th_;
    std::mutex job_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    Job *job_ = nullptr;  // the running job (guarded by mu_)
    size_t active_ = 0;   // workers inside job_ (guarded by mu_)
    uint64_t gen_ = 0;
    bool quit_ = false;
};

// Runs fn(t, begin, end) over [0, n) split into `threads` contiguous ranges.
template <class F>
void parallel_ranges(size_t n, int threads, F fn) {
    const size_t t = (size_t)std::max(1, std::min<int>(threads, (int)std::max<size_t>(1, n / 4096)));
    if (t <= 1) {
        fn(0, (size_t)0, n);
        return;
    }
    const std::function<void(size_t)> task = [&](size_t k) { fn((int)k, n * k / t, n * (k + 1) / t); };
    Workers::get().run(t, task);
}

// int label -> dense index among `labels` (ascending, distinct); -1 when absent.
class LabelIndex {
  public:
    explicit LabelIndex(const std::vector<int> &labels) {
        if (labels.empty()) return;
        lo_ = labels.front();
        const int64_t range = (int64_t)labels.back() - lo_ + 1;
        if (range <= (1 << 22)) {
            table_.assign((size_t)range, -1);
            for (size_t i = 0; i < labels.size(); ++i) table_[(size_t)((int64_t)labels[i] - lo_)] = (int)i;
        } else {
            for (size_t i = 0; i < labels.size(); ++i) map_[labels[i]] = (int)i;
            wide_ = true;
        }
    }
    int operator()(int label) const {
        if (wide_) {
            auto it = map_.find(label);
            return it == map_.end() ? -1 : it->second;
        }
        const int64_t k = (int64_t)label - lo_;
        return (k < 0 || k >= (int64_t)table_.size()) ? -1 : table_[(size_t)k];
    }

  private:
    int lo_ = 0;
    bool wide_ = false;
    std::vector<int> table_;
    std::unordered_map<int, int> map_;
};

// Distinct values of `v`, ascending.
inline std::vector<int> distinct(std::vector<int> v) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
}

}  // namespace fast

// Same result as parse_lg_text (same errors for malformed input), parsed by chunks of lines on
// all threads.
inline RawLg parse_lg_text_fast(const char *data, size_t size, int threads = fast::default_threads()) {
    // chunk boundaries at line starts
    const size_t want = std::max<size_t>(1, std::min<size_t>((size_t)threads, size / (1 << 20) + 1));
    std::vector<size_t> cut{0};
    for (size_t k = 1; k < want; ++k) {
        size_t pos = size * k / want;
        if (pos <= cut.back()) continue;
        const void *nl = std::memchr(data + pos, '\n', size - pos);
        if (!nl) break;
        pos = (size_t)((const char *)nl - data) + 1;
        if (pos > cut.back() && pos < size) cut.push_back(pos);
    }
    cut.push_back(size);
    const size_t chunks = cut.size() - 1;
    struct Part {
        std::vector<std::pair<long, int>> vlines;
        std::vector<std::tuple<uint32_t, uint32_t, int>> edges;
        size_t lines = 0;
        int err_code = 0;
        size_t err_line = 0;  // line number inside the chunk (1-based)
        std::string err;
    };
    std::vector<Part> parts(chunks);
    std::vector<std::thread> th;
    auto work = [&](size_t c) {
        Part &P = parts[c];
        const char *p = data + cut[c], *end = data + cut[c + 1];
        try {
            while (p < end) {
                const char *line_end = (const char *)std::memchr(p, '\n', (size_t)(end - p));
                if (!line_end) line_end = end;
                ++P.lines;
                const char *q = p;
                while (q < line_end && *q == ' ') ++q;
                if (q < line_end && *q != '\r') {
                    const char kind = *q;
                    const char *r = q + 1;
                    bool ok1 = false, ok2 = false, ok3 = false;
                    if (kind == 't' || kind == '#') {
                    } else if (kind == 'v') {
                        const long id = detail::parse_int(r, line_end, ok1);
                        const long lab = detail::parse_int(r, line_end, ok2);
                        if (!ok1 || !ok2 || id < 0) throw LgError(3, "malformed vertex line");
                        P.vlines.emplace_back(id, (int)lab);
                    } else if (kind == 'e') {
                        const long a = detail::parse_int(r, line_end, ok1);
                        const long b = detail::parse_int(r, line_end, ok2);
                        const long l = detail::parse_int(r, line_end, ok3);
                        if (!ok1 || !ok2 || !ok3 || a < 0 || b < 0) throw LgError(3, "malformed edge line");
                        P.edges.emplace_back((uint32_t)a, (uint32_t)b, (int)l);
                    } else {
                        throw LgError(3, "unknown line kind");
                    }
                }
                p = line_end + 1;
            }
        } catch (const LgError &e) {
            P.err_code = e.code;
            P.err_line = P.lines;
            P.err = e.what();
        }
    };
    if (chunks == 1) work(0);
    else {
        for (size_t c = 0; c < chunks; ++c) th.emplace_back(work, c);
        for (auto &x : th) x.join();
    }
    size_t base = 0, nv = 0, ne = 0;
    for (auto &P : parts) {
        if (P.err_code) {
            const std::string what = P.err == "malformed vertex line" ? "malformed vertex line "
                                     : P.err == "malformed edge line" ? "malformed edge line "
                                                                      : "unknown line kind at line ";
            throw LgError(P.err_code, what + std::to_string(base + P.err_line));
        }
        base += P.lines;
        nv += P.vlines.size();
        ne += P.edges.size();
    }
    RawLg raw;
    raw.vlabel.assign(nv, 0);
    raw.edges.reserve(ne);
    size_t i = 0;
    for (auto &P : parts) {
        for (auto &vl : P.vlines) {
            if (vl.first != (long)i)
                throw LgError(3, "vertex ids must be 0..N-1 in order (line for id " + std::to_string(vl.first) + ")");
            raw.vlabel[i++] = vl.second;
        }
        raw.edges.insert(raw.edges.end(), P.edges.begin(), P.edges.end());
    }
    for (auto &e : raw.edges)
        if (std::get<0>(e) >= raw.vlabel.size() || std::get<1>(e) >= raw.vlabel.size())
            throw LgError(3, "edge endpoint out of range");
    return raw;
}

// Edges of the input, read in place: (a, b, label) of edge k in input order.
struct EdgeTuples {
    const std::vector<std::tuple<uint32_t, uint32_t, int>> &e;
    size_t size() const { return e.size(); }
    uint32_t a(size_t k) const { return std::get<0>(e[k]); }
    uint32_t b(size_t k) const { return std::get<1>(e[k]); }
    int l(size_t k) const { return std::get<2>(e[k]); }
};
struct EdgeArrays {
    const uint32_t *src, *dst;
    const int32_t *lab;
    size_t m;
    size_t size() const { return m; }
    uint32_t a(size_t k) const { return src[k]; }
    uint32_t b(size_t k) const { return dst[k]; }
    int l(size_t k) const { return lab[k]; }
};

// Same LgGraph as build_pruned on the same vertex labels and edges (endpoints already checked).
template <class Edges>
LgGraph build_pruned_edges(const std::vector<int> &vlabel_in, const Edges &edges, int tau,
                           int threads = fast::default_threads()) {
    LgGraph g;
    const size_t N = vlabel_in.size(), M = edges.size();
    if (M >= (1ull << 32)) throw LgError(5, "more than 2^32 - 1 edges");
    g.input_vertices = N;
    g.input_edges = M;
    const uint64_t need = (uint64_t)std::max(tau, 0);
    // ---- label frequencies ----
    const std::vector<int> vlabels = fast::distinct(vlabel_in);
    const fast::LabelIndex vidx(vlabels);
    std::vector<uint64_t> vcount(vlabels.size(), 0);
    std::vector<int> vdense_in(N);  // dense index among all input labels
    for (size_t i = 0; i < N; ++i) vcount[(size_t)(vdense_in[i] = vidx(vlabel_in[i]))]++;
    std::vector<int> elabels_all;
    {
        std::vector<int> seen;
        // few distinct edge labels in practice: collect them without sorting 2m values
        int last = 0;
        bool have = false;
        for (size_t k = 0; k < M; ++k) {
            const int l = edges.l(k);
            if (have && l == last) continue;
            have = true;
            last = l;
            seen.push_back(l);
            if (seen.size() > 4096) seen = fast::distinct(seen);
        }
        elabels_all = fast::distinct(seen);
    }
    const fast::LabelIndex eidx_all(elabels_all);
    const int T = std::max(1, threads);
    std::vector<std::vector<uint64_t>> ecount_t((size_t)T);
    fast::parallel_ranges(M, T, [&](int t, size_t k0, size_t k1) {
        auto &c = ecount_t[(size_t)t];
        c.assign(elabels_all.size(), 0);
        for (size_t k = k0; k < k1; ++k) c[(size_t)eidx_all(edges.l(k))]++;
    });
    std::vector<uint64_t> ecount(elabels_all.size(), 0);
    for (auto &c : ecount_t)
        for (size_t i = 0; i < c.size(); ++i) ecount[i] += c[i];
    std::vector<char> vfreq(vlabels.size(), 0), efreq(elabels_all.size(), 0);
    for (size_t k = 0; k < vlabels.size(); ++k)
        if (vcount[k] >= need) {
            vfreq[k] = 1;
            g.freq_vlabels.push_back(vlabels[k]);
        }
    for (size_t k = 0; k < elabels_all.size(); ++k)
        if (ecount[k] >= need) {
            efreq[k] = 1;
            g.freq_elabels.push_back(elabels_all[k]);
        }
    // ---- kept vertices, in input order ----
    std::vector<uint32_t> id_map(N, UINT32_MAX);
    for (size_t i = 0; i < N; ++i)
        if (vfreq[(size_t)vdense_in[i]]) {
            id_map[i] = g.n++;
            g.vlabel.push_back(vlabel_in[i]);
        }
    // ---- CSR of kept edges (both directions), filled in parallel, then every list sorted by
    // (neighbour id, input edge index): the reference's order (neighbour ascending, parallel edges
    // in input order) whatever order the threads filled it in ----
    std::vector<uint32_t> deg((size_t)g.n + 1, 0);
    std::vector<char> ekeep(M);
    std::vector<uint64_t> kept_t((size_t)T, 0);
    fast::parallel_ranges(M, T, [&](int t, size_t k0, size_t k1) {
        uint64_t kept = 0;
        for (size_t k = k0; k < k1; ++k) {
            const uint32_t x = id_map[edges.a(k)], y = id_map[edges.b(k)];
            const bool keep = x != UINT32_MAX && y != UINT32_MAX && efreq[(size_t)eidx_all(edges.l(k))];
            ekeep[k] = keep;
            if (keep) {
                __atomic_fetch_add(&deg[x], 1u, __ATOMIC_RELAXED);
                __atomic_fetch_add(&deg[y], 1u, __ATOMIC_RELAXED);
                ++kept;
            }
        }
        kept_t[(size_t)t] = kept;
    });
    for (uint64_t c : kept_t) g.m += c;
    g.offs.assign((size_t)g.n + 1, 0);
    for (uint32_t v = 0; v < g.n; ++v) {
        g.offs[v + 1] = g.offs[v] + deg[v];
        g.max_degree = std::max(g.max_degree, deg[v]);
    }
    g.nbr.assign(g.offs[g.n], 0);
    g.elab.assign(g.offs[g.n], 0);
    std::vector<uint32_t> src_edge(g.offs[g.n]);  // input edge of each entry
    {
        std::vector<uint64_t> cursor(g.offs.begin(), g.offs.end() - 1);
        fast::parallel_ranges(M, T, [&](int, size_t k0, size_t k1) {
            for (size_t k = k0; k < k1; ++k) {
                if (!ekeep[k]) continue;
                const uint32_t x = id_map[edges.a(k)], y = id_map[edges.b(k)];
                const uint64_t px = __atomic_fetch_add(&cursor[x], 1ull, __ATOMIC_RELAXED);
                g.nbr[px] = y;
                src_edge[px] = (uint32_t)k;
                const uint64_t py = __atomic_fetch_add(&cursor[y], 1ull, __ATOMIC_RELAXED);
                g.nbr[py] = x;
                src_edge[py] = (uint32_t)k;
            }
        });
    }
    fast::parallel_ranges(g.n, T, [&](int, size_t b0, size_t b1) {
        std::vector<uint64_t> key;
        for (size_t v = b0; v < b1; ++v) {
            const uint64_t b = g.offs[v], e = g.offs[v + 1];
            key.clear();
            for (uint64_t i = b; i < e; ++i) key.push_back(((uint64_t)g.nbr[i] << 32) | (uint64_t)src_edge[i]);
            std::sort(key.begin(), key.end());
            for (uint64_t i = b; i < e; ++i) {
                g.nbr[i] = (uint32_t)(key[i - b] >> 32);
                g.elab[i] = edges.l((size_t)(key[i - b] & 0xffffffffu));
            }
        }
    });
    // ---- largest label class ----
    for (size_t k = 0; k < vlabels.size(); ++k)
        if (vfreq[k]) g.max_label_freq = std::max(g.max_label_freq, (uint32_t)vcount[k]);
    // ---- 1-edge pattern endpoint sets, counted per vertex ----
    const fast::LabelIndex fv(g.freq_vlabels), fe(g.freq_elabels);
    const size_t NL = g.freq_vlabels.size(), NE = g.freq_elabels.size();
    const size_t cells = NL * NE * NL;
    std::vector<std::vector<uint32_t>> cnt_a((size_t)T), cnt_b((size_t)T);
    std::vector<std::unordered_map<uint64_t, std::pair<uint32_t, uint32_t>>> cnt_h((size_t)T);
    const bool dense = cells <= (1u << 22);
    std::atomic<int> used(0);
    fast::parallel_ranges(g.n, T, [&](int t, size_t b0, size_t b1) {
        used.fetch_add(1);
        if (dense) {
            cnt_a[(size_t)t].assign(cells, 0);
            cnt_b[(size_t)t].assign(cells, 0);
        }
        std::vector<uint64_t> seen;
        for (size_t x = b0; x < b1; ++x) {
            const uint64_t la = (uint64_t)fv(g.vlabel[x]);
            seen.clear();
            for (uint64_t i = g.offs[x]; i < g.offs[x + 1]; ++i)
                seen.push_back(((uint64_t)fe(g.elab[i]) << 32) | (uint64_t)fv(g.vlabel[g.nbr[i]]));
            std::sort(seen.begin(), seen.end());
            seen.erase(std::unique(seen.begin(), seen.end()), seen.end());
            for (uint64_t s : seen) {
                const uint64_t el = s >> 32, lb = s & 0xffffffffu;
                // x is an endpoint of the triple (min label, el, max label) on its own label's side
                const bool side_a = la <= lb;
                const uint64_t lo = side_a ? la : lb, hi = side_a ? lb : la;
                const uint64_t cell = (lo * NE + el) * NL + hi;
                if (dense) (side_a ? cnt_a : cnt_b)[(size_t)t][cell]++;
                else {
                    auto &c = cnt_h[(size_t)t][cell];
                    (side_a ? c.first : c.second)++;
                }
            }
        }
    });
    std::vector<std::pair<uint32_t, uint32_t>> total;
    std::vector<uint64_t> present;
    if (dense) {
        total.assign(cells, {0, 0});
        for (int t = 0; t < used.load(); ++t)
            for (size_t c = 0; c < cells; ++c) {
                total[c].first += cnt_a[(size_t)t][c];
                total[c].second += cnt_b[(size_t)t][c];
            }
        for (size_t c = 0; c < cells; ++c)
            if (total[c].first || total[c].second) present.push_back(c);
    } else {
        std::unordered_map<uint64_t, std::pair<uint32_t, uint32_t>> all;
        for (auto &h : cnt_h)
            for (auto &kv : h) {
                all[kv.first].first += kv.second.first;
                all[kv.first].second += kv.second.second;
            }
        for (auto &kv : all) present.push_back(kv.first);
        std::sort(present.begin(), present.end());
        total.resize(present.size());
        for (size_t k = 0; k < present.size(); ++k) total[k] = all[present[k]];
    }
    // cells ascend in (la, el, lb) dense order == ascending original labels
    for (size_t k = 0; k < present.size(); ++k) {
        const uint64_t c = present[k];
        const auto &tc = dense ? total[(size_t)c] : total[k];
        const size_t la = (size_t)(c / (NE * NL)), el = (size_t)((c / NL) % NE), lb = (size_t)(c % NL);
        const uint32_t ca = tc.first, cb = la == lb ? tc.first : tc.second;
        if ((int64_t)ca >= tau && (int64_t)cb >= tau)
            g.edge_pairs.push_back({g.freq_vlabels[la], g.freq_elabels[el], g.freq_vlabels[lb], ca, cb});
    }
    return g;
}

// Same LgGraph as build_pruned(raw, tau).
inline LgGraph build_pruned_fast(const RawLg &raw, int tau, int threads = fast::default_threads()) {
    return build_pruned_edges(raw.vlabel, EdgeTuples{raw.edges}, tau, threads);
}

inline LgGraph load_lg_fast(const std::string &path, int tau, int threads = fast::default_threads()) {
    std::vector<char> buf;
    if (!detail::read_file(path, buf)) throw LgError(2, "cannot open graph file " + path);
    RawLg raw = parse_lg_text_fast(buf.data(), buf.size(), threads);
    return build_pruned_fast(raw, tau, threads);
}

}  // namespace tfsm
