#include "miner.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>

#include <unistd.h>

#include "host/lg_fast.hpp"
#include "host/subpattern.hpp"

namespace tfsm {

namespace {

struct Node {
    Pattern pat;
    EvalResult res;
    bool pruned = false;   // a sub-pattern with one edge less is infrequent: decided without search
    std::vector<PushSource> push;  // frequent sub-patterns with one edge less (previous level)
    Level *lvl = nullptr;  // device memory holding this pattern's final domains
    int idx = 0;           // index inside lvl
};

// Runs `work` on `threads` host threads (the caller's and the loader's persistent workers):
// creating a thread per core for every level would cost as much as the level's extension.
class Pool {
  public:
    explicit Pool(int threads) : threads_(std::max(1, threads)) {}
    void run(const std::function<void()> &work) {
        if (threads_ == 1) {
            work();
            return;
        }
        const std::function<void(size_t)> task = [&](size_t) { work(); };
        fast::Workers::get().run((size_t)threads_, task);
    }

  private:
    int threads_;
};

// A level's host growth, computed while the GPU evaluates the level.  A pattern's children
// (rightmost extension + canonical check), its canonical key and vertex order, and its children's
// one-edge-smaller sub-patterns depend only on the pattern, not on its support: a helper thread
// computes them on the host workers for every candidate while the level's engine calls run.  Once
// the results are in (`publish`), candidates that turned out infrequent are skipped; the rest are
// finished by `join`.  Candidates already decided infrequent (pruned) are never extended.
class Growth {
  public:
    Growth(const std::vector<Node> &level, const ExtendContext &ctx, Pool &pool, bool want_subs)
        : ctx_(ctx), pool_(pool), want_subs_(want_subs) {
        const size_t n = level.size();
        pats_.reserve(n);
        for (auto &nd : level) {
            pats_.push_back(nd.pat);
            pruned_.push_back(nd.pruned ? 1 : 0);
        }
        frequent_.assign(n, 0);
        kids_.assign(n, {});
        extended_.assign(n, 0);
        keys_.assign(n, {});
        orders_.assign(n, {});
        subs_.assign(n, {});
        subs_done_.assign(n, 0);
        th_ = std::thread([this]() {
            try {
                work();
            } catch (...) {
                err_ = std::current_exception();
            }
        });
    }
    ~Growth() {
        if (th_.joinable()) {
            known_.store(true, std::memory_order_release);  // every frequent_ flag still 0: stop early
            th_.join();
        }
    }
    Growth(const Growth &) = delete;
    Growth &operator=(const Growth &) = delete;

    // The level's results are in (candidates beyond `level`'s size were dropped): wait for the
    // helper, then finish what it skipped for frequent candidates.
    void join(const std::vector<Node> &level) {
        for (size_t i = 0; i < pats_.size(); ++i) frequent_[i] = i < level.size() && level[i].res.frequent ? 1 : 0;
        known_.store(true, std::memory_order_release);
        th_.join();
        if (err_) std::rethrow_exception(err_);
        for (size_t i = 0; i < pats_.size(); ++i)
            if (frequent_[i]) {
                if (!extended_[i]) extend(i);
                if (want_subs_ && !subs_done_[i]) subs(i);
            }
    }

    // after join: the children of candidate i (frequent ones only), moved out
    std::vector<Pattern> take_kids(size_t i) { return frequent_[i] ? std::move(kids_[i]) : std::vector<Pattern>(); }
    const std::string &key(size_t i) const { return keys_[i]; }
    const std::vector<int> &order(size_t i) const { return orders_[i]; }
    const std::vector<SubPattern> &child_subs(size_t i, size_t j) const { return subs_[i][j]; }

  private:
    bool dropped(size_t i) const {  // known to be infrequent
        return pruned_[i] || (known_.load(std::memory_order_acquire) && !frequent_[i]);
    }
    void extend(size_t i) {
        kids_[i].clear();
        extend_pattern(pats_[i], ctx_, kids_[i]);
        extended_[i] = 1;
    }
    void subs(size_t i) {
        subs_[i].resize(kids_[i].size());
        for (size_t j = 0; j < kids_[i].size(); ++j) one_edge_smaller(kids_[i][j], subs_[i][j]);
        subs_done_[i] = 1;
    }
    void work() {
        const size_t n = pats_.size();
        std::atomic<size_t> k(0);
        const std::function<void()> first = [&]() {
            for (size_t i; (i = k.fetch_add(1)) < n;) {
                if (pruned_[i]) continue;
                if (want_subs_) keys_[i] = canonical_key(small_graph(pats_[i]), &orders_[i]);
                if (!dropped(i)) extend(i);
            }
        };
        pool_.run(first);
        if (!want_subs_) return;
        k.store(0);
        const std::function<void()> second = [&]() {
            for (size_t i; (i = k.fetch_add(1)) < n;)
                if (extended_[i] && !dropped(i)) subs(i);
        };
        pool_.run(second);
    }

    const ExtendContext &ctx_;
    Pool &pool_;
    const bool want_subs_;
    std::vector<Pattern> pats_;
    std::vector<char> pruned_, frequent_, extended_, subs_done_;
    std::atomic<bool> known_{false};
    std::vector<std::vector<Pattern>> kids_;
    std::vector<std::string> keys_;
    std::vector<std::vector<int>> orders_;
    std::vector<std::vector<std::vector<SubPattern>>> subs_;
    std::exception_ptr err_;
    std::thread th_;  // joined in the destructor, before the members above go
};

// Resident host memory of this process in MB (Linux; 0 elsewhere), for the verbose level lines.
double host_rss_mb() {
    FILE *f = std::fopen("/proc/self/statm", "r");
    if (!f) return 0;
    long pages = 0, resident = 0;
    const int got = std::fscanf(f, "%ld %ld", &pages, &resident);
    std::fclose(f);
    return got == 2 ? (double)resident * (double)sysconf(_SC_PAGESIZE) / 1048576.0 : 0.0;
}

}  // namespace

void mine(GpuEngine &eng, const LgGraph &g, const MineOptions &opt, std::vector<MinedPattern> &out, MineStats &st) {
    auto t0 = std::chrono::steady_clock::now();
    out.clear();
    st = MineStats();
    const int threads = opt.host_threads > 0 ? opt.host_threads : fast::default_threads();
    // growth runs beside the engine calls: two threads fewer, so the host thread that prepares
    // and launches the device work keeps a core
    Pool pool(std::max(1, threads - 2));
    ExtendContext ctx;
    ctx.freq_elabels = g.freq_elabels;
    ctx.max_nodes = opt.max_nodes;
    for (auto &ep : g.edge_pairs) {
        ctx.neighbor_labels[ep.la].insert(ep.lb);
        ctx.neighbor_labels[ep.lb].insert(ep.la);
    }
    const uint32_t tau = (uint32_t)std::max(opt.tau, 0);
    const bool verbose = std::getenv("TFSM_VERBOSE") != nullptr;  // per-engine-call summary on stderr
    // Sub-pattern pruning needs every frequent pattern of a level to be generated.  With more than
    // one frequent edge label the reference's canonical check orders forward edges by a relation
    // that is not a strict weak ordering (parallel/canonical.h:40-44), and its mined sets are not
    // closed under sub-patterns; the pruning is then off so that the output stays the reference's.
    const bool prune_subpatterns = opt.subpattern_pruning && g.freq_elabels.size() <= 1;

    // Levels own device memory; a level is released once its children are evaluated.
    std::vector<std::unique_ptr<Level>> prev_levels, cur_levels;

    auto out_of_time = [&]() {
        if (opt.engine.time_limit_s <= 0) return false;
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (s > opt.engine.time_limit_s) st.complete = false;
        return !st.complete;
    };
    // Evaluates a level's candidates.  Batched: consecutive candidates go into one engine call,
    // at most max_batch of them (their parents and push-down sources may come from any of the
    // previous level's calls).  Candidates left when the time limit stops the run are dropped.
    //
    // With call_ms set, the number of candidates per call also follows the calls' cost: a call of
    // k candidates that took t > call_ms makes the following calls take k * call_ms / t of them (at
    // least 4), and a full call that took less doubles that limit again, up to max_batch.  The
    // limit carries over to the next level, whose candidates cost more.  Expensive levels gain
    // from small calls: a call's searches share the GPU, so every pattern waits longer for the
    // searches that decide it, and its long failing searches (hub vertices) run on meanwhile; cheap
    // levels keep one call each.
    size_t batch_limit = 0;
    auto evaluate_level = [&](std::vector<Node> &nodes, const std::vector<int> &parent_of,
                              const std::vector<Node> *parents) {
        if (nodes.empty()) return;
        const int lvl_no = st.levels + 1;
        const EngineOptions &eo = opt.engine_for(lvl_no);
        const double wall_before = eng.times().engine_ms;
        auto parent_ref = [&](size_t i) -> LevelRef {
            if (!parents || parent_of[i] < 0) return LevelRef{};
            const Node &pn = (*parents)[(size_t)parent_of[i]];
            return LevelRef{pn.lvl, pn.idx};
        };
        // sub-pattern pruning decided some candidates already; the engine evaluates the rest
        std::vector<size_t> todo;
        for (size_t i = 0; i < nodes.size(); ++i) {
            if (!nodes[i].pruned) {
                todo.push_back(i);
                continue;
            }
            nodes[i].res = EvalResult();
            nodes[i].res.mni.assign((size_t)nodes[i].pat.size(), 0);
            nodes[i].res.by_filter = true;
            st.evaluations++;
            st.pruned++;
        }
        if (opt.batched) {
            const size_t cap = std::max<size_t>(1, eo.max_batch);
            if (batch_limit == 0 || eo.call_ms <= 0) batch_limit = cap;
            batch_limit = std::min(batch_limit, cap);
            size_t b0 = 0;
            while (b0 < todo.size()) {
                if (out_of_time()) {
                    nodes.resize(todo[b0]);
                    break;
                }
                const size_t b1 = std::min(todo.size(), b0 + batch_limit);
                std::vector<const Pattern *> pats;
                std::vector<LevelRef> par;
                for (size_t k = b0; k < b1; ++k) {
                    const size_t i = todo[k];
                    pats.push_back(&nodes[i].pat);
                    par.push_back(parent_ref(i));
                }
                cur_levels.emplace_back(new Level);
                std::vector<EvalResult> res;
                const KernelTimes before = eng.times();
                const double search_before = before.search_ms;
                std::vector<std::vector<PushSource>> pushes;
                for (size_t kk = b0; kk < b1; ++kk) pushes.push_back(nodes[todo[kk]].push);
                eng.evaluate(pats, par, tau, eo, *cur_levels.back(), res, &pushes);
                st.engine_calls++;
                st.evaluations += b1 - b0;
                if (eo.call_ms > 0) {
                    const double call = eng.times().engine_ms - before.engine_ms;
                    const size_t k = b1 - b0;
                    if (call > eo.call_ms)
                        batch_limit = std::min(batch_limit, std::max<size_t>(std::min<size_t>(4, cap),
                                                                             (size_t)((double)k * eo.call_ms / call)));
                    else if (k >= batch_limit)
                        batch_limit = std::min(cap, 2 * batch_limit);
                }
                if (verbose) {
                    uint64_t mx = 0, srch = 0, nf = 0;
                    for (auto &r : res) {
                        mx = std::max<uint64_t>(mx, r.max_steps);
                        srch += r.searches;
                        nf += r.frequent ? 1 : 0;
                    }
                    std::fprintf(stderr,
                                 "[level %d] %zu patterns (%llu frequent), engine call %.3f ms (init %.3f, refine "
                                 "%.3f, search %.3f), %llu searches, longest search %llu chunk steps\n",
                                 st.levels + 1, b1 - b0, (unsigned long long)nf, eng.times().engine_ms - before.engine_ms,
                                 eng.times().init_ms - before.init_ms, eng.times().refine_ms - before.refine_ms,
                                 eng.times().search_ms - search_before, (unsigned long long)srch,
                                 (unsigned long long)mx);
                    const KernelTimes &now = eng.times();
                    std::fprintf(stderr,
                                 "          host phases ms: desc %.3f pools %.3f init+refine %.3f plans %.3f items %.3f "
                                 "search %.3f results %.3f\n",
                                 now.phase_ms[0] - before.phase_ms[0], now.phase_ms[1] - before.phase_ms[1],
                                 now.phase_ms[2] - before.phase_ms[2], now.phase_ms[3] - before.phase_ms[3],
                                 now.phase_ms[4] - before.phase_ms[4], now.phase_ms[5] - before.phase_ms[5],
                                 now.phase_ms[6] - before.phase_ms[6]);
                    std::fprintf(stderr,
                                 "          passes %llu (%llu set aside), split: %llu searches, %llu tasks\n",
                                 (unsigned long long)(now.search_passes - before.search_passes),
                                 (unsigned long long)(now.abandoned - before.abandoned),
                                 (unsigned long long)(now.split_groups - before.split_groups),
                                 (unsigned long long)(now.split_tasks - before.split_tasks));
                }
                for (size_t k = b0; k < b1; ++k) {
                    const size_t i = todo[k];
                    nodes[i].res = std::move(res[k - b0]);
                    nodes[i].lvl = cur_levels.back().get();
                    nodes[i].idx = (int)(k - b0);
                }
                b0 = b1;
            }
        } else {
            for (size_t i : todo) {
                if (out_of_time()) {
                    nodes.resize(i);
                    break;
                }
                st.evaluations++;
                std::vector<const Pattern *> pats{&nodes[i].pat};
                const std::vector<LevelRef> par{parent_ref(i)};
                cur_levels.emplace_back(new Level);
                std::vector<EvalResult> res;
                const std::vector<std::vector<PushSource>> pushes{nodes[i].push};
                eng.evaluate(pats, par, tau, eo, *cur_levels.back(), res, &pushes);
                st.engine_calls++;
                nodes[i].res = std::move(res[0]);
                nodes[i].lvl = cur_levels.back().get();
                nodes[i].idx = 0;
            }
        }
        for (auto &nd : nodes) {
            st.searches += nd.res.searches;
            st.steps += nd.res.steps;
            st.by_filter += nd.res.by_filter ? 1 : 0;
        }
        if ((size_t)lvl_no >= st.level_ms.size()) st.level_ms.resize((size_t)lvl_no + 1, 0.0);
        st.level_ms[(size_t)lvl_no] += eng.times().engine_ms - wall_before;
    };

    // level 1: the frequent 1-edge patterns (frequent by construction of the pair table,
    // parallel/grami.h:116-153); evaluated on the GPU for their domains
    std::vector<Node> level;
    for (auto &ep : g.edge_pairs) {
        Node nd;
        nd.pat.push(DfsCode{0, 1, ep.la, ep.el, ep.lb});
        level.push_back(std::move(nd));
    }
    const bool want_subs = opt.subpattern_pruning;
    std::unique_ptr<Growth> growth(new Growth(level, ctx, pool, want_subs));
    evaluate_level(level, std::vector<int>(level.size(), -1), nullptr);
    for (auto &nd : level) {
        if (!opt.engine.exact) nd.res.frequent = true;
        else nd.res.frequent = nd.res.support >= tau;
    }
    growth->join(level);
    st.levels = level.empty() ? 0 : 1;
    while (!level.empty()) {
        for (auto &nd : level)
            if (nd.res.frequent) out.push_back({nd.pat, nd.res});
        auto te = std::chrono::steady_clock::now();
        std::vector<Node> next;
        std::vector<int> parent_of;
        std::vector<size_t> child_no;  // by child: its position among its parent's children
        for (size_t i = 0; i < level.size(); ++i) {
            std::vector<Pattern> kids = growth->take_kids(i);
            for (size_t j = 0; j < kids.size(); ++j) {
                Node nd;
                nd.pat = std::move(kids[j]);
                next.push_back(std::move(nd));
                parent_of.push_back((int)i);
                child_no.push_back(j);
            }
        }
        if (want_subs && !next.empty()) {
            // For every child, its one-edge-smaller sub-patterns (keys and canonical vertex orders
            // from the growth), matched against this level's evaluated patterns:
            //   * one evaluated and infrequent: the child is infrequent (MNI is anti-monotone);
            //   * one missing from a complete level (single edge label): infrequent as well;
            //   * the frequent ones bound the child's domains (up to kMaxPushSources of them).
            // An unknown (empty) key, of a pattern too symmetric for the key's search, decides nothing:
            // such a sub-pattern neither prunes nor bounds the child (isomorphic patterns are all
            // unknown, so no frequent pattern is missed).
            std::unordered_map<std::string, size_t> evaluated;
            for (size_t i = 0; i < level.size(); ++i)
                if (!level[i].pruned && !growth->key(i).empty()) evaluated.emplace(growth->key(i), i);
            for (size_t i = 0; i < next.size(); ++i) {
                Node &child = next[i];
                for (const SubPattern &sp : growth->child_subs((size_t)parent_of[i], child_no[i])) {
                    if (sp.key.empty()) continue;
                    auto it = evaluated.find(sp.key);
                    if (it == evaluated.end()) {
                        if (prune_subpatterns) child.pruned = true;
                        if (child.pruned) break;
                        continue;
                    }
                    const Node &sn = level[it->second];
                    if (!sn.res.frequent) {
                        child.pruned = true;
                        break;
                    }
                    if (it->second == (size_t)parent_of[i] || !sn.lvl) continue;
                    if (child.push.size() >= (size_t)kMaxPushSources) continue;
                    PushSource src;
                    src.at = LevelRef{sn.lvl, sn.idx};
                    for (int u = 0; u < (int)sizeof(src.vertex); ++u) src.vertex[u] = -1;
                    const std::vector<int> &ord = growth->order(it->second);
                    for (int u = 0; u < child.pat.size() && u < (int)sizeof(src.vertex); ++u)
                        if (sp.pos_of[(size_t)u] >= 0) src.vertex[u] = (int8_t)ord[(size_t)sp.pos_of[(size_t)u]];
                    child.push.push_back(src);
                }
                if (child.pruned) child.push.clear();
            }
        }
        st.extend_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - te).count();
        if (next.empty()) break;
        if (verbose) {
            size_t pruned = 0, dfree = 0, dtotal = 0;
            for (auto &nd : next) pruned += nd.pruned ? 1 : 0;
            eng.device_memory(dfree, dtotal);
            std::fprintf(stderr, "[level %d starts] %zu candidates (%zu decided by sub-patterns), host RSS %.0f MB, "
                                 "device free %.0f of %.0f MB\n",
                         st.levels + 1, next.size(), pruned, host_rss_mb(), dfree / 1048576.0, dtotal / 1048576.0);
        }
        growth.reset(new Growth(next, ctx, pool, want_subs));  // runs during the next level's engine calls
        prev_levels = std::move(cur_levels);
        cur_levels.clear();
        evaluate_level(next, parent_of, &level);
        prev_levels.clear();  // parents' device memory
        const auto tj = std::chrono::steady_clock::now();
        growth->join(next);
        st.extend_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tj).count();
        level = std::move(next);
        st.levels++;
    }
    st.frequent = out.size();
    st.mine_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

bool write_results(const std::string &path, const std::vector<MinedPattern> &pats) {
    std::ofstream f(path);
    if (!f) return false;
    for (auto &mp : pats) f << mp.pat.to_results_block();
    return (bool)f;
}

}  // namespace tfsm
