// C-ABI boundary (declarations and the reference interface each entry point replaces:
// include/tfsm.h).  Exceptions never cross it; errors become status codes + tfsm_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

#include "../../include/tfsm.h"
#include "engine.hpp"
#if !defined(TFSM_SIMT_EMULATION)
#include "cuda/ingest.hpp"
#endif
#include "host/lg_fast.hpp"
#include "miner.hpp"
#include "noalloc.hpp"

struct tfsm_graph {
    uint64_t serial = next_serial();  // unique per handle (an address may be reused after a free)
    static uint64_t next_serial() {
        static std::atomic<uint64_t> n(0);
        return ++n;
    }
    tfsm::LgGraph lg;
    std::unique_ptr<tfsm::GpuEngine> eng;
    tfsm::EngineOptions opt;  // tuning knobs (tfsm_set_options), order policy and cost model
    int tau = 0;
    double load_ms = 0;
    bool device_ingest = false;  // the device graph was built on the GPU (lg holds no adjacency)
    bool recording = false;
    std::vector<std::pair<bool, tfsm_options>> level_opt;  // tfsm_set_level_options, by level
    mutable std::vector<float> records;  // tfsm_record_orders: 33 floats per record
    std::mutex mu;
};

struct tfsm_cost_model {
    std::unique_ptr<tfsm::CostModel> m;
};

struct tfsm_domains {
    uint64_t graph = 0;               // serial of the graph whose pools these are
    tfsm::Level lvl;                  // the call's bitmap pools
    std::vector<tfsm::Pattern> pats;  // by position in the call (for the sub-pattern check)
    std::vector<int> slot;            // by position in the call: index in lvl, or -1 (not evaluated)
};

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

template <class F>
int guarded(F &&f) {
    try {
        g_err.clear();
        return f();
    } catch (const tfsm::LgError &e) {
        return fail(e.code, e.what());
    } catch (const tfsm::EngineError &e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return fail(TFSM_ERR_INTERNAL, "host out of memory");
    } catch (const std::exception &e) {
        return fail(TFSM_ERR_INTERNAL, e.what());
    } catch (...) {
        return fail(TFSM_ERR_INTERNAL, "unknown error");
    }
}

// Validates a DFS code sequence and builds the pattern (Pattern::add_edge semantics).
bool build_pattern(const tfsm_pattern *tp, tfsm::Pattern &p, std::string &why) {
    if (!tp || tp->n_codes <= 0 || !tp->codes) {
        why = "pattern has no DFS codes";
        return false;
    }
    for (int i = 0; i < tp->n_codes; ++i) {
        const tfsm_dfs_code &c = tp->codes[i];
        tfsm::DfsCode d{c.from, c.to, c.from_label, c.edge_label, c.to_label};
        const int n = p.size();
        if (i == 0) {
            if (c.from != 0 || c.to != 1) {
                why = "first DFS code must be (0,1,...)";
                return false;
            }
        } else {
            const bool fwd = c.to == n && c.from >= 0 && c.from < n;
            const bool bwd = c.from >= 0 && c.from < n && c.to >= 0 && c.to < n && c.from != c.to;
            if (!fwd && !bwd) {
                why = "DFS code " + std::to_string(i) + " neither extends nor closes the pattern";
                return false;
            }
            if (p.label(c.from) != c.from_label || (bwd && p.label(c.to) != c.to_label)) {
                why = "DFS code " + std::to_string(i) + " has vertex labels inconsistent with earlier codes";
                return false;
            }
            if (bwd && p.adjacent(c.from, c.to)) {
                why = "DFS code " + std::to_string(i) + " repeats an edge";
                return false;
            }
            if (fwd && n >= TFSM_MAX_PATTERN_VERTICES) {
                why = "pattern has more than 32 vertices";
                return false;
            }
        }
        p.push(d);
    }
    return true;
}

void fill_result(const tfsm::EvalResult &r, int n, tfsm_result *out) {
    std::memset(out, 0, sizeof(*out));
    out->status = TFSM_OK;
    out->frequent = r.frequent ? 1 : 0;
    out->n_vertices = n;
    out->decided_by_filter = r.by_filter ? 1 : 0;
    out->support = r.support;
    for (int i = 0; i < n && i < TFSM_MAX_PATTERN_VERTICES; ++i) out->mni[i] = r.mni[(size_t)i];
    out->searches = r.searches;
    out->steps = r.steps;
}

const char *const kKnobRules =
    "split_slice, chunk_words, max_batch and isect_ratio must be >= 1; refine_rounds <= 32; refine_scope 0 or 1; "
    "hub_parts in 1..32; "
    "time_limit_s and call_ms >= 0; search_lanes 0, 4, 8 or 32";

bool knobs_valid(const tfsm_options &o) {
    return o.split_slice >= 1 && o.chunk_words >= 1 && o.refine_rounds <= 32 && o.max_batch >= 1 &&
           o.hub_parts >= 1 && o.hub_parts <= 32 && o.isect_ratio >= 1 && o.time_limit_s >= 0 && o.call_ms >= 0 &&
           o.refine_scope <= 1 &&
           (o.search_lanes == 0 || o.search_lanes == 4 || o.search_lanes == 8 || o.search_lanes == 32);
}

// The speed-only knobs of `o` (not the time limit, which belongs to the whole run).
void apply_knobs(const tfsm_options &o, tfsm::EngineOptions &e) {
    e.step_budget = o.step_budget;
    e.split_slice = o.split_slice;
    e.chunk_words = o.chunk_words;
    e.refine_rounds = o.refine_rounds;
    e.max_batch = o.max_batch;
    e.hub_span = o.hub_span;
    e.hub_parts = o.hub_parts;
    e.search_lanes = o.search_lanes == 0 ? 32 : o.search_lanes;
    e.rank_window = o.rank_window;
    e.call_ms = o.call_ms;
    e.isect_ratio = o.isect_ratio;
    e.refine_scope = o.refine_scope;
}

// The engine's knobs as a full tfsm_options.
tfsm_options knobs_of(const tfsm::EngineOptions &e) {
    tfsm_options o;
    std::memset(&o, 0, sizeof(o));
    o.struct_size = sizeof(tfsm_options);
    o.step_budget = e.step_budget;
    o.split_slice = e.split_slice;
    o.chunk_words = e.chunk_words;
    o.refine_rounds = e.refine_rounds;
    o.max_batch = e.max_batch;
    o.hub_span = e.hub_span;
    o.hub_parts = e.hub_parts;
    o.time_limit_s = e.time_limit_s;
    o.search_lanes = e.search_lanes;
    o.rank_window = e.rank_window;
    o.call_ms = e.call_ms;
    o.isect_ratio = e.isect_ratio;
    o.refine_scope = e.refine_scope;
    return o;
}

// A caller's options of struct_size bytes over the current ones (fields past struct_size keep
// their values); false when struct_size is outside [TFSM_OPTIONS_MIN_SIZE, sizeof(tfsm_options)].
bool read_options(const tfsm_options *in, const tfsm::EngineOptions &cur, tfsm_options &out) {
    if (in->struct_size < TFSM_OPTIONS_MIN_SIZE || in->struct_size > sizeof(tfsm_options)) return false;
    out = knobs_of(cur);
    std::memcpy(&out, in, in->struct_size);
    out.struct_size = sizeof(tfsm_options);
    return true;
}

const char *const kSizeRule = "tfsm_options.struct_size must be set to sizeof(tfsm_options) (at least "
                              "TFSM_OPTIONS_MIN_SIZE, at most the library's own size)";

constexpr uint32_t kHubStepBudget = 64;  // default step budget of hub graphs (finish_graph)

tfsm::EngineOptions engine_options(const tfsm_graph *g, uint32_t flags) {
    tfsm::EngineOptions o = g->opt;
    o.exact = (flags & TFSM_FLAG_EXACT) != 0;
    if (flags & TFSM_FLAG_NO_SPLIT) o.split = false;
    o.records = g->recording ? &g->records : nullptr;
    return o;
}

int finish_graph(std::unique_ptr<tfsm_graph> &g, int tau, std::chrono::steady_clock::time_point t0,
                 tfsm_graph **out) {
    g->tau = tau;
    const auto t_prune = std::chrono::steady_clock::now();
    if (!g->eng) g->eng.reset(new tfsm::GpuEngine(g->lg, 0));
    // Hub graphs (a vertex with more than four hub spans of neighbours) split searches later: with
    // hubs of ~40k neighbours a 16-step budget writes ~130 M split tasks per mining run, and 64
    // steps measured 12% faster there; graphs without such hubs keep 16 (64 measured 19% slower on
    // one with hubs of 1.4k).
    if (g->lg.max_degree > 4 * g->opt.hub_span) g->opt.step_budget = kHubStepBudget;
    g->load_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (std::getenv("TFSM_VERBOSE"))
        std::fprintf(stderr, "[load] %s: parse + prune %.3f ms, engine %.3f ms (%s)\n",
                     g->device_ingest ? "device" : "host",
                     std::chrono::duration<double, std::milli>(t_prune - t0).count(), g->eng->upload_ms(),
                     g->eng->load_breakdown().c_str());
    *out = g.release();
    return TFSM_OK;
}

// Graph ingestion runs on the GPU (cuda/ingest.hpp) unless TFSM_INGEST=host selects the host
// loader (host/lg_fast.hpp, then renumbering and upload in the engine); both build the same
// device graph.
// Without a CUDA device the host loader runs, so that malformed input is still reported as such
// before the engine reports the missing device.
bool device_ingest() {
#if defined(TFSM_SIMT_EMULATION)
    return false;
#else
    const char *e = std::getenv("TFSM_INGEST");
    if (e && std::strcmp(e, "host") == 0) return false;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        return false;
    }
    return true;
#endif
}

}  // namespace

extern "C" {

int tfsm_graph_load(const char *path, int32_t tau, tfsm_graph **out) {
    return guarded([&]() -> int {
        if (!path || !out) return fail(TFSM_ERR_ARG, "null argument");
        *out = nullptr;
        auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<tfsm_graph> g(new tfsm_graph);
#if !defined(TFSM_SIMT_EMULATION)
        if (device_ingest()) {
            g->device_ingest = true;
            const std::string file(path);
            g->eng.reset(new tfsm::GpuEngine(
                [&](CUstream_st *s, tfsm::DeviceGraphBuild &b) { tfsm::ingest_lg_file(file, tau, s, b); }, g->lg, 0));
            return finish_graph(g, tau, t0, out);
        }
#endif
        g->lg = tfsm::load_lg_fast(path, tau);
        return finish_graph(g, tau, t0, out);
    });
}

int tfsm_graph_from_edges(uint32_t n_vertices, const int32_t *vlabels, uint64_t n_edges, const uint32_t *src,
                          const uint32_t *dst, const int32_t *elabels, int32_t tau, tfsm_graph **out) {
    return guarded([&]() -> int {
        if (!out || (n_vertices && !vlabels) || (n_edges && (!src || !dst || !elabels)))
            return fail(TFSM_ERR_ARG, "null argument");
        *out = nullptr;
        auto t0 = std::chrono::steady_clock::now();
#if !defined(TFSM_SIMT_EMULATION)
        if (device_ingest()) {
            std::unique_ptr<tfsm_graph> g(new tfsm_graph);
            g->device_ingest = true;
            g->eng.reset(new tfsm::GpuEngine(
                [&](CUstream_st *s, tfsm::DeviceGraphBuild &b) {
                    tfsm::ingest_edge_arrays(n_vertices, vlabels, n_edges, src, dst, elabels, tau, s, b);
                },
                g->lg, 0));
            return finish_graph(g, tau, t0, out);
        }
#endif
        std::atomic<bool> bad(false);
        tfsm::fast::parallel_ranges((size_t)n_edges, tfsm::fast::default_threads(), [&](int, size_t k0, size_t k1) {
            for (size_t k = k0; k < k1 && !bad.load(std::memory_order_relaxed); ++k)
                if (src[k] >= n_vertices || dst[k] >= n_vertices) bad.store(true);
        });
        if (bad) return fail(TFSM_ERR_FORMAT, "edge endpoint out of range");
        const std::vector<int> vl(vlabels, vlabels + n_vertices);
        std::unique_ptr<tfsm_graph> g(new tfsm_graph);
        g->lg = tfsm::build_pruned_edges(vl, tfsm::EdgeArrays{src, dst, elabels, (size_t)n_edges}, tau);
        return finish_graph(g, tau, t0, out);
    });
}

void tfsm_graph_free(tfsm_graph *g) { delete g; }

int tfsm_graph_info(const tfsm_graph *g, tfsm_graph_info_t *info) {
    return guarded([&]() -> int {
        if (!g || !info) return fail(TFSM_ERR_ARG, "null argument");
        std::memset(info, 0, sizeof(*info));
        info->n_vertices = g->lg.n;
        info->n_edges = g->lg.m;
        info->n_frequent_vertex_labels = (uint32_t)g->lg.freq_vlabels.size();
        info->n_frequent_edge_labels = (uint32_t)g->lg.freq_elabels.size();
        info->n_frequent_edge_patterns = (uint32_t)g->lg.edge_pairs.size();
        info->max_degree = g->lg.max_degree;
        info->device_bytes = g->eng->graph_bytes();
        info->load_ms = g->load_ms;
        info->load_h2d_bytes = g->eng->load_h2d_bytes();
        return TFSM_OK;
    });
}

int tfsm_graph_export(const tfsm_graph *g, const tfsm_graph_arrays *a) {
    return guarded([&]() -> int {
        if (!g || !a) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(const_cast<tfsm_graph *>(g)->mu);
        g->eng->export_graph(a->row_off, a->col, a->elab, a->label_start, a->lab_off, a->label_mean_degree);
        if (a->vlabels) std::copy(g->lg.freq_vlabels.begin(), g->lg.freq_vlabels.end(), a->vlabels);
        if (a->elabels) std::copy(g->lg.freq_elabels.begin(), g->lg.freq_elabels.end(), a->elabels);
        if (a->edge_patterns)
            for (size_t i = 0; i < g->lg.edge_pairs.size(); ++i) {
                const tfsm::EdgePair &e = g->lg.edge_pairs[i];
                a->edge_patterns[i] = tfsm_edge_pattern{e.la, e.el, e.lb, e.cand_a, e.cand_b};
            }
        return TFSM_OK;
    });
}

namespace {

// `par` is a sub-pattern of `child` under the same vertex numbering (same labels, every edge kept).
bool is_parent_of(const tfsm::Pattern &par, const tfsm::Pattern &child) {
    if (par.size() > child.size()) return false;
    for (int u = 0; u < par.size(); ++u) {
        if (par.vertices[(size_t)u].label != child.vertices[(size_t)u].label) return false;
        for (const tfsm::PEdge &e : par.vertices[(size_t)u].edges) {
            bool kept = false;
            for (const tfsm::PEdge &f : child.vertices[(size_t)u].edges) kept = kept || (f.to == e.to && f.label == e.label);
            if (!kept) return false;
        }
    }
    return true;
}

}  // namespace

int tfsm_evaluate_level(tfsm_graph *g, const tfsm_pattern *patterns, int32_t n, int32_t tau, uint32_t flags,
                        const tfsm_parent *parents, tfsm_result *results, tfsm_domains **out) {
    return guarded([&]() -> int {
        if (out) *out = nullptr;
        if (!g || (n > 0 && (!patterns || !results)) || n < 0) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(g->mu);
        std::unique_ptr<tfsm_domains> keep(new tfsm_domains);
        keep->graph = g->serial;
        keep->pats.resize((size_t)n);
        keep->slot.assign((size_t)n, -1);
        std::vector<const tfsm::Pattern *> ptrs;
        std::vector<tfsm::LevelRef> par;
        std::vector<int> idx;
        for (int i = 0; i < n; ++i) {
            std::string why;
            std::memset(&results[i], 0, sizeof(tfsm_result));
            tfsm::Pattern &p = keep->pats[(size_t)i];
            tfsm::LevelRef ref;
            bool ok = build_pattern(&patterns[i], p, why);
            if (ok && parents && parents[i].domains) {
                const tfsm_domains *d = parents[i].domains;
                const int j = parents[i].index;
                if (d->graph != g->serial) {
                    ok = false;
                    why = "parent domains belong to another graph";
                } else if (j < 0 || (size_t)j >= d->slot.size() || d->slot[(size_t)j] < 0) {
                    ok = false;
                    why = "parent index names no evaluated pattern of that call";
                } else if (!is_parent_of(d->pats[(size_t)j], p)) {
                    ok = false;
                    why = "parent is not a sub-pattern of the pattern under the same vertex numbering";
                } else {
                    ref = tfsm::LevelRef{&d->lvl, d->slot[(size_t)j]};
                }
            }
            if (!ok) {
                results[i].status = why.find("32 vertices") != std::string::npos ? TFSM_ERR_PATTERN : TFSM_ERR_ARG;
                if (g_err.empty()) g_err = why;  // per-pattern errors are reported in results[i].status
                continue;
            }
            keep->slot[(size_t)i] = (int)ptrs.size();
            ptrs.push_back(&p);
            par.push_back(ref);
            idx.push_back(i);
        }
        if (ptrs.empty()) return TFSM_OK;
        std::vector<tfsm::EvalResult> res;
        g->eng->evaluate(ptrs, par, (uint32_t)std::max(tau, 0), engine_options(g, flags), keep->lvl, res);
        for (size_t k = 0; k < ptrs.size(); ++k) fill_result(res[k], ptrs[k]->size(), &results[idx[k]]);
        if (out) *out = keep.release();
        return TFSM_OK;
    });
}

void tfsm_domains_free(tfsm_domains *d) { delete d; }

int tfsm_evaluate_batch(tfsm_graph *g, const tfsm_pattern *patterns, int32_t n, int32_t tau, uint32_t flags,
                        tfsm_result *results) {
    return tfsm_evaluate_level(g, patterns, n, tau, flags, nullptr, results, nullptr);
}

int tfsm_evaluate_support(tfsm_graph *g, const tfsm_pattern *pattern, int32_t tau, uint32_t flags,
                          tfsm_result *out) {
    if (!pattern || !out) return fail(TFSM_ERR_ARG, "null argument");
    const int rc = tfsm_evaluate_batch(g, pattern, 1, tau, flags, out);
    return rc != TFSM_OK ? rc : out->status;
}

int tfsm_mine(tfsm_graph *g, int32_t tau, int32_t max_nodes, uint32_t flags, const char *results_path,
              tfsm_mine_stats *stats) {
    return guarded([&]() -> int {
        if (!g) return fail(TFSM_ERR_ARG, "null graph");
        std::lock_guard<std::mutex> lk(g->mu);
        tfsm::MineOptions opt;
        opt.tau = tau;
        opt.max_nodes = max_nodes;
        opt.batched = (flags & TFSM_FLAG_PLAIN) == 0;
        opt.subpattern_pruning = (flags & TFSM_FLAG_NO_SUBPATTERN_PRUNING) == 0;
        opt.engine = engine_options(g, flags);
        for (size_t l = 0; l < g->level_opt.size(); ++l) {
            if (!g->level_opt[l].first) continue;
            if (opt.level_engine.size() <= l) opt.level_engine.resize(l + 1);
            tfsm::EngineOptions e = opt.engine;
            apply_knobs(g->level_opt[l].second, e);
            opt.level_engine[l] = {true, e};
        }
        std::vector<tfsm::MinedPattern> pats;
        tfsm::MineStats st;
        g->eng->reset_times();
        tfsm::mine(*g->eng, g->lg, opt, pats, st);
        if (results_path && !tfsm::write_results(results_path, pats))
            return fail(TFSM_ERR_IO, std::string("cannot write ") + results_path);
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            const tfsm::KernelTimes &kt = g->eng->times();
            stats->load_ms = g->load_ms;
            stats->mine_ms = st.mine_ms;
            stats->extend_ms = st.extend_ms;
            stats->init_ms = kt.init_ms;
            stats->refine_ms = kt.refine_ms;
            stats->search_ms = kt.search_ms;
            stats->init_launches = kt.init_launches;
            stats->refine_launches = kt.refine_launches;
            stats->search_launches = kt.search_launches;
            stats->init_words = kt.init_words;
            stats->refine_words = kt.refine_words;
            stats->search_bytes = kt.search_bytes;
            stats->h2d_bytes = kt.h2d_bytes;
            stats->d2h_bytes = kt.d2h_bytes;
            stats->evaluations = st.evaluations;
            stats->frequent = st.frequent;
            stats->searches = st.searches;
            stats->steps = st.steps;
            stats->by_filter = st.by_filter;
            stats->engine_calls = st.engine_calls;
            stats->levels = st.levels;
            stats->complete = st.complete ? 1 : 0;
            for (size_t l = 0; l < st.level_ms.size() && l < TFSM_MAX_LEVELS; ++l) stats->level_ms[l] = st.level_ms[l];
            stats->pruned = st.pruned;
            stats->split_searches = kt.split_groups;
            stats->split_tasks = kt.split_tasks;
            stats->intersections = kt.isects;
        }
        return TFSM_OK;
    });
}

int tfsm_get_options(const tfsm_graph *g, tfsm_options *o) {
    return guarded([&]() -> int {
        if (!g || !o) return fail(TFSM_ERR_ARG, "null argument");
        const uint32_t size = o->struct_size;
        if (size < TFSM_OPTIONS_MIN_SIZE || size > sizeof(tfsm_options)) return fail(TFSM_ERR_ARG, kSizeRule);
        const tfsm_options cur = knobs_of(g->opt);
        std::memcpy(o, &cur, size);
        o->struct_size = size;
        return TFSM_OK;
    });
}

int tfsm_set_options(tfsm_graph *g, const tfsm_options *o) {
    return guarded([&]() -> int {
        if (!g || !o) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(g->mu);
        tfsm_options full;
        if (!read_options(o, g->opt, full)) return fail(TFSM_ERR_ARG, kSizeRule);
        if (!knobs_valid(full)) return fail(TFSM_ERR_ARG, kKnobRules);
        apply_knobs(full, g->opt);
        g->opt.time_limit_s = full.time_limit_s;
        return TFSM_OK;
    });
}

int tfsm_set_level_options(tfsm_graph *g, int32_t level, const tfsm_options *o) {
    return guarded([&]() -> int {
        if (!g) return fail(TFSM_ERR_ARG, "null argument");
        if (level < 0 || level >= TFSM_MAX_LEVELS) return fail(TFSM_ERR_ARG, "level must be in 0..TFSM_MAX_LEVELS-1");
        std::lock_guard<std::mutex> lk(g->mu);
        tfsm_options full;
        if (o && !read_options(o, g->opt, full)) return fail(TFSM_ERR_ARG, kSizeRule);
        if (o && !knobs_valid(full)) return fail(TFSM_ERR_ARG, kKnobRules);
        if (level == 0) {
            g->level_opt.clear();
            return TFSM_OK;
        }
        if (g->level_opt.size() <= (size_t)level) g->level_opt.resize((size_t)level + 1);
        g->level_opt[(size_t)level] = o ? std::make_pair(true, full) : std::make_pair(false, tfsm_options{});
        return TFSM_OK;
    });
}

int tfsm_evaluate_support_noalloc(tfsm_graph *g, const tfsm_pattern *pattern, int32_t tau, uint32_t flags,
                                  tfsm_result *out) {
    return guarded([&]() -> int {
        if (!g || !pattern || !out) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(g->mu);
        const char *msg = "";
        const int rc = tfsm::noalloc_evaluate(*g->eng, pattern, (uint32_t)std::max(tau, 0),
                                              (flags & TFSM_FLAG_EXACT) != 0, out, msg);
        if (rc != TFSM_OK) {
            out->status = rc;
            return fail(rc, msg);
        }
        return TFSM_OK;
    });
}

const char *tfsm_last_error(void) { return g_err.c_str(); }

}  // extern "C"

// ---- learned matching-order cost model ----

int tfsm_cost_model_create(uint64_t seed, tfsm_cost_model **out) {
    return guarded([&]() -> int {
        if (!out) return fail(TFSM_ERR_ARG, "null argument");
        *out = nullptr;
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(TFSM_ERR_NO_DEVICE, "no CUDA device");
        int device = 0;
        if (const char *env = std::getenv("TFSM_DEVICE")) device = std::atoi(env);
        if (device < 0 || device >= ndev) return fail(TFSM_ERR_NO_DEVICE, "TFSM_DEVICE names no CUDA device");
        std::unique_ptr<tfsm_cost_model> m(new tfsm_cost_model);
        m->m.reset(new tfsm::CostModel(seed, device));
        *out = m.release();
        return TFSM_OK;
    });
}

void tfsm_cost_model_free(tfsm_cost_model *m) { delete m; }

int tfsm_cost_model_get_params(const tfsm_cost_model *m, float *params) {
    return guarded([&]() -> int {
        if (!m || !params) return fail(TFSM_ERR_ARG, "null argument");
        const std::vector<float> p = m->m->params();
        std::memcpy(params, p.data(), p.size() * sizeof(float));
        return TFSM_OK;
    });
}

int tfsm_cost_model_set_params(tfsm_cost_model *m, const float *params) {
    return guarded([&]() -> int {
        if (!m || !params) return fail(TFSM_ERR_ARG, "null argument");
        m->m->set_params(params);
        return TFSM_OK;
    });
}

int tfsm_cost_model_predict(const tfsm_cost_model *m, const float *features, uint64_t n, float *costs) {
    return guarded([&]() -> int {
        if (!m || (n && (!features || !costs))) return fail(TFSM_ERR_ARG, "null argument");
        m->m->predict(features, (size_t)n, costs);
        return TFSM_OK;
    });
}

int tfsm_cost_model_gradients(const tfsm_cost_model *m, const float *features, const float *costs, uint64_t n,
                              float *grads) {
    return guarded([&]() -> int {
        if (!m || !features || !costs || !grads || n == 0) return fail(TFSM_ERR_ARG, "null argument or empty batch");
        m->m->gradients(features, costs, (size_t)n, grads);
        return TFSM_OK;
    });
}

int tfsm_cost_model_train(tfsm_cost_model *m, const float *features, const float *costs, uint64_t n, int32_t epochs,
                          int32_t batch, float lr, uint64_t seed, double *final_mse) {
    return guarded([&]() -> int {
        if (!m || !features || !costs || n == 0) return fail(TFSM_ERR_ARG, "null argument or no records");
        if (epochs < 0 || batch < 16 || !(lr > 0)) return fail(TFSM_ERR_ARG, "epochs >= 0, batch >= 16, lr > 0");
        const double mse = m->m->train(features, costs, (size_t)n, epochs, batch, lr, seed);
        if (final_mse) *final_mse = mse;
        return TFSM_OK;
    });
}

int tfsm_set_order_policy(tfsm_graph *g, uint32_t policy, uint64_t seed, const tfsm_cost_model *model) {
    return guarded([&]() -> int {
        if (!g) return fail(TFSM_ERR_ARG, "null argument");
        if (policy > 2) return fail(TFSM_ERR_ARG, "order policy must be 0 (GQL), 1 (random) or 2 (cost model)");
        if (policy == 2 && !model) return fail(TFSM_ERR_ARG, "order policy 2 needs a cost model");
        std::lock_guard<std::mutex> lk(g->mu);
        g->opt.order_policy = policy;
        g->opt.order_seed = seed;
        g->opt.cost_model = policy == 2 ? model->m.get() : nullptr;
        return TFSM_OK;
    });
}

int tfsm_record_orders(tfsm_graph *g, int32_t enable) {
    return guarded([&]() -> int {
        if (!g) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(g->mu);
        g->recording = enable != 0;
        return TFSM_OK;
    });
}

int tfsm_take_records(tfsm_graph *g, float *features, float *costs, uint64_t cap, uint64_t *n) {
    return guarded([&]() -> int {
        if (!g || !n) return fail(TFSM_ERR_ARG, "null argument");
        std::lock_guard<std::mutex> lk(g->mu);
        constexpr size_t W = TFSM_COST_FEATURES + 1;
        const uint64_t have = g->records.size() / W;
        if (!features) {
            *n = have;
            return TFSM_OK;
        }
        if (!costs) return fail(TFSM_ERR_ARG, "null argument");
        const uint64_t k = std::min(have, cap);
        for (uint64_t i = 0; i < k; ++i) {
            std::memcpy(features + i * TFSM_COST_FEATURES, &g->records[i * W], TFSM_COST_FEATURES * sizeof(float));
            costs[i] = g->records[i * W + TFSM_COST_FEATURES];
        }
        g->records.erase(g->records.begin(), g->records.begin() + (ptrdiff_t)(k * W));
        *n = k;
        return TFSM_OK;
    });
}
