// `run`: command-line drop-in for the reference miners (parallel/run.cpp:11-82, serial/run.cpp).
//
//   run -file G.lg -freq TAU [-thread T] [-maxNodes N] [-plain] [-exact] [-out PATH]
//       [-step-budget B] [-split-slice S] [-chunk-words W] [-refine-rounds R] [-refine-scope 0|1] [-max-batch M]
//       [-hub-span S] [-hub-parts K] [-isect-ratio R] [-search-lanes L] [-rank-window W] [-call-ms MS]
//       [-no-split] [-time-limit SECONDS] [-random-orders SEED] [-no-prune]
//
// Frequent patterns go to ./grami_results.txt (or -out PATH) in the serial build's format
// (serial/grami.h:622-635); timing and counts are printed as the parallel build prints them.
// `-thread` is accepted for compatibility; host work uses all cores and mining runs on the GPU.
// Unlike the reference, `-file` may appear anywhere on the command line.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/tfsm.h"

static const char *opt(int argc, char **argv, const char *name) {
    for (int i = 1; i + 1 < argc; ++i)
        if (!std::strcmp(argv[i], name)) return argv[i + 1];
    return nullptr;
}

static bool flag(int argc, char **argv, const char *name) {
    for (int i = 1; i < argc; ++i)
        if (!std::strcmp(argv[i], name)) return true;
    return false;
}

int main(int argc, char **argv) {
    const char *file = opt(argc, argv, "-file");
    const char *freq = opt(argc, argv, "-freq");
    if (!file || !freq) {
        std::fprintf(stderr, "usage: run -file G.lg -freq TAU [-thread T] [-maxNodes N] [-plain] [-exact] [-out PATH]\n");
        return 2;
    }
    const int tau = std::atoi(freq);
    const int max_nodes = opt(argc, argv, "-maxNodes") ? std::atoi(opt(argc, argv, "-maxNodes")) : -1;
    const char *out = opt(argc, argv, "-out") ? opt(argc, argv, "-out") : "./grami_results.txt";
    uint32_t flags = 0;
    if (flag(argc, argv, "-plain")) flags |= TFSM_FLAG_PLAIN;
    if (flag(argc, argv, "-exact")) flags |= TFSM_FLAG_EXACT;
    if (flag(argc, argv, "-no-prune")) flags |= TFSM_FLAG_NO_SUBPATTERN_PRUNING;
    if (flag(argc, argv, "-no-split")) flags |= TFSM_FLAG_NO_SPLIT;

    tfsm_graph *g = nullptr;
    int rc = tfsm_graph_load(file, tau, &g);
    if (rc != TFSM_OK) {
        std::fprintf(stderr, "error %d: %s\n", rc, tfsm_last_error());
        return 1;
    }
    tfsm_options o;
    o.struct_size = sizeof(o);
    tfsm_get_options(g, &o);
    if (opt(argc, argv, "-step-budget")) o.step_budget = (uint32_t)std::atoi(opt(argc, argv, "-step-budget"));
    if (opt(argc, argv, "-split-slice")) o.split_slice = (uint32_t)std::atoi(opt(argc, argv, "-split-slice"));
    if (opt(argc, argv, "-chunk-words")) o.chunk_words = (uint32_t)std::atoi(opt(argc, argv, "-chunk-words"));
    if (opt(argc, argv, "-refine-rounds")) o.refine_rounds = (uint32_t)std::atoi(opt(argc, argv, "-refine-rounds"));
    if (opt(argc, argv, "-refine-scope")) o.refine_scope = (uint32_t)std::atoi(opt(argc, argv, "-refine-scope"));
    if (opt(argc, argv, "-max-batch")) o.max_batch = (uint32_t)std::atoi(opt(argc, argv, "-max-batch"));
    if (opt(argc, argv, "-hub-span")) o.hub_span = (uint32_t)std::atoi(opt(argc, argv, "-hub-span"));
    if (opt(argc, argv, "-hub-parts")) o.hub_parts = (uint32_t)std::atoi(opt(argc, argv, "-hub-parts"));
    if (opt(argc, argv, "-isect-ratio")) o.isect_ratio = (uint32_t)std::atoi(opt(argc, argv, "-isect-ratio"));
    if (opt(argc, argv, "-search-lanes")) o.search_lanes = (uint32_t)std::atoi(opt(argc, argv, "-search-lanes"));
    if (opt(argc, argv, "-rank-window")) o.rank_window = (uint32_t)std::atoi(opt(argc, argv, "-rank-window"));
    if (opt(argc, argv, "-call-ms")) o.call_ms = std::atof(opt(argc, argv, "-call-ms"));
    if (opt(argc, argv, "-time-limit")) o.time_limit_s = std::atof(opt(argc, argv, "-time-limit"));
    rc = tfsm_set_options(g, &o);
    if (rc == TFSM_OK && opt(argc, argv, "-random-orders"))  // random matching orders: same results
        rc = tfsm_set_order_policy(g, 1, (uint64_t)std::atoll(opt(argc, argv, "-random-orders")), nullptr);
    if (rc != TFSM_OK) {
        std::fprintf(stderr, "error %d: %s\n", rc, tfsm_last_error());
        tfsm_graph_free(g);
        return 1;
    }
    tfsm_mine_stats st;
    rc = tfsm_mine(g, tau, max_nodes, flags, out, &st);
    if (rc != TFSM_OK) {
        std::fprintf(stderr, "error %d: %s\n", rc, tfsm_last_error());
        tfsm_graph_free(g);
        return 1;
    }
    std::printf("[TIME] Loading Graph Time: %.3f s\n", st.load_ms / 1e3);
    std::printf("[TIME] Mining Time: %.3f s\n", st.mine_ms / 1e3);
    std::printf("[TIME] Total Elapsed Time: %.3f s\n", (st.load_ms + st.mine_ms) / 1e3);
    std::printf("[INFO] # Frequent Patterns: %llu\n", (unsigned long long)st.frequent);
    std::printf("[INFO] # Support Evaluations: %llu (%.0f /s)\n", (unsigned long long)st.evaluations,
                st.mine_ms > 0 ? st.evaluations / (st.mine_ms / 1e3) : 0.0);
    std::printf("[INFO] # Searches: %llu, # Chunk steps: %llu, decided by filters: %llu (by sub-patterns: %llu), "
                "engine calls: %llu\n",
                (unsigned long long)st.searches, (unsigned long long)st.steps, (unsigned long long)st.by_filter,
                (unsigned long long)st.pruned, (unsigned long long)st.engine_calls);
    if (!st.complete) std::printf("[INFO] TIME LIMIT REACHED: the run is incomplete\n");
    std::printf("[TIME] Device: init %.3f ms (%llu), refine %.3f ms (%llu), search %.3f ms (%llu), host extend %.3f ms\n",
                st.init_ms, (unsigned long long)st.init_launches, st.refine_ms, (unsigned long long)st.refine_launches,
                st.search_ms, (unsigned long long)st.search_launches, st.extend_ms);
    tfsm_graph_free(g);
    return 0;
}
