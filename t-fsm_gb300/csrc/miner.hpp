// Frequent-subgraph miner driving the GPU engine.
//
// Same search space and output as the reference miners: frequent 1-edge patterns from the label
// pair table, rightmost extension with the canonical check (host), MNI support evaluated on the
// GPU, children only of frequent canonical patterns, at most `max_nodes` pattern vertices.
//   batched: every candidate of one growth level is evaluated by one engine call
//   plain:   one engine call (one launch sequence) per candidate pattern
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "engine.hpp"
#include "host/lg_graph.hpp"
#include "host/pattern.hpp"

namespace tfsm {

struct MineOptions {
    int tau = 1;
    int max_nodes = -1;
    bool batched = true;
    int host_threads = 0;  // threads for extension + canonical checks (0: TFSM_HOST_THREADS or the cores)
    bool subpattern_pruning = true;  // Apriori: a child with an infrequent one-edge-smaller sub-pattern is infrequent
    EngineOptions engine;
    // per growth level (index = pattern edges): options for that level's engine calls, when set
    std::vector<std::pair<bool, EngineOptions>> level_engine;
    const EngineOptions &engine_for(int level) const {
        return level >= 0 && (size_t)level < level_engine.size() && level_engine[(size_t)level].first
                   ? level_engine[(size_t)level].second
                   : engine;
    }
};

struct MinedPattern {
    Pattern pat;
    EvalResult res;
};

struct MineStats {
    double mine_ms = 0;
    double extend_ms = 0;           // host pattern growth + canonical checks
    uint64_t evaluations = 0;       // candidate patterns whose support was evaluated
    uint64_t frequent = 0;
    uint64_t searches = 0;
    uint64_t steps = 0;
    uint64_t by_filter = 0;         // decided without search
    uint64_t pruned = 0;            // of these: by an infrequent sub-pattern (no engine call)
    uint64_t engine_calls = 0;
    int levels = 0;
    bool complete = true;           // false when the time limit stopped the run
    std::vector<double> level_ms;   // engine wall time per level (index = pattern edges)
};

// Mines all frequent patterns; `out` lists them level by level in generation order.
void mine(GpuEngine &eng, const LgGraph &g, const MineOptions &opt, std::vector<MinedPattern> &out, MineStats &st);

// Writes `pats` in the serial reference's grami_results.txt format.
bool write_results(const std::string &path, const std::vector<MinedPattern> &pats);

}  // namespace tfsm
