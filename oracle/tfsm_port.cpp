// ORACLE — test infrastructure only.  A complete CPU frequent-subgraph miner built from the
// restated support evaluation in port_mni.hpp and the shared host pattern growth.  It is the
// checker for the CUDA miner (pattern sets and supports) and the CPU baseline timed by bench.py.
//
// Command line as the reference (parallel/run.cpp:11-82, `-file` first):
//   tfsm_port -file G.lg -freq TAU [-thread T] [-maxNodes N] [-exact 1] [-out results.txt]
//             [-supports supports.txt] [-time-limit SECONDS] [-repeat R]
// -time-limit stops a run between candidates after that many seconds of mining; -repeat mines R
// times after one load and prints one [SAMPLE] line per run (the reported totals are the last
// run's).
// Mining is level by level: every frequent pattern of one size is extended (rightmost extension
// + canonical check), and the children are evaluated by T threads, each evaluating whole
// patterns.  Children inherit their parent's final domains (parallel/gmatch.h:334-359).
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <mutex>
#include <string>
#include <thread>

#include "port_mni.hpp"

using namespace tfsm;

namespace {

const char *opt(int argc, char **argv, const char *name) {
    for (int i = 1; i + 1 < argc; ++i)
        if (!std::strcmp(argv[i], name)) return argv[i + 1];
    return nullptr;
}

struct Node {
    Pattern pat;
    int parent = -1;  // index in the previous level
    oracle::Eval ev;
};

}  // namespace

int main(int argc, char **argv) {
    const char *file = opt(argc, argv, "-file");
    const char *freq = opt(argc, argv, "-freq");
    if (!file || !freq) {
        std::fprintf(stderr, "usage: tfsm_port -file G.lg -freq TAU [-thread T] [-maxNodes N] [-exact 1]\n");
        return 2;
    }
    const int tau = std::atoi(freq);
    const int threads = opt(argc, argv, "-thread") ? std::max(1, std::atoi(opt(argc, argv, "-thread"))) : 1;
    const int max_nodes = opt(argc, argv, "-maxNodes") ? std::atoi(opt(argc, argv, "-maxNodes")) : -1;
    const bool exact = opt(argc, argv, "-exact") && std::atoi(opt(argc, argv, "-exact")) != 0;
    const char *out_path = opt(argc, argv, "-out");
    const char *sup_path = opt(argc, argv, "-supports");
    const double time_limit = opt(argc, argv, "-time-limit") ? std::atof(opt(argc, argv, "-time-limit")) : 0.0;

    auto t0 = std::chrono::steady_clock::now();
    LgGraph g;
    try {
        g = load_lg(file, tau);
    } catch (const LgError &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    oracle::PortGraph pg(g);
    auto t1 = std::chrono::steady_clock::now();

    ExtendContext ctx;
    ctx.freq_elabels = g.freq_elabels;
    ctx.max_nodes = max_nodes;
    for (auto &ep : g.edge_pairs) {
        ctx.neighbor_labels[ep.la].insert(ep.lb);
        ctx.neighbor_labels[ep.lb].insert(ep.la);
    }

    std::vector<oracle::Engine *> engines;
    for (int t = 0; t < threads; ++t) engines.push_back(new oracle::Engine(pg));

    // One complete mining run (stopped between candidates once `time_limit` seconds of mining have
    // passed, when set); counts only the candidates actually evaluated.
    struct Run {
        std::vector<std::vector<Node>> all_levels;
        uint64_t evaluations = 0, searches = 0;
        bool timed_out = false;
        double mine_s = 0;
    };
    auto mine_once = [&](Run &run) {
        const auto tm = std::chrono::steady_clock::now();
        std::atomic<uint64_t> evaluated(0);
        std::atomic<bool> timed_out(false);
        std::vector<Node> level;
        for (auto &ep : g.edge_pairs) {
            Node nd;
            nd.pat.push(DfsCode{0, 1, ep.la, ep.el, ep.lb});
            level.push_back(std::move(nd));
        }
        auto eval_level = [&](std::vector<Node> &lv, const std::vector<Node> *parents) {
            std::atomic<size_t> next(0);
            auto work = [&](int tid) {
                oracle::Engine &eng = *engines[(size_t)tid];
                for (;;) {
                    size_t i = next.fetch_add(1);
                    if (i >= lv.size()) break;
                    if (time_limit > 0 &&
                        std::chrono::duration<double>(std::chrono::steady_clock::now() - tm).count() > time_limit) {
                        timed_out = true;
                        continue;
                    }
                    Node &nd = lv[i];
                    const std::vector<std::vector<uint32_t>> *par =
                        (parents && nd.parent >= 0) ? &(*parents)[(size_t)nd.parent].ev.domains : nullptr;
                    nd.ev = oracle::evaluate(eng, nd.pat, par, (uint32_t)tau, exact);
                    evaluated++;
                }
            };
            std::vector<std::thread> th;
            for (int t = 0; t < threads; ++t) th.emplace_back(work, t);
            for (auto &x : th) x.join();
        };
        eval_level(level, nullptr);
        // 1-edge patterns are frequent by construction of the pair table; keep their domains
        for (auto &nd : level) nd.ev.frequent = true;
        while (!level.empty() && !timed_out) {
            run.all_levels.push_back(std::move(level));
            std::vector<Node> &cur = run.all_levels.back();
            std::vector<Node> next;
            for (size_t i = 0; i < cur.size(); ++i) {
                if (!cur[i].ev.frequent) continue;
                std::vector<Pattern> kids;
                extend_pattern(cur[i].pat, ctx, kids);
                for (auto &k : kids) {
                    Node nd;
                    nd.pat = std::move(k);
                    nd.parent = (int)i;
                    next.push_back(std::move(nd));
                }
            }
            if (next.empty()) break;
            eval_level(next, &cur);
            // parents' domains are no longer needed
            for (auto &nd : cur) nd.ev.domains.clear();
            level = std::move(next);
        }
        if (timed_out && !level.empty()) run.all_levels.push_back(std::move(level));
        for (auto &lv : run.all_levels)
            for (auto &nd : lv) run.searches += nd.ev.searches;
        run.evaluations = evaluated;
        run.timed_out = timed_out;
        run.mine_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - tm).count();
    };

    // -repeat R: R mining runs after one load (bounded samples for the CPU baseline); the outputs
    // and totals below are the last run's
    const int repeat = opt(argc, argv, "-repeat") ? std::max(1, std::atoi(opt(argc, argv, "-repeat"))) : 1;
    Run run;
    for (int k = 0; k < repeat; ++k) {
        run = Run();
        mine_once(run);
        if (repeat > 1)
            std::printf("[SAMPLE] %d mine_s %.6f evaluations %llu\n", k, run.mine_s,
                        (unsigned long long)run.evaluations);
    }
    const bool timed_out = run.timed_out;
    std::vector<std::vector<Node>> &all_levels = run.all_levels;
    std::vector<const Node *> reported;
    for (auto &lv : all_levels)
        for (auto &nd : lv)
            if (nd.ev.frequent) reported.push_back(&nd);
    uint64_t intersections = 0;
    for (auto *e : engines) {
        intersections += e->intersections;
        delete e;
    }
    const uint64_t evaluations = run.evaluations, searches = run.searches;
    auto t2 = std::chrono::steady_clock::now();

    if (out_path) {
        std::ofstream f(out_path);
        for (auto *nd : reported) f << nd->pat.to_results_block();
    }
    if (sup_path) {
        std::ofstream f(sup_path);
        for (auto &lv : all_levels)
            for (auto &nd : lv) {
                f << (nd.ev.frequent ? "F " : "I ") << nd.pat.key() << " |";
                for (auto c : nd.ev.mni) f << ' ' << c;
                f << '\n';
            }
    }
    const double load_s = std::chrono::duration<double>(t1 - t0).count();
    const double mine_s = repeat > 1 ? run.mine_s : std::chrono::duration<double>(t2 - t1).count();
    std::printf("[TIME] Loading Graph Time: %.3f s\n", load_s);
    std::printf("[TIME] Mining Time: %.3f s\n", mine_s);
    std::printf("[TIME] Total Elapsed Time: %.3f s\n", load_s + mine_s);
    std::printf("[INFO] # Frequent Patterns: %zu\n", reported.size());
    std::printf("[INFO] # Support Evaluations: %llu\n", (unsigned long long)evaluations);
    std::printf("[INFO] # Searches: %llu\n", (unsigned long long)searches);
    std::printf("[INFO] # Intersections: %llu\n", (unsigned long long)intersections);
    std::printf("[INFO] Threads: %d\n", threads);
    if (timed_out) std::printf("[INFO] TIME LIMIT REACHED\n");
    return timed_out ? 3 : 0;
}
