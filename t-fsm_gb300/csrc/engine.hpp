// GPU support-evaluation engine: device graph, batch evaluation of patterns, level memory.
#pragma once

#include <chrono>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "costmodel/mlp.hpp"
#include "host/lg_graph.hpp"
#include "host/pattern.hpp"

struct CUstream_st;  // cudaStream_t without the CUDA runtime header

namespace tfsm {

namespace dev {
struct Graph;
}
struct DeviceGraphBuild;  // cuda/ingest.hpp

struct EngineError : std::runtime_error {
    int code;
    EngineError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

struct EvalResult {
    bool frequent = false;
    bool by_filter = false;            // decided without search (domain sizes / arc consistency)
    std::vector<uint32_t> mni;         // per pattern vertex; exact in exact mode
    uint32_t support = 0;              // min over vertices of mni
    uint64_t searches = 0;             // candidate checks
    uint64_t steps = 0;                // 32-candidate chunks evaluated by the search
    uint64_t max_steps = 0;            // longest single search of the pattern (chunk evaluations)
};

struct EngineOptions {
    bool exact = false;                // evaluate every candidate (exact MNI), no early exit
    bool split = true;                 // long searches are split into tasks for the split rounds
    uint32_t step_budget = 16;         // chunk evaluations before a search is split (0: never); split
                                       //   tasks get twice that, doubling per later round up to 8x;
                                       //   later passes (for what found no room) multiply it by 8
    uint32_t split_slice = 64;         // anchor positions per split task
    uint32_t hub_span = 4096;          // a search whose first depth has more anchor positions ...
    uint32_t hub_parts = 4;            //   ... is split at once into this many tasks (1: off)
    uint32_t isect_ratio = 16;         // merge a further backward neighbour's candidate run when it
                                       //   is at most this many times the step's survivors, else
                                       //   galloping search
    uint32_t chunk_words = 1;          // bitmap words per search work item (x32 candidates)
    uint32_t search_lanes = 8;         // lanes per search: 32, 8 (four searches per warp, used for calls
                                       //   with several patterns of at most 8 vertices) or 4 (eight per
                                       //   warp, patterns of at most 5 vertices; larger ones fall back)
    uint32_t refine_rounds = 1;        // arc-consistency passes for patterns that need search (0: none)
    uint32_t refine_scope = 1;         // 1: a child's first refinement rounds cover its newest edge's two
                                       //   vertices only (the rest were refined in its parent's call); 0: all
    uint32_t rank_window = 0;          // patterns per window of the vertex-major item order (0: all)
    uint32_t max_batch = 4096;         // miner: patterns per engine call
    double call_ms = 2;                // miner: engine-call time (ms) above which later calls take
                                       //   fewer patterns (0: always max_batch)
    double time_limit_s = 0;           // miner: stop between engine calls after this long (0: none)
    // Matching order of each searched pattern vertex (never changes a result):
    //   0: GQL order (fewest candidates next), 1: a random connected order (seeded; used to log
    //   training records), 2: the order with the lowest cost predicted by `cost_model`
    uint32_t order_policy = 0;
    uint64_t order_seed = 0;
    const CostModel *cost_model = nullptr;
    // when set, one record per searched pattern vertex is appended: 32 features of the order used
    // (costmodel/features.hpp) and log2(1 + chunk evaluations per search) measured for it
    std::vector<float> *records = nullptr;
};

struct KernelTimes {                   // accumulated device time (CUDA events), milliseconds
    double init_ms = 0, refine_ms = 0, search_ms = 0;
    double engine_ms = 0;              // host wall time inside evaluate() (device phases included)
    double phase_ms[7] = {};           // of which: descriptors, pools+upload, init+refine, plans, items,
                                       //   search, results
    uint64_t init_launches = 0, refine_launches = 0, search_launches = 0;  // kernel launches
    uint64_t search_calls = 0;         // search phases (k_search, plus k_split when splitting)
    uint64_t init_words = 0, refine_words = 0;  // bitmap words processed
    uint64_t search_bytes = 0;         // algorithmic bytes read by the search kernels
    uint64_t isects = 0;               // set intersections (chunk x backward neighbour) of the searches
    uint64_t h2d_bytes = 0, d2h_bytes = 0;      // host<->device copies of the evaluations
    uint64_t split_groups = 0;                  // searches split into tasks
    uint64_t split_tasks = 0;                   // split tasks written (all rounds)
    uint64_t abandoned = 0;                     // searches / tasks set aside for a later pass (no room)
    uint64_t search_passes = 0;                 // search passes that ran
    double order_ms = 0;                        // host + cost-model time spent choosing orders
};

// Device memory of one evaluated batch; kept while the batch's patterns are parents.
struct Level {
    struct Impl;
    std::unique_ptr<Impl> impl;
    Level();
    ~Level();
    Level(Level &&) noexcept;
    Level &operator=(Level &&) noexcept;
    size_t size() const;  // patterns in the batch
};

// A pattern evaluated by an earlier engine call: `idx` in the batch that call wrote to `lvl`.
struct LevelRef {
    const Level *lvl = nullptr;
    int idx = -1;
};

// A sub-pattern of a candidate with one edge less, evaluated in the previous growth level
// (push-down pruning: its final domains bound the candidate's).  At most kMaxPushSources per
// candidate.
constexpr int kMaxPushSources = 4;
struct PushSource {
    LevelRef at;        // where its bitmaps are
    int8_t vertex[32];  // per candidate vertex: the sub-pattern vertex it maps to, or -1
};

class GpuEngine {
public:
    // The device graph of a host-built graph (renumbered and uploaded here).
    GpuEngine(const LgGraph &g, int device = 0);
    // The device graph built on the GPU (cuda/ingest.hpp): `build` runs on the engine's stream;
    // the graph's host-side facts (labels, 1-edge patterns, statistics) are moved into `summary`.
    GpuEngine(const std::function<void(CUstream_st *, DeviceGraphBuild &)> &build, LgGraph &summary, int device = 0);
    ~GpuEngine();
    GpuEngine(const GpuEngine &) = delete;
    GpuEngine &operator=(const GpuEngine &) = delete;

    // Evaluate `pats` against the graph.  parent[i] is the pattern's parent (lvl == nullptr:
    // none); parents and push-down sources may come from any number of earlier calls, whose
    // Levels must stay alive during the call.  `out` receives this batch's device memory for the
    // next level.
    void evaluate(const std::vector<const Pattern *> &pats, const std::vector<LevelRef> &parent, uint32_t tau,
                  const EngineOptions &opt, Level &out, std::vector<EvalResult> &res,
                  const std::vector<std::vector<PushSource>> *push = nullptr);

    const KernelTimes &times() const { return times_; }
    void reset_times() { times_ = KernelTimes(); }
    uint64_t graph_bytes() const;
    double upload_ms() const { return upload_ms_; }
    uint64_t load_h2d_bytes() const { return load_h2d_bytes_; }  // host -> device bytes of the graph's construction
    const std::string &load_breakdown() const { return load_breakdown_; }  // engine construction phases
    int dense_label(int label) const;  // -1 when the label is not frequent
    uint32_t n_vertices() const;
    void device_memory(size_t &free_bytes, size_t &total_bytes) const;  // of the engine's device
    // Read-only views used by the allocation-free entry point (noalloc.cu).
    int device() const;
    CUstream_st *stream() const;                     // the engine's own (non-blocking) stream
    const dev::Graph &device_graph() const;
    int dense_edge_label(int label) const;           // -1 when the edge label is not frequent
    uint32_t label_first(int dense) const;           // first vertex id of a dense label
    uint32_t label_size(int dense) const;            // vertices of a dense label
    // Copies of the device graph (any pointer may be null): row_off [n+1], col / elab [m2],
    // label_start [NL+1], lab_off [n*(NL+1)]; and the per-label mean degree [NL].
    void export_graph(uint32_t *row_off, uint32_t *col, uint8_t *elab, uint32_t *label_start, uint32_t *lab_off,
                      float *label_mean_degree) const;

private:
    void open(int device);
    void finish(std::chrono::steady_clock::time_point t0);
    struct Impl;
    std::unique_ptr<Impl> impl_;
    KernelTimes times_;
    double upload_ms_ = 0;
    uint64_t load_h2d_bytes_ = 0;
    std::string load_breakdown_;
};

}  // namespace tfsm
