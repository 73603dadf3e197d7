/*
 * tfsm.h — C ABI of the GB300 T-FSM engine (frequent subgraph mining with MNI support).
 *
 * Plain C, no exceptions across the boundary, caller-owned buffers, status-code returns.
 * Every entry point returns TFSM_OK (0) or a TFSM_ERR_* code; tfsm_last_error() then gives a
 * message for the calling thread.  A graph handle is immutable after loading and owns its device
 * copy on the GPU that was current when it was loaded; calls on one handle are serialised
 * internally, so a handle may be shared by host threads.
 *
 * The reference (lyuheng/T-FSM) has no plugin or FFI layer: its hot path is in-process C++.
 * Each entry point below names the reference interface it replaces.
 */
#ifndef TFSM_H
#define TFSM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TFSM_MAX_LEVELS 32 /* growth levels reported and tunable separately */

#define TFSM_OK 0
#define TFSM_ERR_ARG 1        /* invalid argument (null pointer, bad size, malformed pattern) */
#define TFSM_ERR_IO 2         /* graph file cannot be opened */
#define TFSM_ERR_FORMAT 3     /* malformed .lg input */
#define TFSM_ERR_PATTERN 4    /* pattern larger than TFSM_MAX_PATTERN_VERTICES */
#define TFSM_ERR_LIMIT 5      /* graph beyond the device layout's limits */
#define TFSM_ERR_NO_DEVICE 9  /* no CUDA device */
#define TFSM_ERR_CUDA 10      /* CUDA runtime error */
#define TFSM_ERR_INTERNAL 11

#define TFSM_MAX_PATTERN_VERTICES 32

/* flags */
#define TFSM_FLAG_EXACT 1u    /* exact MNI per vertex: no early exit at tau */
#define TFSM_FLAG_PLAIN 2u    /* tfsm_mine: one engine call per candidate pattern (unbatched) */
#define TFSM_FLAG_NO_SPLIT 4u /* disable splitting of long searches (hub tasks) */
#define TFSM_FLAG_NO_SUBPATTERN_PRUNING 8u /* tfsm_mine: search every candidate, even one with an
                                              infrequent one-edge-smaller sub-pattern */

typedef struct tfsm_graph tfsm_graph;

/* One DFS-code edge, as in the reference's dfs_code_t (parallel/graph.h:225-312). */
typedef struct {
    int32_t from, to, from_label, edge_label, to_label;
} tfsm_dfs_code;

/* A connected pattern given by its DFS code (forward edges introduce vertex `to`). */
typedef struct {
    int32_t n_codes;
    const tfsm_dfs_code *codes;
} tfsm_pattern;

typedef struct {
    int32_t status;        /* TFSM_OK or an error for this pattern */
    int32_t frequent;      /* 1 when MNI support >= tau */
    int32_t n_vertices;
    int32_t decided_by_filter; /* 1 when domain filtering alone decided the result */
    uint32_t support;      /* min over vertices of mni[] (exact with TFSM_FLAG_EXACT) */
    uint32_t mni[TFSM_MAX_PATTERN_VERTICES]; /* per-vertex MNI domain sizes found */
    uint64_t searches;     /* candidate checks (backtracking searches) started */
    uint64_t steps;        /* 32-candidate chunks evaluated by the searches */
} tfsm_result;

typedef struct {
    uint32_t n_vertices;   /* after label pruning */
    uint64_t n_edges;      /* undirected, after label pruning */
    uint32_t n_frequent_vertex_labels;
    uint32_t n_frequent_edge_labels;
    uint32_t n_frequent_edge_patterns; /* frequent 1-edge patterns */
    uint32_t max_degree;
    uint64_t device_bytes; /* device copy of the graph */
    double load_ms;        /* parse + prune + device upload */
    uint64_t load_h2d_bytes; /* host -> device bytes the load copied (file bytes or input arrays with
                                GPU ingestion, the built graph with the host loader) */
} tfsm_graph_info_t;

typedef struct {
    double load_ms, mine_ms, extend_ms;
    double init_ms, refine_ms, search_ms;   /* device time per kernel family (CUDA events) */
    uint64_t init_launches, refine_launches, search_launches; /* kernel launches per family */
    uint64_t init_words, refine_words;      /* bitmap words processed */
    uint64_t search_bytes;  /* algorithmic bytes read by the search kernels (logical loads) */
    uint64_t h2d_bytes, d2h_bytes;          /* host<->device copies made by the mining run */
    uint64_t evaluations;  /* candidate patterns evaluated (support evaluations) */
    uint64_t frequent;     /* frequent patterns, 1-edge patterns included */
    uint64_t searches, steps, by_filter, engine_calls;
    int32_t levels;
    int32_t complete;      /* 0 when the time limit stopped the run early */
    double level_ms[TFSM_MAX_LEVELS]; /* host wall time of the engine calls of each level (index =
                                         pattern edges; 0 unused) */
    uint64_t pruned;       /* candidates decided infrequent by an infrequent sub-pattern (counted in
                              evaluations and by_filter; no engine call) */
    uint64_t split_searches; /* searches split into tasks */
    uint64_t split_tasks;  /* split tasks written (all rounds) */
    uint64_t intersections; /* set intersections of the searches: one per chunk of up to 32 anchor
                               candidates and backward neighbour (the anchor's own range included) */
} tfsm_mine_stats;

/* Load a .lg graph and prune it for threshold `tau` (label frequency, edge-label frequency and
 * the frequent 1-edge pattern table) on CUDA device 0, or on the device whose index the
 * environment variable TFSM_DEVICE holds.  The file's bytes are copied to the device, which
 * parses them and builds the pruned, renumbered graph; TFSM_INGEST=host selects the host loader
 * instead (same graph, same errors).
 * Replaces Graph::load_graph (parallel/graph.h:557-570, serial/graph.h:485-494). */
int tfsm_graph_load(const char *path, int32_t tau, tfsm_graph **out);

/* Same from host arrays: vertex labels [n_vertices], and n_edges undirected edges
 * (src[i], dst[i], elabels[i]), as the `v` / `e` lines of a .lg file in that order. */
int tfsm_graph_from_edges(uint32_t n_vertices, const int32_t *vlabels, uint64_t n_edges, const uint32_t *src,
                          const uint32_t *dst, const int32_t *elabels, int32_t tau, tfsm_graph **out);

void tfsm_graph_free(tfsm_graph *g);

int tfsm_graph_info(const tfsm_graph *g, tfsm_graph_info_t *info);

/* A frequent 1-edge pattern (min label, edge label, max label) with its two endpoint-set sizes:
 * one entry of the reference's 1-edge table (parallel/graph.h:685-803, `hashedEdges`). */
typedef struct {
    int32_t la, el, lb;
    uint32_t cand_a, cand_b;
} tfsm_edge_pattern;

/* Destinations of tfsm_graph_export; a NULL member is not copied.  n, m, L, E and P are
 * tfsm_graph_info's n_vertices, n_edges, n_frequent_vertex_labels, n_frequent_edge_labels and
 * n_frequent_edge_patterns.  Vertex ids are the engine's: each frequent label L owns the ids
 * [label_start[L], label_start[L+1]); inside it vertices are ranked by descending degree. */
typedef struct {
    uint32_t *row_off;            /* [n + 1] adjacency offsets */
    uint32_t *col;                /* [2m] neighbour ids, ascending per vertex (ties: edge label) */
    uint8_t *elab;                /* [2m] edge labels as indices into elabels */
    uint32_t *label_start;        /* [L + 1] */
    uint32_t *lab_off;            /* [(L + 1) * n], label-major: the first position of vertex x's
                                     neighbours with label >= l is at l * n + x */
    int32_t *vlabels;             /* [L] frequent vertex labels, ascending */
    int32_t *elabels;             /* [E] frequent edge labels, ascending */
    tfsm_edge_pattern *edge_patterns; /* [P] ascending (la, el, lb) */
    float *label_mean_degree;     /* [L] mean degree of each frequent label's vertices */
} tfsm_graph_arrays;

/* Copies the graph as the device holds it (for checks and external tools). */
int tfsm_graph_export(const tfsm_graph *g, const tfsm_graph_arrays *arrays);

/* MNI support evaluation of one pattern: is MNI(P) >= tau?  With TFSM_FLAG_EXACT, mni[] holds
 * the exact per-vertex MNI domain sizes.  Replaces GraMi::frequency (serial/grami.h:261-328) and
 * the task_container life cycle of the parallel miner (parallel/comper.h:1552-1700, 1069-1152).
 * `tau` should equal the graph's load threshold (the pruned graph depends on it). */
int tfsm_evaluate_support(tfsm_graph *g, const tfsm_pattern *pattern, int32_t tau, uint32_t flags,
                          tfsm_result *out);

/* Batched form: all `n` patterns are evaluated by one launch sequence.  Returns TFSM_OK when the
 * batch was processed; a pattern that fails validation gets its error in results[i].status
 * (TFSM_ERR_ARG or TFSM_ERR_PATTERN) and the others are still evaluated.  tfsm_evaluate_support
 * returns its single pattern's status. */
int tfsm_evaluate_batch(tfsm_graph *g, const tfsm_pattern *patterns, int32_t n, int32_t tau, uint32_t flags,
                        tfsm_result *results);

/* Final domains of the patterns of one tfsm_evaluate_level call, kept on the device so that the
 * next growth level starts from them.  Replaces the reference's parent PatternProgress and its
 * cache of non-candidates handed to children (parallel/graph.h:402-414,
 * parallel/comper.h:1582-1612). */
typedef struct tfsm_domains tfsm_domains;

/* A pattern's parent: pattern `index` (the position in its call's `patterns`) of an earlier
 * tfsm_evaluate_level call on the same graph, whose domains `domains` holds.  The parent must be a
 * sub-pattern of the child under the same vertex numbering: every parent vertex keeps its id and
 * label, and every parent edge is a child edge, as when the child's DFS code extends the parent's. */
typedef struct {
    const tfsm_domains *domains; /* NULL: no parent */
    int32_t index;
} tfsm_parent;

/* tfsm_evaluate_batch with parents (`parents` may be NULL).  A pattern starts from its parent's
 * final domains (candidates minus proven non-candidates), which only removes vertices that cannot
 * be in its MNI domains: `frequent` equals the result without a parent, and so do `mni` and
 * `support` with TFSM_FLAG_EXACT.  A parent that is not a sub-pattern as above, that belongs to
 * another graph or whose own evaluation failed makes that pattern's status TFSM_ERR_ARG.  With
 * out != NULL the call's final domains stay on the device and *out receives them (NULL when no
 * pattern was evaluated); release them with tfsm_domains_free, which may come before or after
 * tfsm_graph_free but not during a call that reads them. */
int tfsm_evaluate_level(tfsm_graph *g, const tfsm_pattern *patterns, int32_t n, int32_t tau, uint32_t flags,
                        const tfsm_parent *parents, tfsm_result *results, tfsm_domains **out);

void tfsm_domains_free(tfsm_domains *d);

/* Whole mining run: frequent patterns with at most max_nodes vertices (-1: unbounded), written
 * to `results_path` (may be NULL) in the serial reference's grami_results.txt format.
 * Replaces GraMi::project (serial/grami.h:224-234) and Worker::run (parallel/worker.h:226-284). */
int tfsm_mine(tfsm_graph *g, int32_t tau, int32_t max_nodes, uint32_t flags, const char *results_path,
              tfsm_mine_stats *stats);

/* Tuning knobs of the GPU search (no counterpart in the reference, whose only knobs are the
 * compile-time TIMEOUT_THRESHOLD / DECOMPOSE_TIME_THRESHOLD of parallel/global.h:30-33).
 * They change speed only, never results.
 *
 * Versioned by size: set struct_size = sizeof(tfsm_options) before calling tfsm_get_options or
 * tfsm_set_options.  The library reads and writes only the first struct_size bytes, so a caller
 * built against an older header (a shorter struct, fields only ever added at the end) keeps
 * working; a struct_size below TFSM_OPTIONS_MIN_SIZE or above the library's own size is rejected
 * with TFSM_ERR_ARG. */
typedef struct {
    uint32_t struct_size;   /* sizeof(tfsm_options) as the caller compiled it */
    uint32_t step_budget;   /* 32-candidate chunks a search may evaluate before its unexplored
                               branches (at every depth) become split tasks; split tasks get twice
                               that, doubling per round up to 8x; a search whose tasks find no room
                               is retried by a later pass with 8x the budgets (0: never split;
                               default 16, or 64 for a graph with a vertex of more than 4 * hub_span
                               neighbours) */
    uint32_t split_slice;   /* adjacency positions per split task (>= 1) */
    uint32_t chunk_words;   /* 32-bit domain-bitmap words per search work item (>= 1) */
    uint32_t refine_rounds; /* arc-consistency passes for patterns that need a search (0..32; 0: none,
                               distinct-label trees still run to their fixpoint) */
    uint32_t max_batch;     /* tfsm_mine: most patterns per engine call (>= 1) */
    uint32_t hub_span;      /* a search whose first depth has more adjacency positions than this
                               (a hub vertex's label range) is split at once ... */
    uint32_t hub_parts;     /* ... into this many tasks, as many teams (1..32; 1: off) */
    double time_limit_s;    /* tfsm_mine: stop between engine calls after this many seconds (0: none);
                               the run is then reported incomplete */
    uint32_t search_lanes;  /* lanes per search: 8 (default: four searches per warp, for calls with
                               several patterns of at most 8 vertices) or 32; 0 means 32 */
    uint32_t rank_window;   /* patterns per window of the search order: within a window every
                               pattern's vertex with the smallest domain is searched first, then
                               the next one; windows follow one another (0: one window per call) */
    double call_ms;         /* tfsm_mine: an engine call that takes longer than this many milliseconds
                               makes the following calls take proportionally fewer patterns (at
                               least 4); full calls that finish sooner double it again, up to
                               max_batch (default 2; 0: always max_batch) */
    uint32_t isect_ratio;   /* intersection form of a search step against a further backward
                               neighbour: its candidate range is merged (streamed once with 128-bit
                               loads) when it is at most isect_ratio times the anchor's range, and
                               probed by binary search otherwise (>= 1; the reference switches at
                               50; the autotuner tries 4, 16, 64) */
    uint32_t reserved;      /* 0 */
    /* fields added after the first versioned layout */
    uint32_t refine_scope;  /* vertices of the first refinement rounds: 1 (default) for a pattern that
                               starts from its parent's domains only the two vertices of its newest
                               edge (the others were refined against the same edges in the parent's
                               call), 0 every vertex; distinct-label trees always refine every vertex */
    uint32_t reserved2;     /* 0 */
} tfsm_options;

#define TFSM_OPTIONS_MIN_SIZE 64u /* the first versioned layout: struct_size .. reserved */

int tfsm_get_options(const tfsm_graph *g, tfsm_options *opt);
int tfsm_set_options(tfsm_graph *g, const tfsm_options *opt);

/* Options for the engine calls of one growth level only (patterns with `level` edges,
 * 1 <= level < TFSM_MAX_LEVELS), e.g. from the autotuner; opt == NULL clears that level, level 0
 * clears every level.  Levels without their own options use tfsm_set_options'. */
int tfsm_set_level_options(tfsm_graph *g, int32_t level, const tfsm_options *opt);

/* Allocation-free variant of tfsm_evaluate_support (no counterpart in the reference).
 * For callers that must not allocate device memory during the call — for example code under a
 * framework whose own caching allocator owns the device, or latency-critical code that cannot
 * afford the device-wide synchronisation of cudaMalloc / cudaFree.  The call makes no device
 * allocation and calls no allocating library routine: every per-call buffer lives in one fixed
 * 16 MiB device array that the library holds on each GPU it is used on, until the process exits.
 * A pattern whose domain bitmaps do not fit is rejected with TFSM_ERR_LIMIT.  Calls share that array
 * and leave its contents behind (each call clears what must start at zero); calls whose GPU work
 * overlaps would race on it — calls on one graph handle are serialised by the handle.  The first call
 * on a device looks up the array's device address, so make it before any stream capture.  Results
 * equal tfsm_evaluate_support's (mni[] exactly with TFSM_FLAG_EXACT). */
int tfsm_evaluate_support_noalloc(tfsm_graph *g, const tfsm_pattern *pattern, int32_t tau, uint32_t flags,
                                  tfsm_result *out);

/* Message of the last failing call on this thread ("" when none). */
const char *tfsm_last_error(void);

/* ---- Learned matching-order cost model (no counterpart in the reference) ----------------------
 * A 32-64-64-1 MLP (BF16 weights, FP32 accumulation) trained and evaluated on the GPU.  It predicts
 * log2(1 + chunk evaluations per search) of searching a pattern vertex's candidates with a given
 * matching order; with order policy 2 the engine takes the order with the lowest prediction.
 * A matching order never changes a result, only the work. */
#define TFSM_COST_FEATURES 32
#define TFSM_COST_PARAMS 6337 /* W1[32][64], b1[64], W2[64][64], b2[64], W3[64], b3 (FP32 master copy) */

typedef struct tfsm_cost_model tfsm_cost_model;

int tfsm_cost_model_create(uint64_t seed, tfsm_cost_model **out); /* random initial weights */
void tfsm_cost_model_free(tfsm_cost_model *m);
int tfsm_cost_model_get_params(const tfsm_cost_model *m, float *params);
int tfsm_cost_model_set_params(tfsm_cost_model *m, const float *params); /* resets the optimiser */
int tfsm_cost_model_predict(const tfsm_cost_model *m, const float *features, uint64_t n, float *costs);
/* Gradient of the mean squared error of one batch at the current weights (parameter layout). */
int tfsm_cost_model_gradients(const tfsm_cost_model *m, const float *features, const float *costs, uint64_t n,
                              float *grads);
/* Adam over `epochs` shuffled passes in minibatches of `batch` (>= 16) records. */
int tfsm_cost_model_train(tfsm_cost_model *m, const float *features, const float *costs, uint64_t n, int32_t epochs,
                          int32_t batch, float lr, uint64_t seed, double *final_mse);

/* Matching order of every searched pattern vertex on this handle: 0 the GQL order (default;
 * the fixed-order path), 1 a random connected order drawn with `seed` (for logging training
 * records), 2 the order the cost model predicts cheapest (GQL on ties).  The model must outlive its
 * use by the handle. */
int tfsm_set_order_policy(tfsm_graph *g, uint32_t policy, uint64_t seed, const tfsm_cost_model *model);
/* While enabled, every engine call appends one training record per searched pattern vertex:
 * TFSM_COST_FEATURES features of the order used and the measured cost. */
int tfsm_record_orders(tfsm_graph *g, int32_t enable);
/* Moves up to `cap` records out (features: cap x TFSM_COST_FEATURES); features == NULL only
 * counts them into *n. */
int tfsm_take_records(tfsm_graph *g, float *features, float *costs, uint64_t cap, uint64_t *n);

#ifdef __cplusplus
}
#endif

#endif /* TFSM_H */
