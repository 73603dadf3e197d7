// Device-side data layout shared by the host engine and the kernels.
//
// Data graph in HBM (built once per graph, read-only afterwards):
//   vertices are renumbered so that each frequent vertex label owns one contiguous id range
//   [label_start[L], label_start[L+1]) — ids keep the reference's pruned order inside a label.
//   row_off[n+1] (u32) / col[2m] (u32, ascending; followed by kColPad entries of 0xffffffff so
//   that 128-bit loads near the end stay inside the allocation) / elab[2m] (u8, dense edge label)
//   Ascending neighbour ids are therefore ordered by (neighbour label, id): the neighbours of v
//   that carry label L are one sub-range of v's list; a per-vertex table of label offsets gives its
//   bounds with two independent loads.
// Per pattern vertex u, a candidate domain D(u) is a bitmap over the id range of u's label; the
// same layout holds the "found" (MNI domain members proven by an embedding) and "failed"
// (proven non-members) bitmaps.  Offsets are in 32-bit words into three level-wide pools.
#pragma once

#include <cstdint>

namespace tfsm {
namespace dev {

constexpr int kMaxN = 32;          // pattern vertices supported by the device path (the reference's
                                   //   MAX_PATTERN_SIZE, parallel/global.h:36)
constexpr int kTaskMaxN = 16;      // largest pattern whose searches split into tasks (larger ones
                                   //   finish each search in place)
constexpr int kMaxNlf = 8;         // neighbour-label requirements kept per pattern vertex (any
                                   //   subset is a sound filter)
constexpr uint8_t kNoEdge = 0xff;  // edge-label matrix entry for "not adjacent"
constexpr uint32_t kColPad = 128;  // padding entries after col (at least 4 x the widest team)

struct Graph {
    uint32_t n = 0;
    uint64_t m2 = 0;                 // directed adjacency entries (2 * undirected edges)
    int n_labels = 0;
    const uint32_t *row_off = nullptr;   // [n+1]; the host rejects graphs with >= 2^32 adjacency entries
    const uint32_t *col = nullptr;
    const uint8_t *elab = nullptr;
    const uint32_t *label_start = nullptr;  // [n_labels + 1]
    // Label-major: lab_off[L * n + v] = position in col of v's first neighbour with label >= L, for
    // L = 0..n_labels; the neighbours of v with label L are [lab_off[L * n + v],
    // lab_off[(L + 1) * n + v]).  The candidates of one bitmap word are consecutive ids, so a
    // warp's lookups of one label coalesce, and the rows of the few labels a pattern uses stay in L2.
    const uint32_t *lab_off = nullptr;
};


// One pattern of a batch.  Plain old data, copied to the device once per batch.
constexpr int kMaxPush = 4;  // sub-patterns besides the parent whose domains bound a child's

// The bitmap pools of an earlier engine call whose final domains bound this call's initial ones
// (parents, push-down sources).  A source reference is (slot << kSrcShift) | word offset, slot
// indexing the call's table of SourceLevel.
struct SourceLevel {
    const uint32_t *dom;
    const uint32_t *failed;
    uint64_t words;
};
constexpr int kSrcShift = 40;
constexpr uint64_t kSrcMask = (1ull << kSrcShift) - 1;

struct PatDesc {
    int32_t n;
    int32_t n_reps;                     // orbit representatives that get search tasks
    int32_t express;                    // distinct labels + acyclic: decided by arc consistency
    int32_t lab[kMaxN];                 // dense label index
    int32_t deg[kMaxN];
    uint32_t adj[kMaxN];                // adjacency bitmask
    uint8_t el[kMaxN][kMaxN];           // dense edge label or kNoEdge
    uint32_t orbit_mask[kMaxN];         // vertices in the automorphism orbit of u (incl. u)
    int32_t rep[kMaxN];                 // representative of u's orbit
    uint32_t lstart[kMaxN];             // first id of u's label range
    uint32_t lsize[kMaxN];              // size of u's label range
    uint32_t words[kMaxN];              // bitmap words of u = ceil(lsize / 32)
    uint64_t off[kMaxN];                // word offset of u's bitmaps in the level pools
    int64_t parent_off[kMaxN];          // source reference (SourceLevel) of the parent's bitmaps
                                        //   for u, or -1
    int64_t push_off[kMaxPush][kMaxN];  // further sub-patterns (one edge less) of the previous
                                        //   growth level: source reference of their bitmaps for
                                        //   u's image, or -1
    uint32_t filter_mask;               // bit u: domain init tests u's degree and neighbour labels (clear
                                        //   when u's parent domain passed the same test: same degree and
                                        //   neighbour-label requirements in the parent); the engine then
                                        //   gives u a wide domain-init item (kWideItem)
    int8_t hub_shift[kMaxN];            // searches from u split a hub's first depth above
                                        //   hub_span << shift (negative: >>); kNoHubSplit: never
    int32_t nlf_n[kMaxN];               // neighbour-label-frequency requirements of u
    uint8_t nlf_lab[kMaxN][kMaxNlf];
    uint8_t nlf_cnt[kMaxN][kMaxNlf];
    uint8_t order[kMaxN][kMaxN];        // [start vertex][depth] -> pattern vertex
    // (the backward-neighbour mask of depth d, adj[order[d]] & {order[0..d-1]}, is derived on the
    // device when a search loads its plan)
};

// Mutable per-pattern state, updated with atomics by the kernels.
struct PatStatus {
    uint32_t dom_size[kMaxN];
    uint32_t found_cnt[kMaxN];
    uint32_t fail_cnt[kMaxN];
    uint32_t done_mask;     // representatives whose found count reached tau
    uint32_t state;         // 0 running, 1 frequent, 2 infrequent
    uint32_t changed;       // bit r: refinement round r removed a candidate
    uint32_t pad;
    unsigned long long searches;      // candidate checks started
    unsigned long long steps;         // candidate chunks evaluated by the search
    unsigned long long bytes;         // algorithmic bytes read by the search (logical loads)
    unsigned long long max_steps;     // longest single search (chunk evaluations)
    unsigned long long isects;        // set intersections: chunk evaluations x backward neighbours
    unsigned long long steps_u[kMaxN];  // chunk evaluations spent on u's candidates (incl. splits)
    uint32_t searches_u[kMaxN];         // searches started for u's candidates
};

enum : uint32_t { kRunning = 0, kFrequent = 1, kInfrequent = 2 };

// Domain-init items are (pattern << 8 | vertex); a wide one (this bit set) covers 32 bitmap words
// per unit, one lane per word, for a vertex whose words are only its sources' words ANDed.
constexpr uint32_t kWideItem = 0x80000000u;
constexpr int8_t kNoHubSplit = 127;  // PatDesc::hub_shift: no hub split for this start vertex

// Work item of the search kernel: a run of bitmap words of one representative's domain.
struct SearchItem {
    uint32_t pat;
    uint16_t u;
    uint16_t pad;
    uint32_t word_lo;
    uint32_t word_hi;
};

// The search work of one call, decoded by the search kernel from two small tables instead of an
// item array.  The call's (pattern, representative vertex) pairs form groups (in the engine: the
// k-th representative of every pattern of a window); the items of a group run round by round,
// round t holding run t (of `chunk_words` bitmap words) of every entry with more than t runs.
// Entries are sorted by run count, descending, so the entries active in a round are a prefix and
// item k of a group is found by a binary search over `before`.
struct ItemEntry {
    uint32_t pat;
    uint16_t u;
    uint16_t pad;
    uint32_t words;      // bitmap words of u's domain
    uint32_t runs;       // ceil(words / chunk_words), >= 1
    uint64_t before;     // items of the group in rounds [0, runs)
};
struct ItemGroup {
    uint64_t first_item;  // items of the earlier groups
    uint32_t first_entry;
    uint32_t n_entries;   // >= 1
};

// Item `k` (< the items of all groups).
#ifdef __CUDACC__
__host__ __device__
#endif
inline SearchItem item_at(const ItemGroup *gr, uint32_t n_groups, const ItemEntry *en, uint32_t chunk_words,
                          uint64_t k) {
    uint32_t lo = 0, hi = n_groups;  // the last group whose first item is <= k
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (gr[mid].first_item <= k) lo = mid;
        else hi = mid;
    }
    const ItemGroup G = gr[lo];
    const ItemEntry *e = en + G.first_entry;
    const uint64_t kk = k - G.first_item;
    // the last entry i with before > kk: rounds [runs of i + 1, runs of i) hold entries 0..i
    uint32_t a = 0, b = G.n_entries;
    while (b - a > 1) {
        const uint32_t mid = (a + b) >> 1;
        if (e[mid].before > kk) a = mid;
        else b = mid;
    }
    const uint64_t below = a + 1 < G.n_entries ? e[a + 1].before : 0;
    const uint32_t r0 = a + 1 < G.n_entries ? e[a + 1].runs : 0;
    const uint64_t off = kk - below;
    const uint32_t t = r0 + (uint32_t)(off / (a + 1));
    const ItemEntry &E = e[off % (a + 1)];
    SearchItem it;
    it.pat = E.pat;
    it.u = E.u;
    it.pad = 0;
    it.word_lo = t * chunk_words;
    it.word_hi = it.word_lo + chunk_words < E.words ? it.word_lo + chunk_words : E.words;
    return it;
}

// Bits of a 32-candidate word that belong to part `part` of 2^log2 interleaved parts.
#ifdef __CUDACC__
__host__ __device__
#endif
inline uint32_t part_mask(uint32_t part, uint32_t log2) {
    uint32_t m = 0;
    const uint32_t step = 1u << log2;
    for (uint32_t b = part; b < 32; b += step) m |= 1u << b;
    return m;
}

// Split task: an unexplored part of one (u, v) search — the candidates at positions [lo, hi) of the
// anchor list at `depth`, below the partial embedding prefix[0..depth-1] (data vertices of the
// pattern vertices order[0..depth-1] of u's matching order).  A search that exceeds its step budget
// turns its whole unexplored remainder, at every depth, into such tasks (parallel/comper.h:640-749
// spawns every remaining branch with its partial embedding the same way); a search whose first
// depth is a hub's long adjacency range does so at once.
struct SplitTask {
    uint32_t pat;
    uint16_t u;
    uint8_t depth;
    uint8_t pad;
    uint32_t v;              // candidate of u: the search this task belongs to
    uint32_t lo, hi;         // anchor positions at `depth`
    uint32_t group;          // index of the group that decides v
    uint32_t prefix[kTaskMaxN];  // prefix[k] = data vertex of order[k], k < depth
};

// All tasks of one (u, v) search; the last task to finish decides v when none found an embedding
// (parallel/taskprogmap.h:10-85 tracks a split search's subtasks the same way).
constexpr uint32_t kNullTask = 0xffffffffu;  // SplitTask::pat of a slot that holds no task

struct SplitGroup {
    uint32_t pat;
    uint16_t u;
    uint16_t pad;
    uint32_t v;
    uint32_t pending;    // tasks not yet finished
    uint32_t incomplete; // a task stopped without an answer (pattern decided, or set aside for the
                         //   next pass): failure cannot be concluded
};

// Split rounds after a search pass: every round but the last possible one (kMaxRounds - 1) has a
// step budget, so a task keeps being cut until the rounds drain.
constexpr int kMaxRounds = 64;
// Counters of one search pass: [0] next item, [1] groups used, [2 + r] tasks written for round r
// (may pass the buffer capacity; readers clamp), [kClaimBase + r] next task of round r to process,
// [kCntAbandoned] searches and tasks set aside for the next pass (no room for their remainder) and
// teams that stopped starting searches because the buffers were full.
constexpr int kClaimBase = 2 + kMaxRounds + 1;
constexpr int kCntAbandoned = kClaimBase + kMaxRounds + 1;
constexpr int kNumCounters = kCntAbandoned + 1;
// Search passes per engine call: a search may take step_budget chunk steps before its remainder
// becomes split tasks; what did not fit the buffers is retried by the next pass, whose budgets are
// 8x larger; in the last pass such a search finishes in place.
constexpr int kMaxPasses = 4;

struct SearchParams {
    uint32_t tau;
    uint32_t exact;          // 1: evaluate every candidate, no early exit
    uint32_t n_items;
    uint32_t split;          // 0: searches never split (no buffers needed)
    uint32_t step_budget;    // chunk evaluations before a search is split
    uint32_t split_slice;    // anchor positions per split task
    uint32_t hub_span;       // a search whose first depth has more anchor positions than this is
                             //   split at once ...
    uint32_t hub_parts;      //   ... into this many tasks (1: off)
    uint32_t isect_ratio;    // a further backward neighbour's range at most this many times the
                             //   anchor's is merged, a longer one probed
    uint32_t split_cap;      // capacity of each of the two split-task buffers
    uint32_t split_slack;    // slots above a sliced-claim limit, kept for compact remainders
    uint32_t search_fill;    // sliced-claim limit of the search pass (the split rounds use
                             //    split_cap - split_slack): the rounds' tasks can outnumber it
    uint32_t group_cap;      // capacity of the split-group buffer
    uint32_t last;           // 1: the last pass (a remainder without room finishes in place);
                             //   0: it is set aside for the next pass
    uint32_t team_lanes;     // lanes per search: 32, or 8 (four searches per warp; patterns of at
                             //    most 8 vertices)
    uint32_t parts_log2;     // every item is claimed 2^parts_log2 times, claim k searching the bits b of
                             //    its words with b % 2^parts_log2 == k (small calls: more warps busy)
    uint32_t n_pats;         // patterns of the batch
    uint32_t max_n;          // vertices of the batch's largest searched pattern (> kTaskMaxN: no splits)
    uint32_t n_groups;       // item groups (ItemGroup) of the call
    uint32_t chunk_words;    // bitmap words per item
    uint64_t words;          // size of each level bitmap pool (32-bit words)
};

}  // namespace dev
}  // namespace tfsm
