// Device-side data layout shared by the host engine and the kernels.
//
// Data graph in HBM (built once per graph, read-only afterwards):
//   vertices are renumbered so that each frequent vertex label owns one contiguous id range
//   [label_start[L], label_start[L+1]) — ids keep the reference's pruned order inside a label.
//   row_off[n+1] (u32) / col[2m] (u32, ascending) / elab[2m] (u8, dense edge label)
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

constexpr int kMaxN = 16;          // pattern vertices supported by the device path
constexpr uint8_t kNoEdge = 0xff;  // edge-label matrix entry for "not adjacent"

struct Graph {
    uint32_t n = 0;
    uint64_t m2 = 0;                 // directed adjacency entries (2 * undirected edges)
    int n_labels = 0;
    const uint32_t *row_off = nullptr;   // [n+1]; the host rejects graphs with >= 2^32 adjacency entries
    const uint32_t *col = nullptr;
    const uint8_t *elab = nullptr;
    const uint32_t *label_start = nullptr;  // [n_labels + 1]
    // lab_off[v * lab_stride + L] = position in col of v's first neighbour with label >= L, for
    // L = 0..n_labels: the neighbours of v with label L are [lab_off[.. + L], lab_off[.. + L + 1]).
    const uint32_t *lab_off = nullptr;
    uint32_t lab_stride = 0;                // n_labels + 1
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
    int32_t nlf_n[kMaxN];               // neighbour-label-frequency requirements of u
    uint8_t nlf_lab[kMaxN][kMaxN];
    uint8_t nlf_cnt[kMaxN][kMaxN];
    uint8_t order[kMaxN][kMaxN];        // [start vertex][depth] -> pattern vertex
    uint32_t bn[kMaxN][kMaxN];          // [start vertex][depth] -> backward-neighbour mask
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

// Work item of the search kernel: a run of bitmap words of one representative's domain.
struct SearchItem {
    uint32_t pat;
    uint16_t u;
    uint16_t pad;
    uint32_t word_lo;
    uint32_t word_hi;
};

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

// Split task: a donated part of one (u, v) search — the candidates at anchor positions [lo, hi) of
// depth `depth` of u's matching order, below the partial embedding prefix[0..depth-1] (data
// vertices of the pattern vertices order[0..depth-1]).  A search shares out the unexplored
// remainder of its shallowest open depth this way when other teams wait for work, when it has run
// past its step budget, or at once when its first level is a hub's long adjacency range
// (parallel/comper.h:640-749 spawns the remaining branches of a timed-out search with their
// partial embeddings the same way).
struct SplitTask {
    uint32_t pat;
    uint16_t u;
    uint8_t depth;
    uint8_t pad;
    uint32_t v;              // candidate of u: the search this task belongs to
    uint32_t lo, hi;         // anchor positions at `depth`
    uint32_t group;          // group slot that decides v
    uint32_t prefix[kMaxN];  // prefix[k] = data vertex of order[k], k < depth
};
constexpr int kTaskWords = sizeof(SplitTask) / 4;
static_assert(sizeof(SplitTask) % 4 == 0, "task words");

// One slot of the work queue, a bounded multi-producer multi-consumer ring with a sequence number
// per slot (D. Vyukov's bounded MPMC queue): the slot of position p is free for a producer when
// seq == p, holds a task for a consumer when seq == p + 1, and is handed to position p + capacity
// by the consumer that took it.  Producers and consumers claim positions with compare-and-swap on
// the ring's tail / head; no one ever waits on a slot, so a full ring only refuses a donation and
// an empty one only sends the team on to other work.
struct QueueCell {
    uint32_t seq;
    uint32_t pad;
    SplitTask task;
};
static_assert(sizeof(QueueCell) % 8 == 0, "queue cell alignment");

// Group of a split search: one 32-bit word per slot in a recycled table, the number of units (the
// donor and its tasks) not yet finished, plus kGroupIncomplete when one of them stopped without an
// answer (its pattern was decided).  0 is a free slot; a donor claims one with CAS 0 -> 1 and adds
// the tasks it donates before they become visible; the unit whose decrement reaches zero frees
// the slot and, when no unit found an embedding and none stopped early, records v's failure.
constexpr uint32_t kNoGroup = 0xffffffffu;
constexpr uint32_t kGroupIncomplete = 0x80000000u;

// Counters of one search pass (zeroed before the call), one per 128-byte line: the hot ones are
// polled by every waiting team.
enum : int {
    kCntItem = 0,     // next work item
    kCntWork,         // outstanding units: teams inside an item, tasks queued or running
    kCntIdle,         // teams waiting for work
    kCntGroupCursor,  // next group slot to try
    kCntGroups,       // searches that donated (groups claimed)
    kCntTasks,        // tasks donated
    kCntRefused,      // donations refused (no free group slot, or the ring full)
    kCntWaitExpired,  // teams that stopped waiting at the wait limit (a statistic, not an error)
    kCntQueueMax,     // deepest ring seen by a donor
    kCntBadTask,      // tasks taken off the ring with fields out of range (skipped; an engine fault)
    kCntAbandoned,    // searches set aside at the pass's step budget (the next pass retries them)
    kNumCounters
};
constexpr int kCntStride = 32;                       // u32 per counter line
constexpr int kPassCounters = kNumCounters * kCntStride;
constexpr int kMaxPasses = 4;                        // search passes per call
constexpr int kQctlHead = 0, kQctlTail = kCntStride;  // ring positions, one line each

struct SearchParams {
    uint32_t tau;
    uint32_t exact;          // 1: evaluate every candidate, no early exit
    uint32_t n_items;
    uint32_t split;          // 0: searches never donate (no ring or group table needed)
    uint32_t split_slice;    // least anchor positions per donated part of the current depth
    uint32_t hub_span;       // a search whose first depth has more anchor positions than this
                             //   shares it out at once ...
    uint32_t hub_parts;      //   ... into this many parts (the donor keeps one; 1: off)
    uint32_t soft_cap;       // ring depth above which budget and hub donations are skipped
    uint32_t team_lanes;     // lanes per search: 32, or 8 (four searches per warp; patterns of at
                             //    most 8 vertices)
    uint32_t parts_log2;     // every item is claimed 2^parts_log2 times, claim k searching the bits b of
                             //    its words with b % 2^parts_log2 == k (small calls: more warps busy)
    uint32_t n_pats;         // patterns of the batch
    uint32_t qcap;           // ring slots (a power of two)
    uint32_t gcap;           // group slots (a power of two)
    uint32_t budget;         // chunk evaluations a search may take in this pass before it is set
                             //   aside for the next one (0: the last pass, no limit)
    uint32_t max_idle;       // teams that may wait for shared work at once (the others end)
    uint32_t share_steps;    // last pass: a search that has run this many chunk steps also shares
                             //   work while the ring is short of soft_cap (0: only to waiting teams)
    uint64_t words;          // size of each level bitmap pool (32-bit words)
    QueueCell *cells;        // [qcap]
    uint32_t *qctl;          // [kQctlHead] head, [kQctlTail] tail: positions, kept across launches
    uint32_t *groups;        // [gcap]
    const uint32_t *prev;    // the previous pass's counters (nullptr in the first pass): a pass
                             //   whose predecessor set nothing aside has nothing to do
};

}  // namespace dev
}  // namespace tfsm
