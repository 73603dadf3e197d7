// CUDA kernels of the MNI support evaluation (sm_103a).  Integer gather work: no tensor cores.
//
//   k_domain_init  LDF + NLF candidate filter (parallel/gmatch.h:301-415) writing one bitmap
//                  per pattern vertex over its label's id range; children start from the
//                  parent's final domain (candidates minus proven non-candidates).
//   k_refine       one arc-consistency pass over every pattern edge, incl. edge labels
//                  (pruneCandidates, parallel/gmatch.h:600-658, pull direction).  Iterated to a
//                  fixpoint for distinct-label trees, whose domains are then the exact MNI
//                  domains (parallel/comper.h:1619-1653).
//   k_search       backtracking, one search pass: a team of lanes (a warp, or a quarter of one)
//                  per (pattern vertex u, candidate v) search looks for one embedding with u -> v
//                  (LFTJ, serial/gmatch.h:906-987).  Local candidates at each depth are the label
//                  sub-range of the smallest backward neighbour's adjacency, checked G at a time
//                  (one per lane) against the domain bitmap, injectivity and every other backward
//                  neighbour (merged or probed, by their size ratio); the survivors are a ballot
//                  mask.  Found embeddings add all their vertices (and automorphic images) to the
//                  MNI domains; early exit per vertex at tau and per pattern when tau can no
//                  longer be reached (parallel/comper.h:288-297).  A search that exceeds its step
//                  budget (or starts at a hub) turns its unexplored remainder into split tasks
//                  (parallel/comper.h:640-749, 865-973).
//   k_split        one split round over those tasks; the last task of a search to finish decides
//                  its failure (parallel/taskprogmap.h:10-85).
#include <cstdint>
#include <cstdio>

#include "dev_common.cuh"
#include "kernels.h"

// Kernel launch; host-side SIMT emulation builds of this file (tests only) replace the syntax.
#ifdef TFSM_SIMT_EMULATION
#define TFSM_LAUNCH(kern, grid, block, stream, ...) tfsm_emu::launch((grid), (block), [&]() { kern(__VA_ARGS__); })
#else
#define TFSM_LAUNCH(kern, grid, block, stream, ...) kern<<<(grid), (block), 0, (stream)>>>(__VA_ARGS__)
#endif

namespace tfsm {
namespace dev {

// ---- optional self-checking build (TFSM_BOUNDS_CHECK): every global access of the search
// kernels is checked against its buffer; the first violation is recorded (site, index, bound)
// and the access is skipped, so the kernel returns normally and the host reports the record.
#ifdef TFSM_BOUNDS_CHECK
__device__ unsigned long long g_check[4];  // count, site, index, bound
__device__ __forceinline__ bool inb(uint32_t site, uint64_t idx, uint64_t bound) {
    if (idx < bound) return true;
    if (atomicAdd(&g_check[0], 1ull) == 0) {
        g_check[1] = site;
        g_check[2] = idx;
        g_check[3] = bound;
    }
    return false;
}
#define TFSM_IN(site, idx, bound) inb((site), (uint64_t)(idx), (uint64_t)(bound))
#else
#define TFSM_IN(site, idx, bound) true
#endif

namespace {

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *__restrict__ a, uint32_t lo, uint32_t hi,
                                                    uint32_t x) {
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Warp-uniform read of one bitmap word.
__device__ __forceinline__ uint32_t warp_word(const uint32_t *p, uint32_t lane) {
    uint32_t w = 0;
    if (lane == 0) w = __ldcg(p);
    return __shfl_sync(0xffffffffu, w, 0);
}

// Same, adding 4 bytes per probed element to `bytes` (algorithmic-traffic accounting).
__device__ __forceinline__ uint32_t lower_bound_cnt(const uint32_t *__restrict__ a, uint32_t lo, uint32_t hi,
                                                    uint32_t x, uint32_t &bytes, uint64_t bound = ~0ull) {
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        bytes += 4;
        if (!TFSM_IN(1, mid, bound)) return hi;
        if (__ldg(a + mid) < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t find_item(const uint64_t *__restrict__ prefix, uint32_t n_items, uint64_t gw,
                                              uint32_t hint) {
    // items are visited in increasing gw order by a warp: advance from the hint when possible
    if (hint < n_items && prefix[hint] <= gw && gw < prefix[hint + 1]) return hint;
    uint32_t lo = 0, hi = n_items;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= gw) lo = mid;
        else hi = mid;
    }
    return lo;
}

}  // namespace

// The adjacency positions [lo, hi) of v's neighbours with dense label L (label-major table).
__device__ __forceinline__ void label_range(const Graph &g, uint32_t v, uint32_t L, uint32_t &lo, uint32_t &hi) {
    const uint32_t *p = g.lab_off + (size_t)L * g.n + v;
    lo = __ldg(p);
    hi = __ldg(p + g.n);
}

// ------------------------------------------------------------------------------------------------
// K1: LDF + NLF filter.  One warp per bitmap word, one lane per vertex of the word.
// ------------------------------------------------------------------------------------------------
// Bit `lane` of word `word` of a source's final domain (dom & ~failed) at reference `ref`.
__device__ __forceinline__ bool source_bit(const SourceLevel *__restrict__ srcs, uint32_t n_srcs, int64_t ref,
                                           uint32_t word, uint32_t lane) {
    // A restriction only removes candidates, so one that cannot be read is skipped (checked
    // builds also record it): results never depend on it.
    const uint64_t slot = (uint64_t)ref >> kSrcShift;
    const uint64_t o = ((uint64_t)ref & kSrcMask) + word;
    if (!TFSM_IN(32, slot, n_srcs) || slot >= n_srcs) return true;
    const SourceLevel S = srcs[slot];
    if (!TFSM_IN(39, o, S.words) || o >= S.words) return true;
    const uint32_t w = __ldg(S.dom + o) & ~__ldg(S.failed + o);
    return (w >> lane) & 1u;
}

// Word `word` of a source's final domain (all ones when it cannot be read, as above).
__device__ __forceinline__ uint32_t source_word(const SourceLevel *__restrict__ srcs, uint32_t n_srcs, int64_t ref,
                                                uint32_t word) {
    const uint64_t slot = (uint64_t)ref >> kSrcShift;
    const uint64_t o = ((uint64_t)ref & kSrcMask) + word;
    if (!TFSM_IN(32, slot, n_srcs) || slot >= n_srcs) return 0xffffffffu;
    const SourceLevel S = srcs[slot];
    if (!TFSM_IN(39, o, S.words) || o >= S.words) return 0xffffffffu;
    return __ldg(S.dom + o) & ~__ldg(S.failed + o);
}

__global__ void __launch_bounds__(256) k_domain_init(Graph g, const PatDesc *__restrict__ descs,
                                                     PatStatus *__restrict__ st, const uint32_t *__restrict__ item_pu,
                                                     const uint64_t *__restrict__ prefix, uint32_t n_items,
                                                     uint32_t *__restrict__ dom, uint32_t *__restrict__ found,
                                                     uint32_t *__restrict__ failed,
                                                     const SourceLevel *__restrict__ srcs, uint32_t n_srcs,
                                                     uint64_t chk_words) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t total = prefix[n_items];
    uint32_t item = 0;
    for (uint64_t gw = warp; gw < total; gw += nwarps) {
        item = find_item(prefix, n_items, gw, item);
        const uint32_t pu = item_pu[item];
        const uint32_t p = (pu & ~kWideItem) >> 8, u = pu & 0xff;
        const PatDesc &D = descs[p];
        if (pu & kWideItem) {
            // u skips the degree / neighbour-label test: its words are only the sources' words
            // ANDed, 32 words per warp, one lane per word
            const uint32_t word = (uint32_t)(gw - prefix[item]) * 32 + lane;
            const bool ok = word < D.words[u] && TFSM_IN(31, D.off[u] + word, chk_words);
            uint32_t w = 0;
            if (ok) {
                const uint32_t first = word * 32;
                w = D.lsize[u] - first >= 32 ? 0xffffffffu : (1u << (D.lsize[u] - first)) - 1u;
                if (D.parent_off[u] >= 0) w &= source_word(srcs, n_srcs, D.parent_off[u], word);
                for (int k = 0; k < kMaxPush; ++k)
                    if (D.push_off[k][u] >= 0) w &= source_word(srcs, n_srcs, D.push_off[k][u], word);
                const uint64_t o = D.off[u] + word;
                dom[o] = w;
                found[o] = 0;
                failed[o] = 0;
            }
            const uint32_t cnt = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(w));
            if (lane == 0 && cnt) atomicAdd(&st[p].dom_size[u], cnt);
            continue;
        }
        const uint32_t word = (uint32_t)(gw - prefix[item]);
        const uint32_t xl = word * 32 + lane;
        bool pass = xl < D.lsize[u];
        if (!TFSM_IN(30, word, D.words[u]) || !TFSM_IN(31, D.off[u] + word, chk_words)) continue;
        // the parent's final domain, and push-down: every other one-edge-smaller sub-pattern's
        // final domain bounds u's as well (an embedding of the child restricts to one of each)
        if (D.parent_off[u] >= 0) pass = pass && source_bit(srcs, n_srcs, D.parent_off[u], word, lane);
        for (int k = 0; k < kMaxPush; ++k)
            if (D.push_off[k][u] >= 0) pass = pass && source_bit(srcs, n_srcs, D.push_off[k][u], word, lane);
        if (__any_sync(0xffffffffu, pass)) {
            const uint32_t x = D.lstart[u] + xl;
            uint32_t b = 0, e = 0;
            if (pass && !TFSM_IN(33, x, g.n)) pass = false;
            if (pass) {
                b = __ldg(g.row_off + x);
                e = __ldg(g.row_off + x + 1);
                pass = (int32_t)(e - b) >= D.deg[u];
            }
            const int nn = D.nlf_n[u];
            for (int k = 0; k < nn && pass; ++k) {
                uint32_t lo, hi;
                label_range(g, x, D.nlf_lab[u][k], lo, hi);
                pass = hi - lo >= (uint32_t)D.nlf_cnt[u][k];
            }
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, pass);
        if (lane == 0) {
            const uint64_t o = D.off[u] + word;
            dom[o] = mask;
            found[o] = 0;
            failed[o] = 0;
            if (mask) atomicAdd(&st[p].dom_size[u], (uint32_t)__popc(mask));
        }
    }
}

// ------------------------------------------------------------------------------------------------
// K2: one arc-consistency pass.  v stays in D(u) only if, for every pattern neighbour w of u,
// v has a neighbour x in D(w) reached through an edge with the pattern edge's label.
// One warp per bitmap word; the warp scans each candidate's label sub-range 32 entries at a time.
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kLaneScan = 16;  // k_refine: longest label range a single lane scans

// One arc-consistency round `round` (< 32).  A pattern takes part while every domain can still
// reach tau (any non-empty domain in exact mode) and, after the first round, while the previous
// round removed something from it (bit round - 1 of `changed`); a removal sets bit `round`.
__global__ void __launch_bounds__(256) k_refine(Graph g, const PatDesc *__restrict__ descs, PatStatus *__restrict__ st,
                                                const uint32_t *__restrict__ item_pu,
                                                const uint64_t *__restrict__ prefix, uint32_t n_items,
                                                uint32_t *__restrict__ dom, uint64_t chk_words, int round,
                                                uint32_t tau, int exact) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t total = prefix[n_items];
    uint32_t item = 0;
    for (uint64_t gw = warp; gw < total; gw += nwarps) {
        item = find_item(prefix, n_items, gw, item);
        const uint32_t pu = item_pu[item];
        const uint32_t p = (pu & ~kWideItem) >> 8, u = pu & 0xff;
        const PatDesc &D = descs[p];
        const uint32_t word = (uint32_t)(gw - prefix[item]);
        if (!TFSM_IN(34, D.off[u] + word, chk_words)) continue;
        int skip = 0;
        if (lane == 0) {
            const PatStatus &ps = st[p];
            skip = round > 0 && !((__ldcg(&ps.changed) >> (round - 1)) & 1u);
            for (int w = 0; w < D.n && !skip; ++w) {
                const uint32_t ds = __ldcg(&ps.dom_size[w]);
                skip = exact ? ds == 0 : ds < tau;
            }
        }
        if (__shfl_sync(0xffffffffu, skip, 0)) continue;
        uint32_t *wp = dom + D.off[u] + word;
        // other warps clear bits of this pool concurrently: one read, broadcast, keeps the warp's
        // control flow (and its collectives) uniform
        const uint32_t w0 = warp_word(wp, lane);
        if (w0 == 0) continue;
        // Pass 1, one candidate per lane: every pattern neighbour w needs a supporting data
        // neighbour (label, edge label, in w's domain) inside a short label range, scanned serially.
        // A candidate with a range longer than kLaneScan goes to pass 2 (the warp scans it).
        uint32_t keep_lane = 1, hard_lane = 0;
        if ((w0 >> lane) & 1u) {
            const uint32_t v = D.lstart[u] + word * 32 + lane;
            if (TFSM_IN(38, v, g.n)) {
                uint32_t nb = D.adj[u];
                while (nb && keep_lane && !hard_lane) {
                    const int w = __ffs(nb) - 1;
                    nb &= nb - 1;
                    uint32_t lo, hi;
                    label_range(g, v, D.lab[w], lo, hi);
                    if (hi - lo > kLaneScan) {
                        hard_lane = 1;
                        break;
                    }
                    const uint32_t ls = D.lstart[w];
                    const uint8_t el = D.el[u][w];
                    const uint32_t *dw = dom + D.off[w];
                    bool sup = false;
                    for (uint32_t i = lo; i < hi && !sup; ++i) {
                        if (!TFSM_IN(39, i, g.m2) || __ldg(g.elab + i) != el) continue;
                        const uint32_t xl = __ldg(g.col + i) - ls;
                        if (TFSM_IN(40, (uint64_t)D.off[w] + (xl >> 5), chk_words))
                            sup = (__ldcg(dw + (xl >> 5)) >> (xl & 31)) & 1u;
                    }
                    keep_lane = sup ? 1u : 0u;
                }
            }
        }
        const uint32_t hard = __ballot_sync(0xffffffffu, hard_lane) & w0;
        const uint32_t dropped = __ballot_sync(0xffffffffu, !keep_lane && !hard_lane) & w0;
        uint32_t keep = w0 & ~dropped;
        // Pass 2: the warp scans the long ranges of the remaining candidates together.
        uint32_t bits = hard;
        while (bits) {
            const int bit = __ffs(bits) - 1;
            bits &= bits - 1;
            const uint32_t v = D.lstart[u] + word * 32 + bit;
            if (!TFSM_IN(35, v, g.n)) continue;
            uint32_t nb = D.adj[u];
            bool ok = true;
            while (nb && ok) {
                const int w = __ffs(nb) - 1;
                nb &= nb - 1;
                const uint32_t ls = D.lstart[w];
                uint32_t lo, hi;
                label_range(g, v, D.lab[w], lo, hi);
                const uint8_t el = D.el[u][w];
                const uint32_t *dw = dom + D.off[w];
                bool sup = false;
                for (uint32_t base = lo; base < hi && !sup; base += 32) {
                    const uint32_t i = base + lane;
                    bool hit = false;
                    if (i < hi && TFSM_IN(36, i, g.m2) && __ldg(g.elab + i) == el) {
                        const uint32_t xl = __ldg(g.col + i) - ls;
                        if (TFSM_IN(37, (uint64_t)D.off[w] + (xl >> 5), chk_words))
                            hit = (__ldcg(dw + (xl >> 5)) >> (xl & 31)) & 1u;
                    }
                    sup = __any_sync(0xffffffffu, hit);
                }
                ok = sup;
            }
            if (!ok) keep &= ~(1u << bit);
        }
        if (keep != w0 && lane == 0) {
            atomicAnd(wp, keep);
            atomicSub(&st[p].dom_size[u], (uint32_t)__popc(w0 & ~keep));
            atomicOr(&st[p].changed, 1u << round);
        }
    }
}


// ------------------------------------------------------------------------------------------------
// K5 / K6: search passes and split rounds.
// ------------------------------------------------------------------------------------------------
namespace {

// A team: the G lanes (32 or 8) of a warp that run one search.  Small teams run several
// independent searches per warp, which pays when label ranges are short (most lanes of a
// 32-candidate chunk would idle); every collective is masked to the team's lanes.
template <int G>
struct Team {
    uint32_t lane;  // 0 .. G-1
    uint32_t base;  // first warp lane of the team
    uint32_t mask;  // the team's lanes in the warp
    __device__ explicit Team(uint32_t warp_lane)
        : lane(warp_lane & (G - 1)), base(warp_lane & ~(uint32_t)(G - 1)),
          mask(G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (warp_lane & ~(uint32_t)(G - 1)))) {}
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ uint32_t ballot(bool p) const {
        const uint32_t b = __ballot_sync(mask, p);
        return G == 32 ? b : (b >> base) & ((1u << G) - 1u);
    }
    template <class T>
    __device__ __forceinline__ T bcast(T v, int src) const {
        return __shfl_sync(mask, v, src, G);
    }
    template <class T>
    __device__ __forceinline__ T xor_shfl(T v, int m) const {
        return __shfl_xor_sync(mask, v, m, G);
    }
    __device__ __forceinline__ bool any(bool p) const { return __any_sync(mask, p); }
    __device__ __forceinline__ uint32_t sum(uint32_t v) const { return __reduce_add_sync(mask, v); }
    // leader reads a word that other teams may update; the team gets one value
    __device__ __forceinline__ uint32_t word(const uint32_t *p) const {
        uint32_t w = 0;
        if (lane == 0) w = __ldcg(p);
        return bcast(w, 0);
    }
};

// Block shape of a search kernel with teams of G lanes holding state for patterns of up to N
// vertices: the 32-vertex state (about 11 KB per team) fits four whole-warp teams per block in
// static shared memory, and so do the 32 teams of 4 lanes of four warps; otherwise kSearchWarps
// warps.
template <int G, int N>
struct SearchBlock {
    // 32-vertex state, or eight teams of 4 lanes per warp: four warps per block (static shared memory)
    static constexpr int warps = N > kTaskMaxN || G == 4 ? 4 : kSearchWarps;
    static constexpr int min_blocks = N > kTaskMaxN || G == 4 ? 2 * kSearchMinBlocks : kSearchMinBlocks;
};

template <int N>
struct Plan {
    uint32_t off[N];
    uint32_t lstart[N];
    uint32_t lend[N];
    uint32_t orbit[N];
    uint32_t bn[N];       // by depth
    uint8_t order[N];     // by depth
    uint8_t lab[N];       // dense label by pattern vertex
    uint8_t el[N][N];
    int32_t n;
    uint32_t repmask;
    uint32_t key;         // (pattern << 8 | start vertex) the plan was loaded for
    uint64_t words;       // size of the level's bitmap pools (checked builds)
};

template <int N>
struct State {
    uint32_t emb[N];      // by pattern vertex
    uint32_t pos[N];      // by depth: next unevaluated anchor position
    uint32_t end[N];      // by depth: end of the anchor range
    uint32_t base[N];     // by depth: first position of the chunk held in mask / rest
    uint32_t mask[N];     // by depth: surviving candidates already known to be in w's MNI domain
    uint32_t rest[N];     // by depth: the other surviving candidates (tried after `mask`)
    uint8_t anchor[N];    // by depth: pattern vertex whose adjacency is scanned
    uint32_t merge[N];    // by depth: backward neighbours intersected by merging (bit b), the
                          //   others by probing
    uint32_t blo[N][N];   // [depth][backward neighbour b]: the unconsumed part of order[depth]'s
    uint32_t bhi[N][N];   //   label range inside emb[b]'s adjacency (blo advances chunk by chunk)
};

// Staging tile of the merge form: 4 elements per lane, filled with one 128-bit load each.
template <int G>
struct Tile {
    uint32_t v[4 * G];
};

enum : int { kFail = 0, kFound = 1, kAbort = 2, kCancel = 3 };

// What makes a running search pointless: the searched (u, v) has been found by another team's
// embedding, or the pattern (or, lazily, vertex u) has been decided.  Checked every kCheckEvery
// chunk steps; a cancelled search proves nothing about v.
struct Cancel {
    const uint32_t *found_word;  // found-bitmap word holding (u, v)
    uint32_t bit;
    const PatStatus *ps;
    int u;
    bool exact;
};
constexpr uint32_t kCheckEvery = 16;

// Try candidates already known to be in w's MNI domain first.  Measured slower on the benchmark
// graphs (the extra ballot and found-word loads cost more than the reordering saves): off.
constexpr bool kFoundFirst = false;

template <int G, int N>
__device__ __forceinline__ void load_plan(const Team<G> &T, Plan<N> &P, const PatDesc &D, uint32_t p, int u,
                                          uint64_t words) {
    const uint32_t key = (p << 8) | (uint32_t)u;
    if (P.key == key) return;  // every lane of the team reads the same shared value
    T.sync();
    for (uint32_t i = T.lane; i < (uint32_t)N; i += G) {
        P.off[i] = (uint32_t)D.off[i];
        P.lstart[i] = D.lstart[i];
        P.lend[i] = D.lstart[i] + D.lsize[i];
        P.orbit[i] = D.orbit_mask[i];
        uint32_t before = 0;  // the pattern vertices matched before depth i
        for (uint32_t k = 0; k < i; ++k) before |= 1u << D.order[u][k];
        P.bn[i] = i < (uint32_t)D.n ? D.adj[D.order[u][i]] & before : 0u;
        P.order[i] = D.order[u][i];
        P.lab[i] = (uint8_t)D.lab[i];
    }
    for (uint32_t i = T.lane; i < (uint32_t)(N * N); i += G) P.el[i / N][i % N] = D.el[i / N][i % N];
    if (T.lane == 0) {
        P.n = D.n;
        uint32_t rm = 0;
        for (int k = 0; k < D.n; ++k)
            if (D.rep[k] == k) rm |= 1u << k;
        P.repmask = rm;
        P.key = key;
        P.words = words;
    }
    T.sync();
}

// Anchor of depth d: the backward neighbour whose label sub-range is the shortest.  Lane k
// handles the k-th backward neighbour; a team minimum picks the winner.  Every other backward
// neighbour's range is marked for merging when it is at most `ratio` times the anchor's, else for
// probing: the reference's rule (intersection/computesetintersection.cpp:9-44 gallops when one
// list is more than 50 times the other).
template <int G, int N>
__device__ __forceinline__ void setup_depth(const Team<G> &T, const Graph &g, const Plan<N> &P, State<N> &S, int d,
                                            uint32_t ratio, uint32_t &bytes) {
    const int w = P.order[d];
    const uint32_t bnm = P.bn[d];
    const int nb = __popc(bnm);
    unsigned long long key = ~0ull;
    uint32_t lo = 0, hi = 0;
    int b = 0;
    if ((int)T.lane < nb) {
        uint32_t m = bnm;
        for (uint32_t k = 0; k < T.lane; ++k) m &= m - 1;
        b = __ffs(m) - 1;
        const uint32_t y = S.emb[b];
        if (TFSM_IN(2, y, g.n)) {
            label_range(g, y, P.lab[w], lo, hi);
            bytes += 8;
        }
        S.blo[d][b] = lo;  // lane k owns backward neighbour b's slot
        S.bhi[d][b] = hi;
        key = ((unsigned long long)(hi - lo) << 32) | T.lane;
    }
#pragma unroll
    for (int s = G / 2; s > 0; s >>= 1) {
        const unsigned long long o = T.xor_shfl(key, s);
        key = o < key ? o : key;
    }
    const int win = (int)(key & (unsigned long long)(G - 1));
    const uint32_t alen = (uint32_t)(key >> 32);
    uint32_t mbit = (int)T.lane < nb && (int)T.lane != win && (uint64_t)(hi - lo) <= (uint64_t)ratio * alen
                        ? 1u << b
                        : 0u;
#pragma unroll
    for (int s = G / 2; s > 0; s >>= 1) mbit |= T.xor_shfl(mbit, s);
    lo = T.bcast(lo, win);
    hi = T.bcast(hi, win);
    b = T.bcast(b, win);
    if (T.lane == 0) {
        S.pos[d] = lo;
        S.end[d] = hi;
        S.mask[d] = 0;
        S.rest[d] = 0;
        S.anchor[d] = (uint8_t)b;
        S.merge[d] = mbit;
    }
    T.sync();
}

// Is adjacency position `idx` of the depth-d anchor a valid extension apart from the other
// backward neighbours (one lane, one position): edge label, domain bit, not failed, injective.
// `known` is set when x is already proven to be in w's MNI domain (a found embedding maps w to x).
// A candidate proven to be in no embedding as w (its `failed` bit) is rejected: sound pruning.
template <int N>
__device__ __forceinline__ bool check_candidate(const Graph &g, const Plan<N> &P, const State<N> &S,
                                                const uint32_t *__restrict__ dom, const uint32_t *found,
                                                const uint32_t *failed, int d, uint32_t idx, uint32_t &x_out,
                                                bool &known, uint32_t &bytes) {
    const int w = P.order[d];
    const int a = S.anchor[d];
    if (!TFSM_IN(3, idx, g.m2)) return false;
    const uint32_t x = __ldg(g.col + idx);
    x_out = x;
    bytes += 5;  // neighbour id + edge label
    if (__ldg(g.elab + idx) != P.el[w][a]) return false;
    const uint32_t xl = x - P.lstart[w];
    bytes += 4;  // domain bitmap word
    if (!TFSM_IN(4, (uint64_t)P.off[w] + (xl >> 5), P.words)) return false;
    const uint32_t wi = P.off[w] + (xl >> 5), bit = 1u << (xl & 31);
    if (!(__ldg(dom + wi) & bit)) return false;
    bytes += 4;  // failed word
    if (__ldcg(failed + wi) & bit) return false;
    if (kFoundFirst) {
        bytes += 4;
        known = (__ldcg(found + wi) & bit) != 0;
    }
    for (int k = 0; k < d; ++k)
        if (S.emb[P.order[k]] == x) return false;
    return true;
}

// Does adjacency position `pos` of a sorted run [.., hi), or one of the parallel edges after it,
// hold x with edge label `want`?
__device__ __forceinline__ bool edge_at(const Graph &g, uint32_t pos, uint32_t hi, uint32_t x, uint8_t want,
                                        uint32_t &bytes) {
    while (pos < hi && TFSM_IN(6, pos, g.m2) && __ldg(g.col + pos) == x) {  // parallel edges: any with the label
        bytes += 5;
        if (__ldg(g.elab + pos) == want) return true;
        ++pos;
    }
    return false;
}

// Team-uniform: the lanes' candidates x (where `ok`) intersected with the label ranges of the
// depth's other backward neighbours.  The lanes' x ascend with the lane (consecutive anchor
// positions), and so do the chunks of one depth visit, so each range is consumed front to back:
//   merge   (range at most isect_ratio times the anchor's): the range is streamed from its cursor
//           blo in tiles of 4G elements, one 128-bit load per lane, each lane looks its x up in the
//           tile in shared memory, and the cursor moves to the chunk's largest x;
//   probe   (a much longer range): each lane binary-searches its x in [blo, bhi), and blo moves to
//           the largest x's position (the galloping start of the next chunk).
template <int G, int N>
__device__ __forceinline__ bool intersect_others(const Team<G> &T, const Graph &g, const Plan<N> &P, State<N> &S,
                                                 Tile<G> &tile, int d, uint32_t x, bool ok, uint32_t &bytes) {
    const int w = P.order[d];
    uint32_t others = P.bn[d] & ~(1u << S.anchor[d]);
    while (others) {
        const int b = __ffs(others) - 1;
        others &= others - 1;
        const uint32_t lo = S.blo[d][b], hi = S.bhi[d][b];
        const bool merge = (S.merge[d] >> b) & 1u;
        const uint32_t surv = T.ballot(ok);  // also orders every lane's reads before lane 0's writes
        if (!surv) return false;
        const uint8_t want = P.el[w][b];
        const int top = 31 - __clz(surv);
        const uint32_t xtop = T.bcast(x, top);  // the chunk's largest surviving candidate
        uint32_t next = hi;                      // blo for the next chunk
        if (merge) {
            bool hit = false;
            uint32_t cur = lo;
            while (cur < hi) {
                const uint32_t base = cur & ~3u;  // 16-byte aligned (col is 256-byte aligned)
                const uint32_t first = base + 4 * T.lane;
                if (first < hi) {  // col is padded: the 4 elements never pass its allocation
                    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(g.col + first));
                    tile.v[4 * T.lane] = q.x;
                    tile.v[4 * T.lane + 1] = q.y;
                    tile.v[4 * T.lane + 2] = q.z;
                    tile.v[4 * T.lane + 3] = q.w;
                    const uint32_t valid = hi - first;
                    bytes += 4 * (valid < 4 ? valid : 4);
                }
                T.sync();
                const uint32_t n_t = hi - base < 4u * G ? hi - base : 4u * G;
                const uint32_t lo_t = cur - base;
                if (ok && !hit) {
                    uint32_t l = lo_t, h = n_t;
                    while (l < h) {
                        const uint32_t m = (l + h) >> 1;
                        if (tile.v[m] < x) l = m + 1;
                        else h = m;
                    }
                    if (l < n_t && tile.v[l] == x) hit = edge_at(g, base + l, hi, x, want, bytes);
                }
                const uint32_t last = tile.v[n_t - 1];
                uint32_t stop = n_t;
                if (last >= xtop) {  // every candidate of the chunk lies inside this tile: the
                    uint32_t l = lo_t, h = n_t;  // cursor stops at the first element >= xtop
                    while (l < h) {
                        const uint32_t m = (l + h) >> 1;
                        if (tile.v[m] < xtop) l = m + 1;
                        else h = m;
                    }
                    stop = l;
                }
                T.sync();  // every lane is done with the tile before it is refilled
                cur = base + stop;
                if (last >= xtop) break;
            }
            next = cur < hi ? cur : hi;
            ok = ok && hit;
        } else {
            uint32_t at = hi;
            bool hit = false;
            if (ok) {
                at = lower_bound_cnt(g.col, lo, hi, x, bytes, g.m2);
                hit = edge_at(g, at, hi, x, want, bytes);
            }
            next = T.bcast(at, top);
            ok = ok && hit;
        }
        if (T.lane == 0) S.blo[d][b] = next;
    }
    return ok;
}

// Unexplored anchor positions left at depth j of a search that stopped at depth `dabort`: the
// not-yet-taken candidates of j's current chunk, then [pos[j], end[j]).  Candidates of a chunk are
// taken lowest position first, so everything below the lowest pending one is explored.
template <int N>
__device__ __forceinline__ void remainder_at(const State<N> &S, int j, int dabort, uint32_t &from, uint32_t &to) {
    to = S.end[j];
    const uint32_t m = S.mask[j] | S.rest[j];
    from = (j == dabort || m == 0) ? S.pos[j] : S.base[j] + (uint32_t)(__ffs(m) - 1);
    if (from > to) from = to;
}

// Depth-first search for one embedding that extends the partial embedding of depths < start
// (S.emb[order[0..start-1]]).  With `slice`, depth `start` scans only anchor positions [lo, hi).
// The search never backtracks above `start`.  Returns kAbort once `budget` chunk evaluations are
// exceeded (budget 0: unlimited), or at once when the first depth of an unsliced search is longer
// than `hub_span` (hub_span 0: never); `abort_depth` then says where it stopped.  Returns kCancel
// when `cancel` says the search no longer matters.  A chunk is G consecutive anchor positions.
template <int G, int N>
__device__ __forceinline__ int dfs(const Team<G> &T, const Graph &g, const Plan<N> &P, State<N> &S, Tile<G> &tile,
                                   const uint32_t *__restrict__ dom, const uint32_t *found, const uint32_t *failed,
                                   int start, bool slice, uint32_t lo, uint32_t hi, uint32_t budget,
                                   uint32_t hub_span, uint32_t ratio, const Cancel &cancel, uint32_t &steps,
                                   int &abort_depth, uint32_t &bytes, uint32_t &isects) {
    const int n = P.n;
    setup_depth(T, g, P, S, start, ratio, bytes);
    if (slice) {
        if (T.lane == 0) {
            S.pos[start] = lo;
            S.end[start] = hi;
        }
        T.sync();
    } else if (hub_span && S.end[start] - S.pos[start] > hub_span) {
        abort_depth = start;  // a hub's first depth: split before any step
        return kAbort;
    }
    const uint32_t every = budget && budget < kCheckEvery ? budget : kCheckEvery;
    int d = start;
    for (;;) {
        const uint32_t mk = S.mask[d], mr = S.rest[d];
        const uint32_t pos = S.pos[d], end = S.end[d];
        // every lane has read this depth's state before lane 0 may overwrite it below
        T.sync();
        if ((mk | mr) == 0) {
            if (pos >= end) {
                if (d == start) return kFail;
                --d;
                continue;
            }
            if (budget && steps >= budget) {
                abort_depth = d;
                return kAbort;
            }
            if (steps && steps % every == 0) {
                int c = 0;
                if (T.lane == 0) {
                    c = (__ldcg(cancel.found_word) & cancel.bit) || __ldcg(&cancel.ps->state) != kRunning ||
                        (!cancel.exact && ((__ldcg(&cancel.ps->done_mask) >> cancel.u) & 1u));
                }
                if (T.bcast(c, 0)) return kCancel;
            }
            const uint32_t idx = pos + T.lane;
            uint32_t x = 0;
            bool known = false;
            bool ok = idx < end && check_candidate(g, P, S, dom, found, failed, d, idx, x, known, bytes);
            ok = intersect_others(T, g, P, S, tile, d, x, ok, bytes);
            const uint32_t bal = T.ballot(ok);
            const uint32_t pref = kFoundFirst ? T.ballot(ok && known) : 0u;
            ++steps;
            isects += (uint32_t)__popc(P.bn[d]);
            if (d == n - 1) {
                if (bal) {
                    if ((int)T.lane == __ffs(bal) - 1) S.emb[P.order[d]] = x;
                    T.sync();
                    return kFound;
                }
                if (T.lane == 0) S.pos[d] = pos + G;
                T.sync();
                continue;
            }
            if (T.lane == 0) {
                S.base[d] = pos;
                S.pos[d] = pos + G;
                S.mask[d] = pref;
                S.rest[d] = bal & ~pref;
            }
            T.sync();
            continue;
        }
        // candidates known to be in w's MNI domain first: they usually complete an embedding
        const bool from_pref = mk != 0;
        const uint32_t m = from_pref ? mk : mr;
        const int i = __ffs(m) - 1;
        if (T.lane == 0) {
            if (from_pref) S.mask[d] = m & (m - 1);
            else S.rest[d] = m & (m - 1);
            if (TFSM_IN(7, S.base[d] + i, g.m2)) S.emb[P.order[d]] = __ldg(g.col + S.base[d] + i);
        }
        T.sync();
        bytes += 4;  // re-read of the chosen neighbour id
        if (!TFSM_IN(8, d + 1, n)) return kFail;
        ++d;
        setup_depth(T, g, P, S, d, ratio, bytes);
    }
}

// Claims `k` consecutive slots below `limit` with one atomicAdd (no retry loop, so no spurious
// failure under contention); false when they do not all fit.  The counter may then pass `limit`
// (readers clamp it to the buffer size); a failed claim [first, first + k) still owns its slots
// that lie inside the buffer and must fill them (split tasks: with null tasks).  A counter already
// at `limit` is not advanced, so it passes `limit` by at most one claim per running team.
__device__ __forceinline__ bool reserve(uint32_t *counter, uint32_t k, uint32_t limit, uint32_t &first) {
    if (__ldcg(counter) >= limit) {
        first = 0xffffffffu;
        return false;
    }
    first = atomicAdd(counter, k);
    return first <= limit && k <= limit - first;
}

// Team-uniform claim of `k` slots below `limit`; the slots of a failed claim inside the buffer
// (`cap`) become null tasks.
template <int G>
__device__ __forceinline__ bool claim_tasks(const Team<G> &T, SplitTask *out, uint32_t *out_count, uint32_t k,
                                            uint32_t limit, uint32_t cap, uint32_t &t0) {
    int ok = 0;
    if (T.lane == 0) ok = reserve(out_count, k, limit, t0) ? 1 : 0;
    ok = T.bcast(ok, 0);
    t0 = T.bcast(t0, 0);
    if (!ok && t0 < cap) {
        const uint32_t e = (uint64_t)t0 + k < cap ? t0 + k : cap;
        for (uint32_t q = t0 + T.lane; q < e; q += G) out[q].pat = kNullTask;
    }
    return ok != 0;
}

// Writes the unexplored remainder of the current search (depths start..dabort) as split tasks:
// sliced (`slice` anchor positions each) below `limit`; when that does not fit, compact (one task
// per depth, re-split by later rounds) below limit + slack.  Returns how many were written; 0 when
// neither fits (then nothing is written).
template <int G, int N>
__device__ uint32_t emit_remainder(const Team<G> &T, const Plan<N> &P, const State<N> &S, uint32_t p, int u,
                                   uint32_t v, int start, int dabort, uint32_t group, uint32_t slice, SplitTask *out,
                                   uint32_t *out_count, uint32_t cap, uint32_t limit, uint32_t slack, uint64_t m2) {
    uint32_t total = 0, depths = 0;
    for (int j = start; j <= dabort; ++j) {
        uint32_t f, t;
        remainder_at(S, j, dabort, f, t);
        total += t > f ? (t - f - 1) / slice + 1 : 0u;
        depths += t > f ? 1u : 0u;
    }
    if (total == 0) return 0;
    uint32_t t0 = 0;
    if (!claim_tasks(T, out, out_count, total, limit, cap, t0)) {
        if (!claim_tasks(T, out, out_count, depths, limit + slack, cap, t0)) return 0;
        slice = 0xffffffffu;  // compact: one task per non-empty depth
        total = depths;
    }
    for (uint32_t k = T.lane; k < total; k += G) {
        uint32_t acc = 0, f = 0, t = 0, c = 0;
        int j = start;
        for (; j <= dabort; ++j) {
            remainder_at(S, j, dabort, f, t);
            c = t > f ? (t - f - 1) / slice + 1 : 0u;
            if (k < acc + c) break;
            acc += c;
        }
        SplitTask task;
        task.pat = p;
        task.u = (uint16_t)u;
        task.depth = (uint8_t)j;
        task.pad = 0;
        task.v = v;
        task.lo = f + (k - acc) * slice;  // k - acc is 0 when compact
        task.hi = t - task.lo > slice ? task.lo + slice : t;
        task.group = group;
        for (int q = 0; q < kTaskMaxN; ++q) task.prefix[q] = q < j && q < N ? S.emb[P.order[q]] : 0u;
        if (TFSM_IN(14, t0 + k, cap) && TFSM_IN(48, task.hi, m2 + 1)) out[t0 + k] = task;
    }
    return total;
}

// Anchor positions per task when a search's remainder is split: split_slice, or, for a hub's first
// depth split before any step, an even share among hub_parts tasks.
__device__ __forceinline__ uint32_t slice_for(const SearchParams &prm, uint32_t steps, uint32_t first_len) {
    if (steps == 0 && prm.hub_parts > 1) {
        const uint32_t s = (first_len + prm.hub_parts - 1) / prm.hub_parts;
        return s > prm.split_slice ? s : prm.split_slice;
    }
    return prm.split_slice;
}

// Lane 0: v has no embedding as u (nor as any vertex automorphic to u).
template <int N>
__device__ __forceinline__ void fail_vertex(const Plan<N> &P, PatStatus &st, uint32_t *__restrict__ failed, int u,
                                            uint32_t v, uint32_t tau, bool exact) {
    uint32_t orb = P.orbit[u];
    while (orb) {
        const int k = __ffs(orb) - 1;
        orb &= orb - 1;
        const uint32_t xl = v - P.lstart[k];
        const uint32_t bit = 1u << (xl & 31);
        if (!TFSM_IN(10, (uint64_t)P.off[k] + (xl >> 5), P.words)) continue;
        const uint32_t old = atomicOr(failed + P.off[k] + (xl >> 5), bit);
        if (k == u && !(old & bit)) {
            const uint32_t c = atomicAdd(&st.fail_cnt[u], 1u) + 1;
            if (!exact && __ldcg(&st.dom_size[u]) < c + tau) atomicCAS(&st.state, kRunning, kInfrequent);
        }
    }
}

// Add every vertex of the embedding in S (and its automorphic images) to the found bitmaps.
template <int G, int N>
__device__ __forceinline__ void mark_found(const Team<G> &T, const Plan<N> &P, const State<N> &S, PatStatus &st,
                                           uint32_t *__restrict__ found, uint32_t tau, bool exact) {
    for (int q = (int)T.lane; q < P.n; q += G) {
        const uint32_t x = S.emb[q];
        uint32_t orb = P.orbit[q];
        while (orb) {
            const int k = __ffs(orb) - 1;
            orb &= orb - 1;
            const uint32_t xl = x - P.lstart[k];
            const uint32_t bit = 1u << (xl & 31);
            if (!TFSM_IN(9, (uint64_t)P.off[k] + (xl >> 5), P.words)) continue;
            const uint32_t old = atomicOr(found + P.off[k] + (xl >> 5), bit);
            if (!(old & bit)) {
                const uint32_t c = atomicAdd(&st.found_cnt[k], 1u) + 1;
                if (!exact && c == tau && ((P.repmask >> k) & 1u)) {
                    const uint32_t dm = atomicOr(&st.done_mask, 1u << k) | (1u << k);
                    if ((dm & P.repmask) == P.repmask) atomicCAS(&st.state, kRunning, kFrequent);
                }
            }
        }
    }
    T.sync();
}

// Team-uniform: lane 0 reads the shared flags and broadcasts the decision.
template <int G>
__device__ __forceinline__ bool pattern_stops(const Team<G> &T, const PatStatus &st, int u, bool exact) {
    int stop = 0;
    if (T.lane == 0) {
        stop = __ldcg(&st.state) != kRunning;
        if (!stop && !exact) stop = (__ldcg(&st.done_mask) >> u) & 1u;
    }
    return T.bcast(stop, 0) != 0;
}

}  // namespace

// One search pass.  Split tasks of round 0 go to `splits` (the first buffer).  Each team of G lanes
// claims its own items.  Outside the last pass, a search whose remainder finds no room is set aside
// (neither found nor failed), and a team starts no more searches once the first round's share of
// the buffer is full: the next pass, with larger budgets, takes up what is left.
// Instances: teams of 4 lanes for patterns of at most 5 vertices (a depth has at most 4 backward
// neighbours, one per lane in setup_depth), teams of 8 lanes for at most 8, whole warps for at most
// 16, and whole warps for at most 32 (these searches never split: split tasks hold 16-vertex
// prefixes).
template <int G, int N>
__global__ void __launch_bounds__(SearchBlock<G, N>::warps * 32, SearchBlock<G, N>::min_blocks)
    k_search(Graph g, const PatDesc *__restrict__ descs,
                                                              PatStatus *__restrict__ st,
                                                              const ItemGroup *__restrict__ igroups,
                                                              const ItemEntry *__restrict__ ientries, SearchParams prm,
                                                              uint32_t *__restrict__ counters,
                                                              const uint32_t *__restrict__ dom,
                                                              uint32_t *__restrict__ found,
                                                              uint32_t *__restrict__ failed,
                                                              SplitTask *__restrict__ splits,
                                                              SplitGroup *__restrict__ groups) {
    constexpr int kTeams = SearchBlock<G, N>::warps * 32 / G;
    constexpr bool kSplits = N <= kTaskMaxN;
    __shared__ Plan<N> plans[kTeams];
    __shared__ State<N> states[kTeams];
    __shared__ Tile<G> tiles[kTeams];
    const Team<G> T(threadIdx.x & 31);
    Plan<N> &P = plans[threadIdx.x / G];
    State<N> &S = states[threadIdx.x / G];
    Tile<G> &tile = tiles[threadIdx.x / G];
    if (T.lane == 0) P.key = 0xffffffffu;
    T.sync();
    const bool exact = prm.exact != 0;
    // without a budget or a hub span no search aborts, so no split task is ever written
    const uint32_t budget = kSplits && prm.split ? prm.step_budget : 0u;
    const uint32_t hub_span = kSplits && prm.split && prm.hub_parts > 1 ? prm.hub_span : 0u;
    for (;;) {
        uint32_t it = 0;
        if (T.lane == 0) it = atomicAdd(&counters[0], 1u);
        it = T.bcast(it, 0);
        if (it >= (prm.n_items << prm.parts_log2)) break;
        const SearchItem item = item_at(igroups, prm.n_groups, ientries, prm.chunk_words, it >> prm.parts_log2);
        const uint32_t pmask = part_mask(it & ((1u << prm.parts_log2) - 1), prm.parts_log2);
        const uint32_t p = item.pat;
        const int u = item.u;
        if (!TFSM_IN(12, p, prm.n_pats) || !TFSM_IN(20, u, N)) continue;
        if (!TFSM_IN(22, descs[p].n, N + 1)) continue;
        load_plan(T, P, descs[p], p, u, prm.words);
        PatStatus &ps = st[p];
        // this start vertex's hub-split span (the cost model may move it: PatDesc::hub_shift)
        const int shift = descs[p].hub_shift[u];
        uint32_t u_hub_span = hub_span;
        if (shift == kNoHubSplit) u_hub_span = 0u;
        else if (shift > 0) u_hub_span = hub_span << (shift < 8 ? shift : 8);
        else if (shift < 0) u_hub_span = hub_span >> (-shift < 8 ? -shift : 8);
        if (hub_span && shift != kNoHubSplit && u_hub_span == 0) u_hub_span = 1;
        unsigned long long n_search = 0, n_steps = 0, n_bytes = 0, max_steps = 0, n_isects = 0;
        bool stop = false, stopped = false;
        for (uint32_t word = item.word_lo; word < item.word_hi && !stop; ++word) {
            if (pattern_stops(T, ps, u, exact)) break;
            const uint32_t o = P.off[u] + word;
            if (!TFSM_IN(13, o, prm.words)) break;
            uint32_t cand = T.word(dom + o) & ~T.word(found + o) & ~T.word(failed + o) & pmask;
            while (cand) {
                const int b = __ffs(cand) - 1;
                cand &= cand - 1;
                if ((T.word(found + o) >> b) & 1u) continue;
                if (pattern_stops(T, ps, u, exact)) {
                    stop = true;
                    break;
                }
                if (budget && !prm.last) {
                    // the first split round's share of the buffer is full: this team starts no
                    // more searches in this pass; the next pass takes up what is left
                    int full = 0;
                    if (T.lane == 0) full = __ldcg(&counters[2]) >= prm.search_fill;
                    if (T.bcast(full, 0)) {
                        stop = stopped = true;
                        break;
                    }
                }
                const uint32_t v = P.lstart[u] + word * 32 + b;
                if (T.lane == 0) S.emb[u] = v;
                T.sync();
                uint32_t steps = 0, bytes = 12, isects = 0;  // + domain, found and failed words of v
                int adepth = 0;
                ++n_search;
                const Cancel cancel{found + o, 1u << b, &ps, u, exact};
                int r = dfs(T, g, P, S, tile, dom, found, failed, 1, false, 0, 0, budget, u_hub_span, prm.isect_ratio,
                            cancel, steps, adepth, bytes, isects);
                if (r == kAbort) {
                    // The unexplored remainder becomes tasks for the split rounds, grouped so that
                    // the last one to finish can decide v.
                    const uint32_t first_len = S.end[1] - S.pos[1];
                    uint32_t g0 = 0;
                    int okg = 0;
                    if (T.lane == 0)
                        okg = reserve(&counters[1], 1, prm.group_cap, g0) && TFSM_IN(15, g0, prm.group_cap) ? 1 : 0;
                    okg = T.bcast(okg, 0);
                    g0 = T.bcast(g0, 0);
                    uint32_t added = 0;
                    if (okg)
                        added = emit_remainder(T, P, S, p, u, v, 1, adepth, g0, slice_for(prm, steps, first_len),
                                               splits, &counters[2], prm.split_cap, prm.search_fill, prm.split_slack,
                                               g.m2);
                    if (T.lane == 0 && okg) {  // read only by the split rounds, which run after this kernel
                        groups[g0].pat = p;
                        groups[g0].u = (uint16_t)u;
                        groups[g0].v = v;
                        groups[g0].pending = added;
                        groups[g0].incomplete = 0;
                    }
                    if (added || !prm.last) {
                        if (!added && T.lane == 0) atomicAdd(&counters[kCntAbandoned], 1u);  // buffers full
                        n_steps += steps;
                        n_isects += isects;
                        n_bytes += T.sum(bytes);
                        continue;  // decided by the split rounds, or by the next pass
                    }
                    // buffers full, last pass: finish this search here without a budget
                    if (T.lane == 0) S.emb[u] = v;
                    T.sync();
                    r = dfs(T, g, P, S, tile, dom, found, failed, 1, false, 0, 0, 0, 0, prm.isect_ratio, cancel, steps,
                            adepth, bytes, isects);
                }
                n_steps += steps;
                n_isects += isects;
                max_steps = steps > max_steps ? steps : max_steps;
                n_bytes += T.sum(bytes);
                if (r == kFound) mark_found(T, P, S, ps, found, prm.tau, exact);
                else if (r == kFail && T.lane == 0) fail_vertex(P, ps, failed, u, v, prm.tau, exact);
                T.sync();
            }
        }
        if (T.lane == 0 && n_search) {
            atomicAdd(&ps.searches, n_search);
            atomicAdd(&ps.steps, n_steps);
            atomicAdd(&ps.isects, n_isects);
            atomicAdd(&ps.bytes, n_bytes);
            atomicMax(&ps.max_steps, max_steps);
            atomicAdd(&ps.steps_u[u], n_steps);
            atomicAdd(&ps.searches_u[u], (uint32_t)n_search);
        }
        if (stopped) {
            if (T.lane == 0) atomicAdd(&counters[kCntAbandoned], 1u);
            return;
        }
    }
}

// One split round: processes the tasks of round `round` (in `in`), searching each below its
// partial embedding; a task that exceeds `budget` (0: never, as in the last round) emits its own
// unexplored remainder into `out` for the next round, inside the same group.  Outside the last
// pass, a remainder without room is set aside (the group is marked incomplete, so v stays
// undecided for the next pass).
template <int G, int N>
__global__ void __launch_bounds__(SearchBlock<G, N>::warps * 32, SearchBlock<G, N>::min_blocks)
    k_split(Graph g, const PatDesc *__restrict__ descs,
                                                             PatStatus *__restrict__ st, SearchParams prm,
                                                             uint32_t *__restrict__ counters, int round,
                                                             uint32_t budget, const uint32_t *__restrict__ dom,
                                                             uint32_t *__restrict__ found,
                                                             uint32_t *__restrict__ failed,
                                                             const SplitTask *__restrict__ in,
                                                             SplitTask *__restrict__ out,
                                                             SplitGroup *__restrict__ groups) {
    static_assert(N <= kTaskMaxN, "split tasks hold prefixes of at most kTaskMaxN vertices");
    constexpr int kTeams = SearchBlock<G, N>::warps * 32 / G;
    __shared__ Plan<N> plans[kTeams];
    __shared__ State<N> states[kTeams];
    __shared__ Tile<G> tiles[kTeams];
    const Team<G> T(threadIdx.x & 31);
    Plan<N> &P = plans[threadIdx.x / G];
    State<N> &S = states[threadIdx.x / G];
    Tile<G> &tile = tiles[threadIdx.x / G];
    if (T.lane == 0) P.key = 0xffffffffu;
    T.sync();
    const bool exact = prm.exact != 0;
    const uint32_t n_tasks = min(counters[2 + round], prm.split_cap);
    for (;;) {
        uint32_t it = 0;
        if (T.lane == 0) it = atomicAdd(&counters[kClaimBase + round], 1u);
        it = T.bcast(it, 0);
        if (it >= n_tasks) break;
        const SplitTask &t = in[it];  // fields read one by one; the prefix stays in memory
        const uint32_t p = t.pat;
        if (p == kNullTask) continue;  // a slot of a claim that did not fit
        const int u = t.u;
        const int depth = t.depth;
        if (!TFSM_IN(16, p, prm.n_pats) || !TFSM_IN(17, t.group, prm.group_cap) || !TFSM_IN(21, u, N)) continue;
        if (!TFSM_IN(23, descs[p].n, N + 1)) continue;
        load_plan(T, P, descs[p], p, u, prm.words);
        PatStatus &ps = st[p];
        SplitGroup &grp = groups[t.group];
        const uint32_t xl = t.v - P.lstart[u];
        const uint32_t o = P.off[u] + (xl >> 5);
        const uint32_t bit = 1u << (xl & 31);
        if (!TFSM_IN(18, o, prm.words) || !TFSM_IN(44, depth, P.n) || !TFSM_IN(45, t.lo, (uint64_t)t.hi + 1) ||
            !TFSM_IN(47, t.hi, g.m2 + 1) || !TFSM_IN(46, depth, N))
            continue;
        bool searched = false;
        uint32_t added = 0;
        if (!pattern_stops(T, ps, u, exact) && !(T.word(found + o) & bit)) {
            for (int q = (int)T.lane; q < depth; q += G) S.emb[P.order[q]] = t.prefix[q];
            T.sync();
            uint32_t steps = 0, bytes = 12, isects = 0;
            int adepth = 0;
            const Cancel cancel{found + o, bit, &ps, u, exact};
            int r = dfs(T, g, P, S, tile, dom, found, failed, depth, true, t.lo, t.hi, budget, 0, prm.isect_ratio,
                        cancel, steps, adepth, bytes, isects);
            if (r == kAbort) {
                added = emit_remainder(T, P, S, p, u, t.v, depth, adepth, t.group, prm.split_slice, out,
                                       &counters[2 + round + 1], prm.split_cap, prm.split_cap - prm.split_slack,
                                       prm.split_slack, g.m2);
                if (!added && !prm.last) {  // no room: v stays undecided for the next pass
                    if (T.lane == 0) atomicAdd(&counters[kCntAbandoned], 1u);
                    r = kCancel;
                } else if (!added) {  // no room, last pass: finish the task here
                    r = dfs(T, g, P, S, tile, dom, found, failed, depth, true, t.lo, t.hi, 0, 0, prm.isect_ratio,
                            cancel, steps, adepth, bytes, isects);
                }
            }
            if (r == kFound) mark_found(T, P, S, ps, found, prm.tau, exact);
            const unsigned long long wb = T.sum(bytes);
            if (T.lane == 0) {
                atomicAdd(&ps.steps, (unsigned long long)steps);
                atomicAdd(&ps.isects, (unsigned long long)isects);
                atomicAdd(&ps.bytes, wb);
                atomicMax(&ps.max_steps, (unsigned long long)steps);
                atomicAdd(&ps.steps_u[u], (unsigned long long)steps);
            }
            searched = r != kCancel;
        }
        if (T.lane == 0) {
            if (!searched && !(__ldcg(found + o) & bit)) atomicOr(&grp.incomplete, 1u);
            if (added) atomicAdd(&grp.pending, added);  // before this task's own completion below
            __threadfence();
            const uint32_t left = atomicSub(&grp.pending, 1u) - 1;
            if (left == 0) {
                __threadfence();
                // every task of the search finished without an embedding: v fails as u
                if (!(__ldcg(found + o) & bit) && __ldcg(&grp.incomplete) == 0)
                    fail_vertex(P, ps, failed, u, t.v, prm.tau, exact);
            }
        }
        T.sync();
    }
}

// ------------------------------------------------------------------------------------------------
// Host-side launchers.
// ------------------------------------------------------------------------------------------------
bool read_bounds_check(unsigned long long rec[4]) {
#ifdef TFSM_BOUNDS_CHECK
    const cudaError_t e = cudaMemcpyFromSymbol(rec, g_check, sizeof(unsigned long long) * 4);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "tfsm checked build: cannot read the check record: %s\n", cudaGetErrorString(e));
        rec[0] = 1;
        rec[1] = rec[2] = rec[3] = ~0ull;
        return true;
    }
    std::fprintf(stderr, "tfsm checked build: check record count %llu site %llu index %llu bound %llu\n", rec[0],
                 rec[1], rec[2], rec[3]);
    return rec[0] != 0;
#else
    rec[0] = rec[1] = rec[2] = rec[3] = 0;
    return false;
#endif
}

static int g_num_sms = 0;

static int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

cudaError_t launch_domain_init(const Graph &g, const PatDesc *descs, PatStatus *st, const uint32_t *item_pu,
                               const uint64_t *prefix, uint32_t n_items, uint64_t total_words, uint32_t *dom,
                               uint32_t *found, uint32_t *failed, const SourceLevel *srcs, uint32_t n_srcs,
                               uint64_t chk_words, cudaStream_t s) {
    if (n_items == 0 || total_words == 0) return cudaSuccess;
    const uint64_t warps = total_words;
    uint64_t blocks = (warps * 32 + 255) / 256;
    const uint64_t cap = (uint64_t)num_sms() * 8 * 4;
    if (blocks > cap) blocks = cap;
    TFSM_LAUNCH(k_domain_init, (unsigned)blocks, 256, s, g, descs, st, item_pu, prefix, n_items, dom, found, failed,
                srcs, n_srcs, chk_words);
#ifdef TFSM_BOUNDS_CHECK
    if (cudaStreamSynchronize(s) != cudaSuccess) return cudaGetLastError();
#endif
    return cudaGetLastError();
}

cudaError_t launch_refine(const Graph &g, const PatDesc *descs, PatStatus *st, const uint32_t *item_pu,
                          const uint64_t *prefix, uint32_t n_items, uint64_t total_words, uint32_t *dom,
                          uint64_t chk_words, int round, uint32_t tau, bool exact, cudaStream_t s) {
    if (n_items == 0 || total_words == 0) return cudaSuccess;
    if (round < 0 || round >= 32) return cudaErrorInvalidValue;
    uint64_t blocks = (total_words * 32 + 255) / 256;
    const uint64_t cap = (uint64_t)num_sms() * 8 * 4;
    if (blocks > cap) blocks = cap;
    TFSM_LAUNCH(k_refine, (unsigned)blocks, 256, s, g, descs, st, item_pu, prefix, n_items, dom, chk_words, round,
                tau, exact ? 1 : 0);
#ifdef TFSM_BOUNDS_CHECK
    if (cudaStreamSynchronize(s) != cudaSuccess) return cudaGetLastError();
#endif
    return cudaGetLastError();
}

namespace {

template <int G, int N>
cudaError_t launch_search_t(const Graph &g, const PatDesc *descs, PatStatus *st, const ItemGroup *igroups,
                            const ItemEntry *ientries, const SearchParams &prm, uint32_t *counters,
                            const uint32_t *dom, uint32_t *found, uint32_t *failed, SplitTask *splits,
                            SplitGroup *groups, cudaStream_t s) {
    constexpr int kThreads = SearchBlock<G, N>::warps * 32;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<G, N>, kThreads, 0);
    if (per_sm <= 0) per_sm = 1;
    uint64_t blocks = (uint64_t)num_sms() * (uint64_t)per_sm;
    const uint64_t teams = (uint64_t)kThreads / G;
    const uint64_t need = (((uint64_t)prm.n_items << prm.parts_log2) + teams - 1) / teams;
    if (blocks > need) blocks = need;
    TFSM_LAUNCH((k_search<G, N>), (unsigned)blocks, kThreads, s, g, descs, st, igroups, ientries, prm, counters, dom,
                found, failed, splits, groups);
    return cudaGetLastError();
}

template <int G, int N>
cudaError_t launch_split_t(const Graph &g, const PatDesc *descs, PatStatus *st, const SearchParams &prm,
                           uint32_t *counters, int round, uint32_t budget, const uint32_t *dom, uint32_t *found,
                           uint32_t *failed, const SplitTask *in, SplitTask *out, SplitGroup *groups,
                           cudaStream_t s) {
    constexpr int kThreads = SearchBlock<G, N>::warps * 32;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_split<G, N>, kThreads, 0);
    if (per_sm <= 0) per_sm = 1;
    TFSM_LAUNCH((k_split<G, N>), (unsigned)(num_sms() * per_sm), kThreads, s, g, descs, st, prm, counters, round,
                budget, dom, found, failed, in, out, groups);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_search(const Graph &g, const PatDesc *descs, PatStatus *st, const ItemGroup *igroups,
                          const ItemEntry *ientries, const SearchParams &prm, uint32_t *counters, const uint32_t *dom,
                          uint32_t *found, uint32_t *failed, SplitTask *splits, SplitGroup *groups, cudaStream_t s) {
    if (prm.n_items == 0) return cudaSuccess;
    if (prm.n_groups == 0 || prm.chunk_words == 0 || !igroups || !ientries) return cudaErrorInvalidValue;
    if (prm.split && (!splits || !groups || prm.split_cap == 0 || prm.group_cap == 0 || prm.split_slice == 0))
        return cudaErrorInvalidValue;
    if (prm.max_n > (uint32_t)kMaxN || (prm.team_lanes == 8 && prm.max_n > 8) ||
        (prm.team_lanes == 4 && prm.max_n > 5))
        return cudaErrorInvalidValue;
    if (prm.split && prm.max_n > (uint32_t)kTaskMaxN) return cudaErrorInvalidValue;
    cudaError_t e;
    if (prm.team_lanes == 4)
        e = launch_search_t<4, 8>(g, descs, st, igroups, ientries, prm, counters, dom, found, failed, splits, groups,
                                  s);
    else if (prm.team_lanes == 8)
        e = launch_search_t<8, 8>(g, descs, st, igroups, ientries, prm, counters, dom, found, failed, splits, groups,
                                  s);
    else if (prm.team_lanes == 32 && prm.max_n <= (uint32_t)kTaskMaxN)
        e = launch_search_t<32, kTaskMaxN>(g, descs, st, igroups, ientries, prm, counters, dom, found, failed, splits,
                                           groups, s);
    else if (prm.team_lanes == 32)
        e = launch_search_t<32, kMaxN>(g, descs, st, igroups, ientries, prm, counters, dom, found, failed, splits,
                                       groups, s);
    else return cudaErrorInvalidValue;
#ifdef TFSM_BOUNDS_CHECK
    if (e == cudaSuccess && cudaStreamSynchronize(s) != cudaSuccess) {
        std::fprintf(stderr, "tfsm checked build: fault in k_search\n");
        return cudaGetLastError();
    }
#endif
    return e;
}

uint32_t resident_search_warps() {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<32, kTaskMaxN>, kSearchWarps * 32, 0);
    if (per_sm <= 0) per_sm = 1;
    return (uint32_t)(num_sms() * per_sm * kSearchWarps);
}

cudaError_t launch_split_round(const Graph &g, const PatDesc *descs, PatStatus *st, const SearchParams &prm,
                               uint32_t *counters, int round, uint32_t budget, const uint32_t *dom, uint32_t *found,
                               uint32_t *failed, SplitTask *splits, SplitGroup *groups, cudaStream_t s) {
    if (round < 0 || round >= kMaxRounds) return cudaErrorInvalidValue;
    const SplitTask *in = splits + (size_t)(round % 2) * prm.split_cap;
    SplitTask *out = splits + (size_t)((round + 1) % 2) * prm.split_cap;
    if (round + 1 == kMaxRounds) budget = 0;  // the last possible round completes every task
    if (prm.max_n > (uint32_t)kTaskMaxN || (prm.team_lanes == 8 && prm.max_n > 8) ||
        (prm.team_lanes == 4 && prm.max_n > 5))
        return cudaErrorInvalidValue;
    cudaError_t e;
    if (prm.team_lanes == 4)
        e = launch_split_t<4, 8>(g, descs, st, prm, counters, round, budget, dom, found, failed, in, out, groups, s);
    else if (prm.team_lanes == 8)
        e = launch_split_t<8, 8>(g, descs, st, prm, counters, round, budget, dom, found, failed, in, out, groups, s);
    else if (prm.team_lanes == 32)
        e = launch_split_t<32, kTaskMaxN>(g, descs, st, prm, counters, round, budget, dom, found, failed, in, out,
                                          groups, s);
    else return cudaErrorInvalidValue;
#ifdef TFSM_BOUNDS_CHECK
    if (e == cudaSuccess && cudaStreamSynchronize(s) != cudaSuccess) {
        std::fprintf(stderr, "tfsm checked build: fault in k_split\n");
        return cudaGetLastError();
    }
#endif
    return e;
}

}  // namespace dev
}  // namespace tfsm
