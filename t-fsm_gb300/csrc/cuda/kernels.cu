// CUDA kernels of the MNI support evaluation (sm_103a).  Integer gather work: no tensor cores.
//
//   k_domain_init  LDF + NLF candidate filter (parallel/gmatch.h:301-415) writing one bitmap
//                  per pattern vertex over its label's id range; children start from the
//                  parent's final domain (candidates minus proven non-candidates).
//   k_refine       one arc-consistency pass over every pattern edge, incl. edge labels
//                  (pruneCandidates, parallel/gmatch.h:600-658, pull direction).  Iterated to a
//                  fixpoint for distinct-label trees, whose domains are then the exact MNI
//                  domains (parallel/comper.h:1619-1653).
//   k_search       persistent backtracking: a team of lanes (a warp, or a quarter of one) per
//                  (pattern vertex u, candidate v) search looks for one embedding with u -> v
//                  (LFTJ, serial/gmatch.h:906-987).  Local candidates at each depth are the label
//                  sub-range of the smallest backward neighbour's adjacency, checked G at a time
//                  (one per lane) against the domain bitmap, injectivity and every other backward
//                  neighbour; the survivors are a ballot mask.  Found embeddings add all their
//                  vertices (and automorphic images) to the MNI domains; early exit per vertex at
//                  tau and per pattern when tau can no longer be reached
//                  (parallel/comper.h:288-297).  Long searches share out their unexplored
//                  branches as tasks on a device ring that any team takes (work sharing for hub
//                  vertices, parallel/comper.h:640-749, 865-973); the last unit of a split search
//                  to finish decides its failure (parallel/taskprogmap.h:10-85).
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
        const uint32_t p = pu >> 8, u = pu & 0xff;
        const PatDesc &D = descs[p];
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
            const uint32_t *lo_x = g.lab_off + (size_t)x * g.lab_stride;
            for (int k = 0; k < nn && pass; ++k) {
                const int L = D.nlf_lab[u][k];
                pass = (__ldg(lo_x + L + 1) - __ldg(lo_x + L)) >= (uint32_t)D.nlf_cnt[u][k];
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
        const uint32_t p = pu >> 8, u = pu & 0xff;
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
                const uint32_t *lo_v = g.lab_off + (size_t)v * g.lab_stride;
                uint32_t nb = D.adj[u];
                while (nb && keep_lane && !hard_lane) {
                    const int w = __ffs(nb) - 1;
                    nb &= nb - 1;
                    const uint32_t lo = __ldg(lo_v + D.lab[w]), hi = __ldg(lo_v + D.lab[w] + 1);
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
            const uint32_t *lo_v = g.lab_off + (size_t)v * g.lab_stride;
            uint32_t nb = D.adj[u];
            bool ok = true;
            while (nb && ok) {
                const int w = __ffs(nb) - 1;
                nb &= nb - 1;
                const uint32_t ls = D.lstart[w];
                const uint32_t lo = __ldg(lo_v + D.lab[w]), hi = __ldg(lo_v + D.lab[w] + 1);
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
// K5 / K6: persistent search with device-side work sharing.
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

// Largest pattern a team of G lanes searches (its per-depth state is sized for it).
template <int G>
struct TeamMaxN {
    static constexpr int value = G == 32 ? kMaxN : 8;
};

// Acquire load / release store at device scope: the hand-over of a ring slot between the team
// that writes a task and the team that reads it.
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
#ifdef TFSM_SIMT_EMULATION
    return __atomic_load_n(p, __ATOMIC_ACQUIRE);
#else
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
#endif
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
#ifdef TFSM_SIMT_EMULATION
    __atomic_store_n(p, v, __ATOMIC_RELEASE);
#else
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
#endif
}

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
    uint32_t blo[N][N];   // [depth][backward neighbour b]: label range of order[depth]'s
    uint32_t bhi[N][N];   //   label inside emb[b]'s adjacency
};

enum : int { kFail = 0, kFound = 1, kCancel = 3, kAbandon = 4 };

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
// A waiting team sleeps between looks at the ring (doubling from 256 ns up to 16 us) and stops
// waiting after this many looks (about two seconds): the teams still at work finish every unit
// they hold and every task they shared, so leaving early only costs balance, never a result.
constexpr uint32_t kMaxWaits = 1u << 17;
constexpr uint32_t kNapMin = 256, kNapMax = 16384;

// Try candidates already known to be in w's MNI domain first.  Measured slower on the benchmark
// graphs (the extra ballot and found-word loads cost more than the reordering saves): off.
constexpr bool kFoundFirst = false;

// The search's share of the launch: which (pattern, vertex, candidate) it decides and the group
// it belongs to once it has shared work (kNoGroup before).
struct Donor {
    uint32_t p;
    int u;
    uint32_t v;
    uint32_t group;
};

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
        P.bn[i] = D.bn[u][i];
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
// handles the k-th backward neighbour; a team minimum picks the winner.
template <int G, int N>
__device__ __forceinline__ void setup_depth(const Team<G> &T, const Graph &g, const Plan<N> &P, State<N> &S, int d,
                                            uint32_t &bytes) {
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
            const uint32_t *lo_y = g.lab_off + (size_t)y * g.lab_stride + P.lab[w];
            lo = __ldg(lo_y);
            hi = __ldg(lo_y + 1);
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
    lo = T.bcast(lo, win);
    hi = T.bcast(hi, win);
    b = T.bcast(b, win);
    if (T.lane == 0) {
        S.pos[d] = lo;
        S.end[d] = hi;
        S.mask[d] = 0;
        S.rest[d] = 0;
        S.anchor[d] = (uint8_t)b;
    }
    T.sync();
}

// Is adjacency position `idx` of the depth-d anchor a valid extension?  (one lane, one position)
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
    uint32_t others = P.bn[d] & ~(1u << a);
    while (others) {
        const int b = __ffs(others) - 1;
        others &= others - 1;
        const uint32_t re = S.bhi[d][b];
        uint32_t pos = lower_bound_cnt(g.col, S.blo[d][b], re, x, bytes, g.m2);
        bool hit = false;
        const uint8_t want = P.el[w][b];
        while (pos < re && TFSM_IN(6, pos, g.m2) && __ldg(g.col + pos) == x) {  // parallel edges: any with the label
            bytes += 5;
            if (__ldg(g.elab + pos) == want) {
                hit = true;
                break;
            }
            ++pos;
        }
        if (!hit) return false;
    }
    return true;
}

// Unexplored anchor positions left at depth j of a search whose deepest open depth is `dcur`:
// the not-yet-taken survivors of j's current chunk, then [pos[j], end[j]).  Survivors of a chunk
// are taken lowest position first, so everything below the lowest pending one is explored.
template <int N>
__device__ __forceinline__ void remainder_at(const State<N> &S, int j, int dcur, uint32_t &from, uint32_t &to) {
    to = S.end[j];
    const uint32_t m = S.mask[j] | S.rest[j];
    from = (j == dcur || m == 0) ? S.pos[j] : S.base[j] + (uint32_t)(__ffs(m) - 1);
    if (from > to) from = to;
}

// Lane 0: a free group slot for v's split search (CAS 0 -> 1, the donor being its first unit), or
// kNoGroup when none is found within a few tries.
__device__ __forceinline__ uint32_t claim_group(const SearchParams &prm, uint32_t *cnt) {
    for (int a = 0; a < 16; ++a) {
        const uint32_t g = atomicAdd(&cnt[kCntGroupCursor * kCntStride], 1u) & (prm.gcap - 1);
        if (atomicCAS(&prm.groups[g], 0u, 1u) == 0u) {
            atomicAdd(&cnt[kCntGroups * kCntStride], 1u);
            return g;
        }
    }
    return kNoGroup;
}

// Team-uniform: reserves k consecutive ring positions (k <= G); returns the first, or ~0u when the
// ring has no k free slots after them (or the claim keeps losing to other producers).
template <int G>
__device__ __forceinline__ uint32_t reserve_slots(const Team<G> &T, const SearchParams &prm, uint32_t k) {
    const uint32_t m = prm.qcap - 1;
    for (int a = 0; a < 8; ++a) {
        uint32_t t = 0;
        if (T.lane == 0) t = __ldcg(&prm.qctl[kQctlTail]);
        t = T.bcast(t, 0);
        int dif = 0;
        if (T.lane < k) dif = (int)(ld_acquire(&prm.cells[(t + T.lane) & m].seq) - (t + T.lane));
        if (T.any(dif < 0)) return ~0u;  // a slot still holds a task of the previous lap: full
        if (T.any(dif > 0)) continue;    // another producer took these positions first
        int won = 0;
        if (T.lane == 0) won = atomicCAS(&prm.qctl[kQctlTail], t, t + k) == t;
        if (T.bcast(won, 0)) return t;
    }
    return ~0u;
}

// Team-uniform: shares out the unexplored remainder of the shallowest open depth j (start <= j <=
// dcur) as `demand` parts at most (at most G), each a task of the same group.  The current depth
// keeps its first part; a shallower depth (whose pending branches lie above the search's current
// path) is given away whole.  Returns true when tasks were queued; the local state then no longer
// covers the donated positions.
template <int G, int N>
__device__ bool donate(const Team<G> &T, const Plan<N> &P, State<N> &S, const SearchParams &prm, uint32_t *cnt,
                       Donor &dn, int start, int dcur, uint32_t demand) {
    int j = -1;
    uint32_t from = 0, to = 0;
    for (int q = start; q <= dcur; ++q) {
        uint32_t f, t;
        remainder_at(S, q, dcur, f, t);
        const uint32_t least = q == dcur ? prm.split_slice + 1 : 1;  // current depth: worth a part
        if (t > f && t - f >= least) {
            j = q;
            from = f;
            to = t;
            break;
        }
    }
    if (j < 0) return false;
    const uint32_t R = to - from;
    const uint32_t keep = j == dcur ? 1u : 0u;
    uint32_t k = demand < (uint32_t)G ? demand : (uint32_t)G;
    if (keep) {
        const uint32_t fit = R / prm.split_slice;  // parts of at least split_slice positions, one kept
        k = fit > 1 && k > fit - 1 ? fit - 1 : (fit > 1 ? k : 0u);
    } else {
        k = k < R ? k : R;
    }
    if (k == 0) return false;
    // R positions in k + keep parts, the first `rem` of them one longer: part q is
    // [from + q * base + min(q, rem), from + (q + 1) * base + min(q + 1, rem)), never empty
    const uint32_t parts = k + keep, base = R / parts, rem = R % parts;
    uint32_t ok = 1;
    if (T.lane == 0 && dn.group == kNoGroup) {
        dn.group = claim_group(prm, cnt);
        ok = dn.group != kNoGroup;
    }
    dn.group = T.bcast(dn.group, 0);
    if (!T.bcast(ok, 0)) {
        if (T.lane == 0) atomicAdd(&cnt[kCntRefused * kCntStride], 1u);
        return false;
    }
    const uint32_t t0 = reserve_slots(T, prm, k);
    if (t0 == ~0u) {
        if (T.lane == 0) atomicAdd(&cnt[kCntRefused * kCntStride], 1u);
        return false;
    }
    if (T.lane == 0) {
        // the units count before any of them can be taken (and finish)
        atomicAdd(&prm.groups[dn.group], k);
        atomicAdd(&cnt[kCntWork * kCntStride], k);
        atomicAdd(&cnt[kCntTasks * kCntStride], k);
        atomicMax(&cnt[kCntQueueMax * kCntStride], t0 + k - __ldcg(&prm.qctl[kQctlHead]));
    }
    const uint32_t cut = from + keep * base + (keep < rem ? keep : rem);
    if (T.lane < k) {
        const uint32_t q = T.lane + keep;
        const uint32_t lo = from + q * base + (q < rem ? q : rem);
        const uint32_t hi = from + (q + 1) * base + (q + 1 < rem ? q + 1 : rem);
        QueueCell &c = prm.cells[(t0 + T.lane) & (prm.qcap - 1)];
        SplitTask &task = c.task;
        task.pat = dn.p;
        task.u = (uint16_t)dn.u;
        task.depth = (uint8_t)j;
        task.pad = 0;
        task.v = dn.v;
        task.lo = lo;
        task.hi = hi;
        task.group = dn.group;
        for (int q2 = 0; q2 < kMaxN; ++q2) task.prefix[q2] = q2 < j && q2 < N ? S.emb[P.order[q2]] : 0u;
        __threadfence();
        st_release(&c.seq, t0 + T.lane + 1);
    }
    T.sync();
    if (T.lane == 0) {
        // the donated positions leave this search: depth j ends at `cut`, and survivors of its
        // current chunk at or past `cut` are dropped
        S.end[j] = cut;
        if (j != dcur) {
            const uint32_t b0 = S.base[j];
            const uint32_t keep_bits = cut <= b0 ? 0u : (cut - b0 >= 32 ? 0xffffffffu : (1u << (cut - b0)) - 1u);
            S.mask[j] &= keep_bits;
            S.rest[j] &= keep_bits;
        }
    }
    T.sync();
    return true;
}

// Depth-first search for one embedding that extends the partial embedding of depths < start
// (S.emb[order[0..start-1]]).  With `slice`, depth `start` scans only anchor positions [lo, hi).
// The search never backtracks above `start`.  Returns kCancel when `cancel` says the search no
// longer matters, kAbandon when it reaches the pass's step budget (it is retried from the start
// by the next pass, with a larger budget).  In the last pass (no budget) the search looks every
// kCheckEvery chunk steps at the teams waiting for work and may share out part of its remainder
// (donate); a first depth longer than hub_span is shared out at once.  A chunk is G consecutive
// anchor positions.
template <int G, int N>
__device__ __forceinline__ int dfs(const Team<G> &T, const Graph &g, const Plan<N> &P, State<N> &S,
                                   const uint32_t *__restrict__ dom, const uint32_t *found, const uint32_t *failed,
                                   int start, bool slice, uint32_t lo, uint32_t hi, const Cancel &cancel,
                                   const SearchParams &prm, uint32_t *cnt, Donor &dn, uint32_t &steps,
                                   uint32_t &bytes, uint32_t &isects) {
    const int n = P.n;
    setup_depth(T, g, P, S, start, bytes);
    if (slice) {
        if (T.lane == 0) {
            S.pos[start] = lo;
            S.end[start] = hi;
        }
        T.sync();
    }
    const bool share = prm.split && prm.budget == 0;
    if (share && prm.hub_parts > 1 && !slice && S.end[start] - S.pos[start] > prm.hub_span) {
        int room = 0;
        if (T.lane == 0) room = __ldcg(&prm.qctl[kQctlTail]) - __ldcg(&prm.qctl[kQctlHead]) < prm.soft_cap;
        if (T.bcast(room, 0)) donate(T, P, S, prm, cnt, dn, start, start, prm.hub_parts - 1);
    }
    // look at cancellation and demand every kCheckEvery chunk steps, or every share_steps steps
    // when that is smaller (a test setting that makes short searches share work too)
    const uint32_t every = share && prm.share_steps && prm.share_steps < kCheckEvery ? prm.share_steps : kCheckEvery;
    uint32_t checked = 0;
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
            if (prm.budget && steps >= prm.budget) return kAbandon;
            if (steps != checked && steps % every == 0) {
                checked = steps;
                int c = 0;
                uint32_t demand = 0;
                if (T.lane == 0) {
                    c = (__ldcg(cancel.found_word) & cancel.bit) || __ldcg(&cancel.ps->state) != kRunning ||
                        (!cancel.exact && ((__ldcg(&cancel.ps->done_mask) >> cancel.u) & 1u));
                    if (!c && share) {
                        const uint32_t idle = __ldcg(&cnt[kCntIdle * kCntStride]);
                        const uint32_t qd = __ldcg(&prm.qctl[kQctlTail]) - __ldcg(&prm.qctl[kQctlHead]);
                        demand = idle > qd ? idle - qd : 0u;
                        if (!demand && prm.share_steps && steps >= prm.share_steps && qd < prm.soft_cap) demand = 1;
                    }
                }
                if (T.bcast(c, 0)) return kCancel;
                demand = T.bcast(demand, 0);
                if (demand && donate(T, P, S, prm, cnt, dn, start, d, demand)) continue;  // re-read the state
            }
            const uint32_t idx = pos + T.lane;
            uint32_t x = 0;
            bool known = false;
            const bool ok = idx < end && check_candidate(g, P, S, dom, found, failed, d, idx, x, known, bytes);
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
        setup_depth(T, g, P, S, d, bytes);
    }
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

// End of one unit of a search (the search itself, or one of its tasks), after mark_found when it
// found an embedding.  Without a group the unit is the whole search: a failure is final.  In a
// group, the unit that finishes last decides: v fails when no unit found an embedding and none
// stopped without an answer.
template <int G, int N>
__device__ __forceinline__ void finish_unit(const Team<G> &T, const Plan<N> &P, const SearchParams &prm,
                                            PatStatus &st, uint32_t *__restrict__ failed, const uint32_t *found,
                                            const Donor &dn, int r, uint32_t fo, uint32_t fbit, bool exact) {
    if (T.lane == 0) {
        if (dn.group == kNoGroup) {
            if (r == kFail) fail_vertex(P, st, failed, dn.u, dn.v, prm.tau, exact);
        } else {
            uint32_t *gw = &prm.groups[dn.group];
            if ((r == kCancel || r == kAbandon) && !(__ldcg(found + fo) & fbit)) atomicOr(gw, kGroupIncomplete);
            __threadfence();  // this unit's found / incomplete marks before its completion
            const uint32_t old = atomicSub(gw, 1u);
            if ((old & ~kGroupIncomplete) == 1u) {
                __threadfence();
                atomicExch(gw, 0u);  // the slot is free again
                if (!(old & kGroupIncomplete) && !(__ldcg(found + fo) & fbit))
                    fail_vertex(P, st, failed, dn.u, dn.v, prm.tau, exact);
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

// Team-uniform: takes the oldest task off the ring into `t` (fields the team needs), or false
// when the ring looks empty.
template <int G>
__device__ __forceinline__ bool pop_task(const Team<G> &T, const SearchParams &prm, SplitTask &t) {
    const uint32_t m = prm.qcap - 1;
    uint32_t pos = 0;
    int got = 0;
    if (T.lane == 0) {
        for (int a = 0; a < 16; ++a) {
            pos = __ldcg(&prm.qctl[kQctlHead]);
            const int dif = (int)(ld_acquire(&prm.cells[pos & m].seq) - (pos + 1));
            if (dif < 0) break;  // empty (or its producer has not finished writing it)
            if (dif > 0) continue;
            if (atomicCAS(&prm.qctl[kQctlHead], pos, pos + 1) == pos) {
                got = 1;
                break;
            }
        }
    }
    if (!T.bcast(got, 0)) return false;
    pos = T.bcast(pos, 0);
    QueueCell &c = prm.cells[pos & m];
    (void)ld_acquire(&c.seq);  // every lane synchronises with the producer before reading
    t.pat = __ldcg(&c.task.pat);
    const uint32_t w1 = __ldcg(reinterpret_cast<const uint32_t *>(&c.task.u));
    t.u = (uint16_t)(w1 & 0xffffu);
    t.depth = (uint8_t)((w1 >> 16) & 0xffu);
    t.v = __ldcg(&c.task.v);
    t.lo = __ldcg(&c.task.lo);
    t.hi = __ldcg(&c.task.hi);
    t.group = __ldcg(&c.task.group);
    // lane q % G keeps prefix[q] (a team of G lanes searches patterns of at most 2G vertices)
    t.prefix[0] = T.lane < kMaxN ? __ldcg(&c.task.prefix[T.lane]) : 0u;
    t.prefix[1] = T.lane + G < kMaxN ? __ldcg(&c.task.prefix[T.lane + G]) : 0u;
    __threadfence();
    T.sync();
    if (T.lane == 0) st_release(&c.seq, pos + prm.qcap);  // the slot goes to the next lap
    return true;
}

}  // namespace

// The search launch.  Each team of G lanes takes, in this order: a task another team shared (it
// completes a search already under way), the next work item (a run of bitmap words of one
// representative's domain: one search per still-undecided candidate), or, when both are gone,
// waits for a task while any unit of work is still outstanding.  Counters: kCnt* in
// dev_common.cuh, zero on entry.
template <int G>
__global__ void __launch_bounds__(kSearchWarps * 32) k_search(Graph g, const PatDesc *__restrict__ descs,
                                                              PatStatus *__restrict__ st,
                                                              const SearchItem *__restrict__ items, SearchParams prm,
                                                              uint32_t *__restrict__ cnt,
                                                              const uint32_t *__restrict__ dom,
                                                              uint32_t *__restrict__ found,
                                                              uint32_t *__restrict__ failed) {
    constexpr int N = TeamMaxN<G>::value;
    constexpr int kTeams = kSearchWarps * 32 / G;
    __shared__ Plan<N> plans[kTeams];
    __shared__ State<N> states[kTeams];
    // a later pass whose predecessor set no search aside has nothing to do (uniform per block)
    if (prm.prev && __ldcg(&prm.prev[kCntAbandoned * kCntStride]) == 0u) return;
    const Team<G> T(threadIdx.x & 31);
    Plan<N> &P = plans[threadIdx.x / G];
    State<N> &S = states[threadIdx.x / G];
    if (T.lane == 0) P.key = 0xffffffffu;
    T.sync();
    const bool exact = prm.exact != 0;
    const bool share = prm.split && prm.budget == 0;  // only the last pass shares work
    const uint32_t n_claims = prm.n_items << prm.parts_log2;
    bool items_left = true, idle = false;
    uint32_t waits = 0, nap = kNapMin;
    for (;;) {
        // ---- a shared task ----
        SplitTask t;
        if (share && pop_task(T, prm, t)) {
            if (idle && T.lane == 0) atomicSub(&cnt[kCntIdle * kCntStride], 1u);
            idle = false;
            waits = 0;
            nap = kNapMin;
            const uint32_t p = t.pat;
            const int u = t.u, depth = t.depth;
            Donor dn{p, u, t.v, t.group};
            // a task with fields out of range would be an engine fault: counted, never dereferenced
            const bool sane = p < prm.n_pats && t.group < prm.gcap && u < N && depth < N && t.lo <= t.hi &&
                              t.hi <= g.m2;
            if (!sane && T.lane == 0) atomicAdd(&cnt[kCntBadTask * kCntStride], 1u);
            if (sane && TFSM_IN(16, p, prm.n_pats) && TFSM_IN(17, t.group, prm.gcap) && TFSM_IN(21, u, N) &&
                TFSM_IN(23, descs[p].n, N + 1)) {
                load_plan(T, P, descs[p], p, u, prm.words);
                PatStatus &ps = st[p];
                const uint32_t xl = t.v - P.lstart[u];
                const uint32_t o = P.off[u] + (xl >> 5);
                const uint32_t bit = 1u << (xl & 31);
                int r = kCancel;
                if (TFSM_IN(18, o, prm.words) && TFSM_IN(44, depth, P.n) && TFSM_IN(45, t.lo, (uint64_t)t.hi + 1) &&
                    TFSM_IN(47, t.hi, g.m2 + 1) && TFSM_IN(46, depth, N)) {
                    if (!pattern_stops(T, ps, u, exact) && !(T.word(found + o) & bit)) {
                        if ((int)T.lane < depth) S.emb[P.order[T.lane]] = t.prefix[0];
                        if ((int)(T.lane + G) < depth) S.emb[P.order[T.lane + G]] = t.prefix[1];
                        T.sync();
                        uint32_t steps = 0, bytes = 12, isects = 0;
                        const Cancel cancel{found + o, bit, &ps, u, exact};
                        r = dfs(T, g, P, S, dom, found, failed, depth, true, t.lo, t.hi, cancel, prm, cnt, dn, steps,
                                bytes, isects);
                        if (r == kFound) mark_found(T, P, S, ps, found, prm.tau, exact);
                        const unsigned long long wb = T.sum(bytes);
                        if (T.lane == 0) {
                            atomicAdd(&ps.steps, (unsigned long long)steps);
                            atomicAdd(&ps.isects, (unsigned long long)isects);
                            atomicAdd(&ps.bytes, wb);
                            atomicMax(&ps.max_steps, (unsigned long long)steps);
                            atomicAdd(&ps.steps_u[u], (unsigned long long)steps);
                        }
                    }
                    finish_unit(T, P, prm, ps, failed, found, dn, r, o, bit, exact);
                }
            }
            if (T.lane == 0) atomicSub(&cnt[kCntWork * kCntStride], 1u);
            T.sync();
            continue;
        }
        // ---- the next work item ----
        if (items_left) {
            uint32_t it = 0;
            if (T.lane == 0) {
                atomicAdd(&cnt[kCntWork * kCntStride], 1u);  // before the claim: no team sees the launch idle meanwhile
                it = atomicAdd(&cnt[kCntItem * kCntStride], 1u);
                if (it >= n_claims) atomicSub(&cnt[kCntWork * kCntStride], 1u);
            }
            it = T.bcast(it, 0);
            if (it >= n_claims) {
                items_left = false;
                continue;
            }
            const SearchItem item = items[it >> prm.parts_log2];
            const uint32_t pmask = part_mask(it & ((1u << prm.parts_log2) - 1), prm.parts_log2);
            const uint32_t p = item.pat;
            const int u = item.u;
            if (TFSM_IN(12, p, prm.n_pats) && TFSM_IN(20, u, N) && TFSM_IN(22, descs[p].n, N + 1)) {
                load_plan(T, P, descs[p], p, u, prm.words);
                PatStatus &ps = st[p];
                unsigned long long n_search = 0, n_steps = 0, n_bytes = 0, max_steps = 0, n_isects = 0;
                uint32_t n_abandoned = 0;
                bool stop = false;
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
                        const uint32_t v = P.lstart[u] + word * 32 + b;
                        if (T.lane == 0) S.emb[u] = v;
                        T.sync();
                        uint32_t steps = 0, bytes = 12, isects = 0;  // + domain, found and failed words of v
                        ++n_search;
                        Donor dn{p, u, v, kNoGroup};
                        const Cancel cancel{found + o, 1u << b, &ps, u, exact};
                        const int r = dfs(T, g, P, S, dom, found, failed, 1, false, 0, 0, cancel, prm, cnt, dn, steps,
                                          bytes, isects);
                        n_steps += steps;
                        n_isects += isects;
                        max_steps = steps > max_steps ? steps : max_steps;
                        n_bytes += T.sum(bytes);
                        if (r == kFound) mark_found(T, P, S, ps, found, prm.tau, exact);
                        n_abandoned += r == kAbandon ? 1u : 0u;
                        finish_unit(T, P, prm, ps, failed, found, dn, r, o, 1u << b, exact);
                    }
                }
                if (T.lane == 0 && n_abandoned) atomicAdd(&cnt[kCntAbandoned * kCntStride], n_abandoned);
                if (T.lane == 0 && n_search) {
                    atomicAdd(&ps.searches, n_search);
                    atomicAdd(&ps.steps, n_steps);
                    atomicAdd(&ps.isects, n_isects);
                    atomicAdd(&ps.bytes, n_bytes);
                    atomicMax(&ps.max_steps, max_steps);
                    atomicAdd(&ps.steps_u[u], n_steps);
                    atomicAdd(&ps.searches_u[u], (uint32_t)n_search);
                }
            }
            if (T.lane == 0) atomicSub(&cnt[kCntWork * kCntStride], 1u);
            T.sync();
            continue;
        }
        // ---- nothing to take: done when no unit is outstanding, else wait for a shared task (at
        // most max_idle teams wait; the others end) ----
        if (!share) break;
        int done = 0;
        if (T.lane == 0) done = __ldcg(&cnt[kCntWork * kCntStride]) == 0u;
        if (T.bcast(done, 0)) break;
        if (!idle) {
            int over = 0;
            if (T.lane == 0 && atomicAdd(&cnt[kCntIdle * kCntStride], 1u) >= prm.max_idle) {
                atomicSub(&cnt[kCntIdle * kCntStride], 1u);
                over = 1;
            }
            if (T.bcast(over, 0)) break;
        }
        idle = true;
        if (++waits > kMaxWaits) {
            if (T.lane == 0) atomicAdd(&cnt[kCntWaitExpired * kCntStride], 1u);
            break;
        }
#ifdef TFSM_SIMT_EMULATION
        tfsm_emu_nap(nap);
#else
        __nanosleep(nap);
#endif
        nap = nap < kNapMax ? 2 * nap : kNapMax;
    }
    if (idle && T.lane == 0) atomicSub(&cnt[kCntIdle * kCntStride], 1u);
}

// Sets every ring slot free for its first lap and both positions to zero (once per engine; the
// ring is empty again after every launch).
__global__ void k_queue_init(QueueCell *cells, uint32_t qcap, uint32_t *qctl, uint32_t *groups, uint32_t gcap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = i; k < qcap; k += stride) cells[k].seq = k;
    for (uint32_t k = i; k < gcap; k += stride) groups[k] = 0;
    if (i == 0) qctl[kQctlHead] = qctl[kQctlTail] = 0;
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

cudaError_t launch_queue_init(QueueCell *cells, uint32_t qcap, uint32_t *qctl, uint32_t *groups, uint32_t gcap,
                              cudaStream_t s) {
    if (qcap == 0 || (qcap & (qcap - 1)) || gcap == 0 || (gcap & (gcap - 1))) return cudaErrorInvalidValue;
    const uint32_t n = qcap > gcap ? qcap : gcap;
    uint32_t blocks = (n + 255) / 256;
    const uint32_t cap = (uint32_t)num_sms() * 4;
    if (blocks > cap) blocks = cap;
    TFSM_LAUNCH(k_queue_init, blocks, 256, s, cells, qcap, qctl, groups, gcap);
    return cudaGetLastError();
}

namespace {

template <int G>
cudaError_t launch_search_t(const Graph &g, const PatDesc *descs, PatStatus *st, const SearchItem *items,
                            const SearchParams &prm, uint32_t *counters, const uint32_t *dom, uint32_t *found,
                            uint32_t *failed, cudaStream_t s) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<G>, kSearchWarps * 32, 0);
    if (per_sm <= 0) per_sm = 1;
    // persistent: at most one block per resident slot (a waiting team must not hold back a block
    // that has not started); without sharing, no more teams than claims
    uint64_t blocks = (uint64_t)num_sms() * (uint64_t)per_sm;
    if (!prm.split) {
        const uint64_t teams = (uint64_t)kSearchWarps * 32 / G;
        const uint64_t need = (((uint64_t)prm.n_items << prm.parts_log2) + teams - 1) / teams;
        if (blocks > need) blocks = need;
    }
    TFSM_LAUNCH(k_search<G>, (unsigned)blocks, kSearchWarps * 32, s, g, descs, st, items, prm, counters, dom, found,
                failed);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_search(const Graph &g, const PatDesc *descs, PatStatus *st, const SearchItem *items,
                          const SearchParams &prm, uint32_t *counters, const uint32_t *dom, uint32_t *found,
                          uint32_t *failed, cudaStream_t s) {
    if (prm.n_items == 0) return cudaSuccess;
    if (prm.split && (!prm.cells || !prm.qctl || !prm.groups || prm.qcap == 0 || (prm.qcap & (prm.qcap - 1)) ||
                      prm.gcap == 0 || (prm.gcap & (prm.gcap - 1)) || prm.split_slice == 0))
        return cudaErrorInvalidValue;
    cudaError_t e;
    if (prm.team_lanes == 8) e = launch_search_t<8>(g, descs, st, items, prm, counters, dom, found, failed, s);
    else if (prm.team_lanes == 32) e = launch_search_t<32>(g, descs, st, items, prm, counters, dom, found, failed, s);
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search<32>, kSearchWarps * 32, 0);
    if (per_sm <= 0) per_sm = 1;
    return (uint32_t)(num_sms() * per_sm * kSearchWarps);
}

}  // namespace dev
}  // namespace tfsm
