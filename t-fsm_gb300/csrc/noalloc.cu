// Allocation-free support evaluation: tfsm_evaluate_support_noalloc (include/tfsm.h).
//
// Who needs it: callers that must not allocate device memory while they evaluate a pattern —
// for example code that runs under a framework whose caching allocator owns the whole device
// (a stray cudaMalloc fragments its pool or exceeds its memory cap), latency-critical callers for
// whom the implicit device-wide synchronisation of cudaMalloc/cudaFree is unacceptable, or code that
// has run out of device memory and still has to finish its work.  Those callers get the same
// kernels as tfsm_evaluate_support, but every per-call buffer (pattern descriptor, status,
// work-item tables, the three domain bitmaps) is carved out of one file-scope device array of fixed size,
// so the call itself allocates nothing on the device and calls no allocating library routine.
//
// Limits and sharing:
//   * the array holds kScratchBytes (16 MiB) on every GPU that loads the library, until exit;
//   * a pattern whose domain bitmaps need more than that is rejected with TFSM_ERR_LIMIT;
//   * hub splitting is off on this path (its task buffers would need more scratch); automorphic
//     vertices are searched separately — both change speed only, never results;
//   * every call on a device reuses the same array and leaves its contents behind: the status block
//     and counters are cleared at the start of each call and the kernels rewrite every bitmap word
//     they read, but two calls whose work overlaps on the GPU race on the array, so calls must not
//     overlap (calls on one graph handle are serialised by the handle's lock);
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current; make that first call before any stream capture;
//   * the address is kept for the life of the process: after cudaDeviceReset (or anything else
//     that destroys the device's primary context) this entry point must not be called again;
//   * the work runs on the graph handle's own non-blocking stream, and the caller's current
//     device is restored before the call returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/tfsm.h"
#include "cuda/dev_common.cuh"
#include "cuda/kernels.h"
#include "engine.hpp"
#include "noalloc.hpp"

namespace tfsm {

namespace {

constexpr size_t kScratchBytes = 16u << 20;  // the fixed maximum: 16 MiB per device
constexpr int kMaxDevices = 64;
constexpr uint32_t kChunkWords = 8;          // bitmap words per search item on this path
constexpr size_t kAlign = 256;

// The scratch array itself.  In host code this name is only a host-side stand-in for the device
// object; kernels must be given the address returned by cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on `device` (which must be current); looked up once.
int scratch_address(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return TFSM_ERR_LIMIT;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return TFSM_ERR_CUDA;
        g_scratch_ptr[device] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[device];
    return TFSM_OK;
}

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Makes `device` current for the guard's lifetime and restores the caller's device afterwards.
struct DeviceGuard {
    int saved = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&saved) != cudaSuccess) return;
        ok = saved == device || cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

#define NA_CK(x)                                   \
    do {                                           \
        if ((x) != cudaSuccess) {                  \
            msg = "CUDA error in " #x;             \
            return TFSM_ERR_CUDA;                  \
        }                                          \
    } while (0)

// Same rule as the engine's plan: fewest candidates next, ties to the larger pattern degree.
void plan_from(int n, const uint32_t *adj, const int *deg, const uint32_t *dsize, int start, uint8_t *order,
               uint32_t *bn) {
    uint32_t visited = 1u << start, reach = adj[start];
    order[0] = (uint8_t)start;
    bn[0] = 0;
    for (int i = 1; i < n; ++i) {
        int next = -1;
        for (int j = 0; j < n; ++j) {
            if (((visited >> j) & 1u) || !((reach >> j) & 1u)) continue;
            if (next < 0 || dsize[j] < dsize[next] || (dsize[j] == dsize[next] && deg[j] > deg[next])) next = j;
        }
        order[i] = (uint8_t)next;
        bn[i] = adj[next] & visited;
        visited |= 1u << next;
        reach |= adj[next];
    }
}

}  // namespace

int noalloc_evaluate(const GpuEngine &eng, const tfsm_pattern *tp, uint32_t tau, bool exact, tfsm_result *out,
                     const char *&msg) {
    using dev::PatDesc;
    using dev::PatStatus;
    msg = "";
    std::memset(out, 0, sizeof(*out));
    // ---- pattern from its DFS codes (fixed-size storage only) ----
    if (!tp || tp->n_codes <= 0 || !tp->codes) {
        msg = "pattern has no DFS codes";
        return TFSM_ERR_ARG;
    }
    int n = 0;
    int label[dev::kMaxN];
    uint32_t adj[dev::kMaxN] = {0};
    int deg[dev::kMaxN] = {0};
    int elab[dev::kMaxN][dev::kMaxN];
    for (int i = 0; i < tp->n_codes; ++i) {
        const tfsm_dfs_code &c = tp->codes[i];
        if (i == 0) {
            if (c.from != 0 || c.to != 1) {
                msg = "first DFS code must be (0,1,...)";
                return TFSM_ERR_ARG;
            }
            label[0] = c.from_label;
            label[1] = c.to_label;
            n = 2;
        } else {
            const bool fwd = c.to == n && c.from >= 0 && c.from < n;
            const bool bwd = c.from >= 0 && c.from < n && c.to >= 0 && c.to < n && c.from != c.to;
            if (!fwd && !bwd) {
                msg = "a DFS code neither extends nor closes the pattern";
                return TFSM_ERR_ARG;
            }
            if (fwd && n >= dev::kMaxN) {
                msg = "pattern has more than 16 vertices";
                return TFSM_ERR_PATTERN;
            }
            if (label[c.from] != c.from_label || (bwd && label[c.to] != c.to_label)) {
                msg = "a DFS code has vertex labels inconsistent with earlier codes";
                return TFSM_ERR_ARG;
            }
            if (bwd && ((adj[c.from] >> c.to) & 1u)) {
                msg = "a DFS code repeats an edge";
                return TFSM_ERR_ARG;
            }
            if (fwd) label[n++] = c.to_label;
        }
        adj[c.from] |= 1u << c.to;
        adj[c.to] |= 1u << c.from;
        deg[c.from]++;
        deg[c.to]++;
        elab[c.from][c.to] = elab[c.to][c.from] = c.edge_label;
    }
    out->n_vertices = n;
    // ---- descriptor ----
    PatDesc D;
    std::memset(&D, 0, sizeof(D));
    for (int k = 0; k < dev::kMaxPush; ++k)  // no previous level on this path: no push-down sources
        for (int u = 0; u < dev::kMaxN; ++u) D.push_off[k][u] = -1;
    std::memset(D.el, dev::kNoEdge, sizeof(D.el));
    D.n = n;
    D.n_reps = n;
    D.filter_mask = 0xffffffffu;  // no parent: every vertex is tested
    bool trivial = false, distinct = true;
    uint64_t words = 0;
    for (int u = 0; u < n; ++u) {
        const int dl = eng.dense_label(label[u]);
        if (dl < 0) trivial = true;
        D.lab[u] = dl < 0 ? 0 : dl;
        D.deg[u] = deg[u];
        D.adj[u] = adj[u];
        D.rep[u] = u;
        D.orbit_mask[u] = 1u << u;
        D.parent_off[u] = -1;
        for (int w = 0; w < n; ++w) {
            if (!((adj[u] >> w) & 1u)) continue;
            const int de = eng.dense_edge_label(elab[u][w]);
            if (de < 0) trivial = true;
            else D.el[u][w] = (uint8_t)de;
        }
        for (int v = 0; v < u; ++v) distinct = distinct && label[v] != label[u];
    }
    if (trivial) {  // a label that is not frequent: no embedding in the pruned graph
        out->status = TFSM_OK;
        out->decided_by_filter = 1;
        return TFSM_OK;
    }
    int n_edges = 0;
    for (int u = 0; u < n; ++u) n_edges += deg[u];
    n_edges /= 2;
    D.express = distinct && n_edges == n - 1;
    for (int u = 0; u < n; ++u) {
        // neighbour-label-frequency requirements
        for (int w = 0; w < n; ++w) {
            if (!((adj[u] >> w) & 1u)) continue;
            int k = 0;
            while (k < D.nlf_n[u] && D.nlf_lab[u][k] != (uint8_t)D.lab[w]) ++k;
            if (k == dev::kMaxNlf) continue;  // requirements beyond the first kMaxNlf labels are dropped
            if (k == D.nlf_n[u]) {
                D.nlf_lab[u][k] = (uint8_t)D.lab[w];
                D.nlf_cnt[u][k] = 0;
                D.nlf_n[u]++;
            }
            D.nlf_cnt[u][k]++;
        }
        D.lstart[u] = eng.label_first(D.lab[u]);
        D.lsize[u] = eng.label_size(D.lab[u]);
        D.words[u] = (D.lsize[u] + 31) / 32;
        D.off[u] = words;
        words += D.words[u];
    }
    // ---- scratch layout ----
    const size_t o_desc = 0;
    const size_t o_status = align_up(o_desc + sizeof(PatDesc));
    const size_t o_counters = align_up(o_status + sizeof(PatStatus));
    const size_t o_item_pu = align_up(o_counters + dev::kNumCounters * sizeof(uint32_t));
    const size_t o_prefix = align_up(o_item_pu + dev::kMaxN * sizeof(uint32_t));
    const size_t o_igroup = align_up(o_prefix + (dev::kMaxN + 1) * sizeof(uint64_t));
    const size_t o_ientries = align_up(o_igroup + sizeof(dev::ItemGroup));
    const size_t o_pools = align_up(o_ientries + dev::kMaxN * sizeof(dev::ItemEntry));
    const size_t need = o_pools + 3 * words * sizeof(uint32_t);
    if (need > kScratchBytes) {
        msg = "pattern too large for the allocation-free path: its domain bitmaps and work items need more than "
              "the 16 MiB scratch array (use tfsm_evaluate_support)";
        return TFSM_ERR_LIMIT;
    }
    // ---- set-up on the graph's device ----
    const DeviceGuard on_device(eng.device());
    if (!on_device.ok) {
        msg = "cannot make the graph's device current";
        return TFSM_ERR_CUDA;
    }
    unsigned char *base = nullptr;
    const int rc = scratch_address(eng.device(), &base);
    if (rc != TFSM_OK) {
        msg = "cannot look up the scratch array's device address";
        return rc;
    }
    PatDesc *d_desc = reinterpret_cast<PatDesc *>(base + o_desc);
    PatStatus *d_status = reinterpret_cast<PatStatus *>(base + o_status);
    uint32_t *d_counters = reinterpret_cast<uint32_t *>(base + o_counters);
    uint32_t *d_item_pu = reinterpret_cast<uint32_t *>(base + o_item_pu);
    uint64_t *d_prefix = reinterpret_cast<uint64_t *>(base + o_prefix);
    dev::ItemGroup *d_igroup = reinterpret_cast<dev::ItemGroup *>(base + o_igroup);
    dev::ItemEntry *d_ientries = reinterpret_cast<dev::ItemEntry *>(base + o_ientries);
    uint32_t *d_dom = reinterpret_cast<uint32_t *>(base + o_pools);
    uint32_t *d_found = d_dom + words;
    uint32_t *d_failed = d_found + words;
    cudaStream_t s = eng.stream();
    const dev::Graph &g = eng.device_graph();

    uint32_t item_pu[dev::kMaxN];
    uint64_t prefix[dev::kMaxN + 1];
    prefix[0] = 0;
    for (int u = 0; u < n; ++u) {
        item_pu[u] = (uint32_t)u;  // pattern 0
        prefix[u + 1] = prefix[u] + D.words[u];
    }
    NA_CK(cudaMemcpyAsync(d_desc, &D, sizeof(D), cudaMemcpyHostToDevice, s));
    NA_CK(cudaMemsetAsync(d_status, 0, sizeof(PatStatus), s));  // the previous call's status stays behind
    NA_CK(cudaMemsetAsync(d_counters, 0, dev::kNumCounters * sizeof(uint32_t), s));
    NA_CK(cudaMemcpyAsync(d_item_pu, item_pu, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    NA_CK(cudaMemcpyAsync(d_prefix, prefix, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    // every bitmap word of every vertex is written here, so no clearing of the pools is needed
    NA_CK(dev::launch_domain_init(g, d_desc, d_status, d_item_pu, d_prefix, (uint32_t)n, words, d_dom, d_found,
                                  d_failed, nullptr, 0, words, s));
    PatStatus st;
    NA_CK(cudaMemcpyAsync(&st, d_status, sizeof(st), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    // arc consistency: two rounds, express patterns to the fixpoint (32 rounds at most; one not
    // settled by then is searched instead)
    const int rounds_cap = D.express ? 32 : 2;
    bool settled = true;
    for (int round = 0; round < rounds_cap; ++round) {
        bool viable = true;
        for (int u = 0; u < n; ++u) viable = viable && (exact ? st.dom_size[u] > 0 : st.dom_size[u] >= tau);
        if (!viable || (round > 0 && !((st.changed >> (round - 1)) & 1u))) break;
        NA_CK(dev::launch_refine(g, d_desc, d_status, d_item_pu, d_prefix, (uint32_t)n, words, d_dom, words, round, tau,
                                 exact, s));
        NA_CK(cudaMemcpyAsync(&st, d_status, sizeof(st), cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        settled = !((st.changed >> round) & 1u);
    }
    const bool express = D.express && settled;
    uint32_t mn = UINT32_MAX;
    for (int u = 0; u < n; ++u) mn = mn < st.dom_size[u] ? mn : st.dom_size[u];
    out->status = TFSM_OK;
    if (express || (exact ? mn == 0 : mn < tau)) {
        out->decided_by_filter = 1;
        if (express && mn > 0)
            for (int u = 0; u < n; ++u) out->mni[u] = st.dom_size[u];
        out->support = express && mn > 0 ? mn : 0;
        out->frequent = express && mn >= tau && mn > 0;
        return TFSM_OK;
    }
    // ---- search ----
    for (int u = 0; u < n; ++u) {
        uint32_t bn[dev::kMaxN];
        plan_from(n, adj, deg, st.dom_size, u, D.order[u], bn);
    }
    NA_CK(cudaMemcpyAsync(d_desc, &D, sizeof(D), cudaMemcpyHostToDevice, s));
    // One item group over every vertex: their runs of words interleaved round by round, as the
    // engine interleaves its items (dev::item_at decodes them on the device).
    dev::ItemEntry ent[dev::kMaxN];
    size_t m = 0;
    for (int u = 0; u < n; ++u) {
        if (!D.words[u]) continue;
        dev::ItemEntry &e = ent[m++];
        std::memset(&e, 0, sizeof(e));
        e.pat = 0;
        e.u = (uint16_t)u;
        e.words = D.words[u];
        e.runs = (D.words[u] + kChunkWords - 1) / kChunkWords;
    }
    std::stable_sort(ent, ent + m, [](const dev::ItemEntry &x, const dev::ItemEntry &y) { return x.runs > y.runs; });
    uint64_t n_items = 0;
    for (size_t i = m; i-- > 0;) {
        const uint32_t below = i + 1 < m ? ent[i + 1].runs : 0;
        n_items += (uint64_t)(i + 1) * (ent[i].runs - below);
        ent[i].before = n_items;
    }
    dev::ItemGroup grp;
    grp.first_item = 0;
    grp.first_entry = 0;
    grp.n_entries = (uint32_t)m;
    if (m) {
        NA_CK(cudaMemcpyAsync(d_igroup, &grp, sizeof(grp), cudaMemcpyHostToDevice, s));
        NA_CK(cudaMemcpyAsync(d_ientries, ent, m * sizeof(dev::ItemEntry), cudaMemcpyHostToDevice, s));
    }
    dev::SearchParams prm;
    std::memset(&prm, 0, sizeof(prm));
    prm.tau = tau;
    prm.exact = exact ? 1 : 0;
    prm.n_items = (uint32_t)n_items;
    prm.n_groups = 1;
    prm.max_n = (uint32_t)n;
    prm.chunk_words = kChunkWords;
    prm.split = 0;  // no hub splitting on this path (its task buffers would need more scratch)
    prm.isect_ratio = 16;
    prm.team_lanes = 32;
    prm.n_pats = 1;
    prm.words = words;
    NA_CK(dev::launch_search(g, d_desc, d_status, d_igroup, d_ientries, prm, d_counters, d_dom, d_found, d_failed,
                             nullptr, nullptr, s));
    NA_CK(cudaMemcpyAsync(&st, d_status, sizeof(st), cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    mn = UINT32_MAX;
    bool all = true;
    for (int u = 0; u < n; ++u) {
        out->mni[u] = st.found_cnt[u];
        mn = mn < st.found_cnt[u] ? mn : st.found_cnt[u];
        all = all && st.found_cnt[u] >= tau;
    }
    out->support = mn;
    out->frequent = exact ? mn >= tau : (st.state == dev::kFrequent || (st.state == dev::kRunning && all));
    out->searches = st.searches;
    out->steps = st.steps;
    return TFSM_OK;
}

}  // namespace tfsm
