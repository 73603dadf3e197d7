// Host orchestration of the GPU support evaluation.
//
// evaluate() runs, for one batch of patterns (one pattern in the plain path, a growth level or
// a slice of one in the batched path):
//   1. k_domain_init     LDF + NLF bitmaps, children starting from their parent's final domains
//                        (and those of further sub-patterns), read from earlier calls' pools
//   2. k_refine x R      arc consistency (to a fixpoint for distinct-label trees)
//   3. host              decide what the domain sizes already decide; matching orders (GQL
//                        order by domain size, serial/gmatch.h:584-685) for the rest
//   4. k_search/k_split  backtracking with early exit and hub splitting
// The device graph is uploaded once in the constructor (label-grouped ids, see dev_common.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <array>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <random>
#include <numeric>

#include "cuda/dev_common.cuh"
#include "cuda/kernels.h"
#include "engine.hpp"
#include "costmodel/features.hpp"
#include "host/lg_fast.hpp"
#if !defined(TFSM_SIMT_EMULATION)
#include "cuda/ingest.hpp"
#endif

namespace tfsm {

namespace {

#define TFSM_CK(x)                                                                                   \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) throw EngineError(10, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device buffers of the levels of one engine (bitmap pools, descriptors).  Blocks are carved from
// slabs of at least 64 MiB and handed back to the cache when their level dies, for later levels:
// a mining run calls cudaMalloc (which synchronises the device) once per slab instead of once per
// pool of every engine call, although the calls of a growth level all keep their pools (they are
// the next level's push-down sources).  Shared by the levels, so it outlives the engine if they do.
struct BufferCache {
    static constexpr size_t kSlab = 64u << 20;
    std::mutex mu;
    std::multimap<size_t, void *> free;  // bytes -> block
    std::vector<void *> slabs;
    char *cur = nullptr;                 // unused tail of the newest slab
    size_t left = 0;
    ~BufferCache() {
        for (void *p : slabs) cudaFree(p);
    }
    // a new block of `bytes` (a multiple of 64 KiB keeps every block 64 KiB-aligned)
    void *carve(size_t bytes) {
        std::lock_guard<std::mutex> lk(mu);
#if defined(TFSM_SIMT_EMULATION)  // one allocation per block: the sanitizers see each block's bounds
        left = 0;
#endif
        if (bytes > left) {
            void *p = nullptr;
#if defined(TFSM_SIMT_EMULATION)
            const size_t sz = bytes;
#else
            const size_t sz = std::max(bytes, kSlab);
#endif
            TFSM_CK(cudaMalloc(&p, sz));
            slabs.push_back(p);
            cur = static_cast<char *>(p);
            left = sz;
        }
        void *q = cur;
        cur += bytes;
        left -= bytes;
        return q;
    }
    void *take(size_t bytes, size_t &got) {  // best fit, at most twice the size asked for
        std::lock_guard<std::mutex> lk(mu);
        auto it = free.lower_bound(bytes);
        if (it == free.end() || it->first > 2 * bytes) return nullptr;
        void *p = it->second;
        got = it->first;
        free.erase(it);
        return p;
    }
    void give(void *p, size_t bytes) {
        std::lock_guard<std::mutex> lk(mu);
        free.emplace(bytes, p);
    }
};

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    size_t bytes = 0;
    std::shared_ptr<BufferCache> cache;  // null: plain cudaMalloc / cudaFree
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            if (cache) cache->give(p, bytes);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        bytes = 0;
    }
    // takes over a plain cudaMalloc allocation of `b` bytes
    void adopt(void *q, size_t b) {
        release();
        cache.reset();
        p = static_cast<T *>(q);
        bytes = b;
        n = b / sizeof(T);
    }
    // Room for at least k elements.  Cache-backed buffers come in power-of-two sizes (64 KiB at
    // least), so that pools freed by earlier calls fit later ones; other buffers grow to at least
    // twice their size.  A reallocation (cudaMalloc synchronises the device) is then rare.
    void ensure(size_t k) {
        if (k <= n && p) return;
        size_t want = sizeof(T) * std::max<size_t>(k, cache ? 1 : 2 * n);
        if (cache) {
            size_t b = 64u << 10;
            while (b < want) b *= 2;
            want = b;
        }
        release();
        size_t got = 0;
        void *q = cache ? cache->take(want, got) : nullptr;
        if (!q && cache) {
            q = cache->carve(want);
            got = want;
        } else if (!q) {
            TFSM_CK(cudaMalloc(&q, want));
            got = want;
        }
        p = static_cast<T *>(q);
        bytes = got;
        n = got / sizeof(T);
    }
};

// Page-locked staging of a call's small host -> device copies (descriptors, source table, item
// tables): a copy from it is an asynchronous DMA, where one from pageable memory waits for a staging
// copy inside the driver.  A bump allocator, rewound at the start of each engine call (every call
// ends with a synchronisation); when full, it synchronises the stream and starts over (growing if
// one copy does not fit).
struct Staging {
    unsigned char *p = nullptr;
    size_t cap = 0, used = 0;
    Staging() = default;
    Staging(const Staging &) = delete;
    Staging &operator=(const Staging &) = delete;
    ~Staging() {
        if (p) cudaFreeHost(p);
    }
    void h2d(void *dst, const void *src, size_t bytes, cudaStream_t s) {
        if (!bytes) return;
        const size_t at = (used + 255) & ~(size_t)255;
        if (at + bytes > cap) {
            TFSM_CK(cudaStreamSynchronize(s));  // earlier copies out of the buffer are done
            used = 0;
            if (bytes > cap) {
                if (p) cudaFreeHost(p);
                p = nullptr;
                cap = 0;
                const size_t want = std::max<size_t>(bytes, 4u << 20);
                TFSM_CK(cudaHostAlloc((void **)&p, want, cudaHostAllocDefault));
                cap = want;
            }
            return h2d(dst, src, bytes, s);
        }
        std::memcpy(p + at, src, bytes);
        TFSM_CK(cudaMemcpyAsync(dst, p + at, bytes, cudaMemcpyHostToDevice, s));
        used = at + bytes;
    }
};

// Page-locked landing buffer of device -> host reads (the batch's status records).
template <class T>
struct PinnedBuf {
    T *p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    void ensure(size_t k) {
        if (k <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        const size_t want = std::max<size_t>(k, 2 * n) + 16;
        TFSM_CK(cudaHostAlloc((void **)&p, want * sizeof(T), cudaHostAllocDefault));
        n = want;
    }
};

using dev::PatDesc;
using dev::PatStatus;

// An event record inside a captured launch sequence: captured as an event-record node (plain
// records inside a capture only order streams), so that it can time the graph's kernels.
inline cudaError_t record_in_sequence(cudaEvent_t e, cudaStream_t s) {
#if defined(TFSM_SIMT_EMULATION) || defined(TFSM_BOUNDS_CHECK)
    return cudaEventRecord(e, s);
#else
    return cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
#endif
}

// Records the launches of `enqueue` on stream `s` as a CUDA graph and runs it.  `exec` keeps the
// instantiated graph between calls: a sequence of the same shape (same kernels, new arguments)
// is applied with cudaGraphExecUpdate instead of a new instantiation.  The checked build (which
// synchronises inside its launchers) and the CPU emulation launch directly.
template <class F>
void run_captured(cudaStream_t s, cudaGraphExec_t &exec, F enqueue) {
#if defined(TFSM_SIMT_EMULATION) || defined(TFSM_BOUNDS_CHECK)
    (void)exec;
    (void)s;
    enqueue();
#else
    TFSM_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t graph = nullptr;
    try {
        enqueue();
    } catch (...) {
        cudaStreamEndCapture(s, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    TFSM_CK(cudaStreamEndCapture(s, &graph));
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(exec, graph, &info) != cudaSuccess) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    if (!exec) {
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) {
            exec = nullptr;
            cudaGraphDestroy(graph);
            TFSM_CK(e);
        }
    }
    cudaGraphDestroy(graph);
    TFSM_CK(cudaGraphLaunch(exec, s));
#endif
}

}  // namespace

struct Level::Impl {
    DevBuf<uint32_t> dom, found, failed;  // from the engine's BufferCache
    DevBuf<PatDesc> descs;
    std::vector<PatDesc> hdescs;
    uint64_t words = 0;
};

Level::Level() : impl(new Impl) {}
Level::~Level() = default;
Level::Level(Level &&) noexcept = default;
Level &Level::operator=(Level &&) noexcept = default;
size_t Level::size() const { return impl ? impl->hdescs.size() : 0; }

struct GpuEngine::Impl {
    dev::Graph g;
    DevBuf<uint32_t> row_off, col, label_start, lab_off;
    DevBuf<uint8_t> elab;
    std::map<int, int> vdense, edense;
    std::vector<uint32_t> lstart;  // host copy, n_labels + 1
    std::vector<float> label_mean_deg;  // per dense label: mean degree of its vertices
    uint32_t n = 0;
    uint64_t m2 = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
    // instantiated launch sequences, updated in place while their shape stays the same
    cudaGraphExec_t exec_init = nullptr, exec_search = nullptr;
    // per-call scratch
    DevBuf<PatStatus> status;
    DevBuf<uint32_t> item_pu;
    DevBuf<uint64_t> prefix;
    DevBuf<uint32_t> ritem_pu;  // the first refinement rounds' (pattern, vertex) items
    DevBuf<uint64_t> rprefix;
    DevBuf<dev::ItemGroup> igroups;    // the call's search work (dev::item_at)
    DevBuf<dev::ItemEntry> ientries;
    DevBuf<dev::SourceLevel> srcs;      // the earlier calls' pools read by this call's domain init
    DevBuf<uint32_t> counters;
    DevBuf<dev::SplitTask> splits;  // two buffers of split tasks (ping-pong between rounds)
    DevBuf<dev::SplitGroup> groups;
    std::vector<PatStatus> hstatus;
    Staging stage;                     // this call's host -> device copies
    PinnedBuf<PatStatus> status_land;  // status reads land here, then go to hstatus
    int device = 0;
    std::shared_ptr<BufferCache> cache = std::make_shared<BufferCache>();
    // also runs when a constructor throws after open()
    ~Impl() {
        if (stream) cudaStreamSynchronize(stream);
        if (exec_init) cudaGraphExecDestroy(exec_init);
        if (exec_search) cudaGraphExecDestroy(exec_search);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev_mid) cudaEventDestroy(ev_mid);
        if (stream) cudaStreamDestroy(stream);
    }
};

// The device and the engine's stream and events.
void GpuEngine::open(int device) {
    if (const char *env = std::getenv("TFSM_DEVICE")) device = std::atoi(env);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device)
        throw EngineError(9, "no CUDA device available for the GPU engine");
    TFSM_CK(cudaSetDevice(device));
    Impl &I = *impl_;
    I.device = device;
    TFSM_CK(cudaStreamCreateWithFlags(&I.stream, cudaStreamNonBlocking));
    TFSM_CK(cudaEventCreate(&I.ev0));
    TFSM_CK(cudaEventCreate(&I.ev1));
    TFSM_CK(cudaEventCreate(&I.ev_mid));
}

#if !defined(TFSM_SIMT_EMULATION)  // the CPU emulation builds its graphs on the host only
GpuEngine::GpuEngine(const std::function<void(CUstream_st *, DeviceGraphBuild &)> &build, LgGraph &summary,
                     int device)
    : impl_(new Impl) {
    auto t0 = std::chrono::steady_clock::now();
    open(device);
    Impl &I = *impl_;
    DeviceGraphBuild b;
    build(I.stream, b);
    load_breakdown_ = b.breakdown;
    load_h2d_bytes_ = b.h2d_bytes;
    summary = std::move(b.summary);
    const LgGraph &lg = summary;
    for (size_t i = 0; i < lg.freq_vlabels.size(); ++i) I.vdense[lg.freq_vlabels[i]] = (int)i;
    for (size_t i = 0; i < lg.freq_elabels.size(); ++i) I.edense[lg.freq_elabels[i]] = (int)i;
    I.lstart = std::move(b.lstart);
    I.label_mean_deg = std::move(b.label_mean_deg);
    I.n = lg.n;
    I.m2 = b.m2;
    I.row_off.adopt(b.row_off.release(), b.row_off.bytes);
    I.col.adopt(b.col.release(), b.col.bytes);
    I.elab.adopt(b.elab.release(), b.elab.bytes);
    I.label_start.adopt(b.label_start.release(), b.label_start.bytes);
    I.lab_off.adopt(b.lab_off.release(), b.lab_off.bytes);
    finish(t0);
}
#endif

GpuEngine::GpuEngine(const LgGraph &lg, int device) : impl_(new Impl) {
    auto t0 = std::chrono::steady_clock::now();
    open(device);
    Impl &I = *impl_;
    if (lg.offs[lg.n] >= (1ull << 32)) throw EngineError(5, "graph has >= 2^32 adjacency entries");
    // dense labels
    for (size_t i = 0; i < lg.freq_vlabels.size(); ++i) I.vdense[lg.freq_vlabels[i]] = (int)i;
    for (size_t i = 0; i < lg.freq_elabels.size(); ++i) I.edense[lg.freq_elabels[i]] = (int)i;
    if (I.edense.size() > 250) throw EngineError(5, "more than 250 frequent edge labels");
    const int NL = (int)lg.freq_vlabels.size();
    if (NL > 250) throw EngineError(5, "more than 250 frequent vertex labels");
    auto tck = std::chrono::steady_clock::now();
    auto checkpoint = [&](const char *what) {
        const auto now = std::chrono::steady_clock::now();
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%s%s %.2f", load_breakdown_.empty() ? "" : ", ", what,
                      std::chrono::duration<double, std::milli>(now - tck).count());
        load_breakdown_ += buf;
        tck = now;
    };
    checkpoint("device");
    const fast::LabelIndex vidx(lg.freq_vlabels), eidx(lg.freq_elabels);
    const int threads = fast::default_threads();
    // label-grouped renumbering: internal id = label_start[L] + rank within the label
    std::vector<int> dl(lg.n);
    std::vector<uint32_t> cnt((size_t)NL + 1, 0);
    for (uint32_t v = 0; v < lg.n; ++v) cnt[(size_t)(dl[v] = vidx(lg.vlabel[v])) + 1]++;
    I.lstart.assign((size_t)NL + 1, 0);
    for (int L = 0; L < NL; ++L) I.lstart[(size_t)L + 1] = I.lstart[(size_t)L] + cnt[(size_t)L + 1];
    // Inside a label, vertices are ranked by descending degree (ties: pruned order) and the ranks
    // fill the label's bitmap words column by column: bit 0 of every word holds the top ranks, bit
    // 1 the next ones, and so on.  Warps take words in parallel and bits in order, so the search
    // meets well-connected candidates first (they usually complete an embedding quickly: a
    // frequent pattern reaches tau with fewer exhaustive failures), while every word keeps a mix of
    // degrees for the per-word refinement.  Any order gives the same results.
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> members((size_t)NL);  // (-degree, v)
    for (int L = 0; L < NL; ++L) members[(size_t)L].reserve(cnt[(size_t)L + 1]);
    for (uint32_t v = 0; v < lg.n; ++v) members[(size_t)dl[v]].push_back({~lg.degree(v), v});
    std::vector<uint32_t> to_int(lg.n);
    for (int L = 0; L < NL; ++L) {
        auto &mv = members[(size_t)L];
        std::sort(mv.begin(), mv.end());  // descending degree, then ascending pruned id
        const uint32_t c = (uint32_t)mv.size(), words = (c + 31) / 32;
        uint32_t r = 0;
        for (uint32_t bit = 0; bit < 32 && r < c; ++bit)
            for (uint32_t w = 0; w < words && r < c; ++w) {
                const uint32_t local = w * 32 + bit;
                if (local < c) to_int[mv[r++].second] = I.lstart[(size_t)L] + local;
            }
    }
    std::vector<uint32_t> from_int(lg.n);
    for (uint32_t v = 0; v < lg.n; ++v) from_int[to_int[v]] = v;
    {
        std::vector<double> dsum((size_t)NL, 0.0);
        for (uint32_t v = 0; v < lg.n; ++v) dsum[(size_t)dl[v]] += lg.degree(v);
        I.label_mean_deg.assign((size_t)NL, 0.f);
        for (int L = 0; L < NL; ++L)
            if (cnt[(size_t)L + 1]) I.label_mean_deg[(size_t)L] = (float)(dsum[(size_t)L] / cnt[(size_t)L + 1]);
    }
    // CSR in internal ids, each list sorted by (internal id, edge label): row x is v's list mapped
    // through to_int and re-sorted (ids of one label keep their order, labels are regrouped).
    std::vector<uint32_t> off((size_t)lg.n + 1, 0);
    for (uint32_t x = 0; x < lg.n; ++x) off[(size_t)x + 1] = off[x] + lg.degree(from_int[x]);
    std::vector<uint32_t> col(off[lg.n]);
    std::vector<uint8_t> el(off[lg.n]);
    // label offsets, label-major: lab_off[L * n + x] = first position of x's neighbours >= label L
    const size_t stride = (size_t)NL + 1;
    if ((size_t)lg.n * stride >= (1ull << 34)) throw EngineError(5, "label-offset table too large");
    std::vector<uint32_t> lab_off((size_t)lg.n * stride);
    fast::parallel_ranges(lg.n, threads, [&](int, size_t x0, size_t x1) {
        std::vector<uint64_t> key;
        for (size_t x = x0; x < x1; ++x) {
            const uint32_t v = from_int[x];
            key.clear();
            for (uint64_t i = lg.offs[v]; i < lg.offs[v + 1]; ++i)
                key.push_back(((uint64_t)to_int[lg.nbr[i]] << 8) | (uint64_t)eidx(lg.elab[i]));
            std::sort(key.begin(), key.end());
            const uint32_t b = off[x];
            for (size_t k = 0; k < key.size(); ++k) {
                col[b + k] = (uint32_t)(key[k] >> 8);
                el[b + k] = (uint8_t)(key[k] & 0xffu);
            }
            uint32_t pos = b;
            const uint32_t end = off[x + 1];
            for (int L = 0; L <= NL; ++L) {
                const uint32_t first = I.lstart[(size_t)L];  // lstart[NL] == n: past every id
                while (pos < end && col[pos] < first) ++pos;
                lab_off[(size_t)L * lg.n + x] = L == NL ? end : pos;
            }
        }
    });
    checkpoint("csr+labels");
    I.n = lg.n;
    I.m2 = off[lg.n];
    I.row_off.ensure(off.size());
    I.col.ensure(col.size() + dev::kColPad);  // padded for the search's 128-bit loads
    I.elab.ensure(el.size());
    I.label_start.ensure(I.lstart.size());
    I.lab_off.ensure(lab_off.size());
    if (!lab_off.empty())
        TFSM_CK(cudaMemcpyAsync(I.lab_off.p, lab_off.data(), lab_off.size() * 4, cudaMemcpyHostToDevice, I.stream));
    TFSM_CK(cudaMemcpyAsync(I.row_off.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice, I.stream));
    TFSM_CK(cudaMemsetAsync(I.col.p + col.size(), 0xff, dev::kColPad * 4, I.stream));
    if (!col.empty()) {
        TFSM_CK(cudaMemcpyAsync(I.col.p, col.data(), col.size() * 4, cudaMemcpyHostToDevice, I.stream));
        TFSM_CK(cudaMemcpyAsync(I.elab.p, el.data(), el.size(), cudaMemcpyHostToDevice, I.stream));
    }
    TFSM_CK(cudaMemcpyAsync(I.label_start.p, I.lstart.data(), I.lstart.size() * 4, cudaMemcpyHostToDevice,
                            I.stream));
    TFSM_CK(cudaStreamSynchronize(I.stream));
    checkpoint("upload");
    load_h2d_bytes_ = (lab_off.size() + off.size() + col.size() + I.lstart.size()) * 4 + el.size();
    finish(t0);
}

// Device graph view, counters, split buffers and staging, once the graph arrays are in place.
void GpuEngine::finish(std::chrono::steady_clock::time_point t0) {
    Impl &I = *impl_;
    const int NL = (int)I.lstart.size() - 1;
    I.g.n = I.n;
    I.g.m2 = I.m2;
    I.g.n_labels = NL;
    I.g.row_off = I.row_off.p;
    I.g.col = I.col.p;
    I.g.elab = I.elab.p;
    I.g.label_start = I.label_start.p;
    I.g.lab_off = I.lab_off.p;
    I.counters.ensure((size_t)dev::kMaxPasses * dev::kNumCounters);
    // Two buffers of split tasks (88 B each) and as many groups (20 B each): one task per directed
    // adjacency entry, 2 M to 16 M (at most 3.1 GB; searches that find no room are set aside for the
    // next pass).  TFSM_SPLIT_CAPACITY sets both counts (tests use a tiny one to drive the
    // buffer-full paths).
    size_t task_cap = 2u << 20;
    while (task_cap < (16u << 20) && task_cap < (size_t)I.m2) task_cap *= 2;
    size_t group_cap = task_cap;
    if (const char *env = std::getenv("TFSM_SPLIT_CAPACITY")) {
        const long c = std::atol(env);
        if (c < 1 || c > (1l << 26)) throw EngineError(1, "TFSM_SPLIT_CAPACITY must be in 1..2^26");
        task_cap = group_cap = (size_t)c;
    }
    I.splits.ensure(2 * task_cap);
    I.groups.ensure(group_cap);

    upload_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

GpuEngine::~GpuEngine() = default;

uint64_t GpuEngine::graph_bytes() const {
    return (uint64_t)(impl_->n + 1) * 4 + impl_->m2 * 5 + (uint64_t)impl_->n * impl_->lstart.size() * 4;
}
uint32_t GpuEngine::n_vertices() const { return impl_->n; }
void GpuEngine::device_memory(size_t &free_bytes, size_t &total_bytes) const {
    free_bytes = total_bytes = 0;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return;
    if (cur != impl_->device) cudaSetDevice(impl_->device);
    if (cudaMemGetInfo(&free_bytes, &total_bytes) != cudaSuccess) free_bytes = total_bytes = 0;
    if (cur != impl_->device) cudaSetDevice(cur);
}
int GpuEngine::dense_label(int label) const {
    auto it = impl_->vdense.find(label);
    return it == impl_->vdense.end() ? -1 : it->second;
}
int GpuEngine::device() const { return impl_->device; }
CUstream_st *GpuEngine::stream() const { return impl_->stream; }
const dev::Graph &GpuEngine::device_graph() const { return impl_->g; }
int GpuEngine::dense_edge_label(int label) const {
    auto it = impl_->edense.find(label);
    return it == impl_->edense.end() ? -1 : it->second;
}
void GpuEngine::export_graph(uint32_t *row_off, uint32_t *col, uint8_t *elab, uint32_t *label_start,
                             uint32_t *lab_off, float *label_mean_degree) const {
    const Impl &I = *impl_;
    const size_t stride = I.lstart.size();
    auto get = [&](void *dst, const void *src, size_t bytes) {
        if (dst && bytes) TFSM_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, I.stream));
    };
    get(row_off, I.row_off.p, ((size_t)I.n + 1) * 4);
    get(col, I.col.p, I.m2 * 4);
    get(elab, I.elab.p, I.m2);
    get(label_start, I.label_start.p, stride * 4);
    get(lab_off, I.lab_off.p, (size_t)I.n * stride * 4);
    TFSM_CK(cudaStreamSynchronize(I.stream));
    if (label_mean_degree)
        std::copy(I.label_mean_deg.begin(), I.label_mean_deg.end(), label_mean_degree);
}

uint32_t GpuEngine::label_first(int dense) const { return impl_->lstart[(size_t)dense]; }
uint32_t GpuEngine::label_size(int dense) const {
    return impl_->lstart[(size_t)dense + 1] - impl_->lstart[(size_t)dense];
}

namespace {

// GQL-style order from `start` (serial/gmatch.h:584-620): repeatedly take the unvisited vertex
// adjacent to the visited set with the fewest candidates, ties to the larger pattern degree.
void gql_plan(const Pattern &pat, const uint32_t *dsize, int start, uint8_t *order, uint32_t *bn) {
    const int n = pat.size();
    uint32_t visited = 1u << start, adjm = 0;
    for (auto &e : pat.vertices[start].edges) adjm |= 1u << e.to;
    order[0] = (uint8_t)start;
    bn[0] = 0;
    for (int i = 1; i < n; ++i) {
        int next = -1;
        for (int j = 0; j < n; ++j) {
            if ((visited >> j) & 1u || !((adjm >> j) & 1u)) continue;
            if (next < 0 || dsize[j] < dsize[next] || (dsize[j] == dsize[next] && pat.degree(j) > pat.degree(next)))
                next = j;
        }
        uint32_t b = 0;
        for (auto &e : pat.vertices[next].edges)
            if ((visited >> e.to) & 1u) b |= 1u << e.to;
        order[i] = (uint8_t)next;
        bn[i] = b;
        visited |= 1u << next;
        for (auto &e : pat.vertices[next].edges) adjm |= 1u << e.to;
    }
}

}  // namespace

void GpuEngine::evaluate(const std::vector<const Pattern *> &pats, const std::vector<LevelRef> &parent,
                         uint32_t tau, const EngineOptions &opt, Level &out, std::vector<EvalResult> &res,
                         const std::vector<std::vector<PushSource>> *push) {
    Impl &I = *impl_;
    struct WallClock {  // host wall time of the whole call, every return path
        double &acc;
        std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
        ~WallClock() {
            acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
    } wall{times_.engine_ms};
    // host wall time per phase: descriptors, init+refine, plans, items, search, results
    auto tphase = std::chrono::steady_clock::now();
    auto phase = [&](int k) {
        const auto now = std::chrono::steady_clock::now();
        times_.phase_ms[k] += std::chrono::duration<double, std::milli>(now - tphase).count();
        tphase = now;
    };
    const size_t P = pats.size();
    res.assign(P, EvalResult());
    if (!out.impl) out.impl.reset(new Level::Impl);
    Level::Impl &L = *out.impl;
    L.dom.cache = L.found.cache = L.failed.cache = I.cache;
    L.descs.cache = I.cache;
    L.hdescs.assign(P, PatDesc());
    std::vector<char> trivial(P, 0), express(P, 0);
    uint64_t total = 0;
    // the earlier calls' pools this call reads (parents, push-down sources): one table slot each
    std::vector<dev::SourceLevel> srcs;
    std::map<const Level::Impl *, uint32_t> slot_of;
    auto source = [&](const LevelRef &r) -> const PatDesc * {
        if (!r.lvl || !r.lvl->impl || r.idx < 0 || (size_t)r.idx >= r.lvl->impl->hdescs.size()) return nullptr;
        return &r.lvl->impl->hdescs[(size_t)r.idx];
    };
    auto ref = [&](const LevelRef &r, uint64_t off) -> int64_t {
        const Level::Impl *li = r.lvl->impl.get();
        auto it = slot_of.find(li);
        if (it == slot_of.end()) {
            // slot << kSrcShift must stay a non-negative int64 (a negative reference means none)
            if (srcs.size() >= (1ull << (63 - dev::kSrcShift))) throw EngineError(6, "too many source levels");
            it = slot_of.emplace(li, (uint32_t)srcs.size()).first;
            srcs.push_back({li->dom.p, li->failed.p, li->words});
        }
        return (int64_t)(((uint64_t)it->second << dev::kSrcShift) | off);
    };
    for (size_t p = 0; p < P; ++p) {
        const Pattern &pat = *pats[p];
        PatDesc &D = L.hdescs[p];
        std::memset(&D, 0, sizeof(D));
        const int n = pat.size();
        if (n > dev::kMaxN) throw EngineError(4, "pattern has more than 32 vertices");
        D.n = n;
        res[p].mni.assign((size_t)n, 0);
        std::memset(D.el, dev::kNoEdge, sizeof(D.el));
        for (int u = 0; u < n; ++u) {
            const int dl = dense_label(pat.label(u));
            if (dl < 0) trivial[p] = 1;
            D.lab[u] = dl < 0 ? 0 : dl;
            D.deg[u] = pat.degree(u);
            for (auto &e : pat.vertices[u].edges) {
                D.adj[u] |= 1u << e.to;
                auto it = I.edense.find(e.label);
                if (it == I.edense.end()) trivial[p] = 1;
                else D.el[u][e.to] = (uint8_t)it->second;
            }
            std::map<int, int> need;
            for (auto &e : pat.vertices[u].edges) need[dense_label(pat.label(e.to))]++;
            for (auto &kv : need) {
                if (kv.first < 0 || D.nlf_n[u] == dev::kMaxNlf) continue;
                D.nlf_lab[u][D.nlf_n[u]] = (uint8_t)kv.first;
                D.nlf_cnt[u][D.nlf_n[u]] = (uint8_t)std::min(kv.second, 255);
                D.nlf_n[u]++;
            }
            D.lstart[u] = I.lstart[(size_t)D.lab[u]];
            D.lsize[u] = I.lstart[(size_t)D.lab[u] + 1] - D.lstart[u];
            D.words[u] = (D.lsize[u] + 31) / 32;
            D.off[u] = total;
            total += D.words[u];
            D.parent_off[u] = -1;
            const PatDesc *PD = p < parent.size() ? source(parent[p]) : nullptr;
            if (PD && u < PD->n) D.parent_off[u] = ref(parent[p], PD->off[u]);
        }
        static_assert(kMaxPushSources == dev::kMaxPush, "push-down sources");
        for (int k = 0; k < dev::kMaxPush; ++k)
            for (int u = 0; u < dev::kMaxN; ++u) D.push_off[k][u] = -1;
        if (push && p < push->size()) {
            int k = 0;
            for (const PushSource &src : (*push)[p]) {
                if (k == dev::kMaxPush) break;
                const PatDesc *SD = source(src.at);
                if (!SD) continue;
                bool any = false;
                for (int u = 0; u < n; ++u) {
                    const int s = src.vertex[u];
                    if (s < 0 || s >= SD->n || SD->lab[s] != D.lab[u]) continue;  // same label: same word range
                    D.push_off[k][u] = ref(src.at, SD->off[s]);
                    any = true;
                }
                k += any ? 1 : 0;
            }
        }
        // Domain init tests degree and neighbour labels of u unless u starts from a parent domain
        // that passed the same test (same degree, same requirements): a child's vertices away from
        // its newest edge.
        D.filter_mask = 0;
        {
            const PatDesc *PD = p < parent.size() ? source(parent[p]) : nullptr;
            for (int u = 0; u < n; ++u) {
                bool same = PD && u < PD->n && D.parent_off[u] >= 0 && PD->deg[u] == D.deg[u] &&
                            PD->nlf_n[u] == D.nlf_n[u];
                for (int k = 0; same && k < D.nlf_n[u]; ++k)
                    same = PD->nlf_lab[u][k] == D.nlf_lab[u][k] && PD->nlf_cnt[u][k] == D.nlf_cnt[u][k];
                if (!same) D.filter_mask |= 1u << u;
            }
        }
        const std::vector<int> orb = automorphism_orbits(pat);
        for (int u = 0; u < n; ++u) {
            D.rep[u] = orb[u];
            for (int k = 0; k < n; ++k)
                if (orb[k] == orb[u]) D.orbit_mask[u] |= 1u << k;
            if (orb[u] == u) D.n_reps++;
        }
        express[p] = pat.distinct_labels() && pat.acyclic();
        D.express = express[p];
    }
    if (total >= (1ull << 32)) throw EngineError(6, "batch needs more than 2^32 bitmap words");
    phase(0);
    L.words = total;
    L.dom.ensure(total);
    L.found.ensure(total);
    L.failed.ensure(total);
    L.descs.ensure(P);
    I.status.ensure(P);
    I.hstatus.assign(P, PatStatus());
    I.status_land.ensure(P);
    I.stage.used = 0;  // the previous call ended with a synchronisation
    I.stage.h2d(L.descs.p, L.hdescs.data(), P * sizeof(PatDesc), I.stream);
    times_.h2d_bytes += P * sizeof(PatDesc);
    TFSM_CK(cudaMemsetAsync(I.status.p, 0, P * sizeof(PatStatus), I.stream));

    I.srcs.ensure(std::max<size_t>(1, srcs.size()));
    if (!srcs.empty()) {
        I.stage.h2d(I.srcs.p, srcs.data(), srcs.size() * sizeof(dev::SourceLevel), I.stream);
        times_.h2d_bytes += srcs.size() * sizeof(dev::SourceLevel);
    }

    // ---- domain init over every (pattern, vertex) ----
    std::vector<uint32_t> item_pu;
    std::vector<uint64_t> prefix;
    // `wide`: the domain-init form, where a vertex with filter_mask clear takes one unit per 32 words
    auto build_items = [&](const std::vector<char> &active, bool wide) {
        item_pu.clear();
        prefix.assign(1, 0);
        for (size_t p = 0; p < P; ++p) {
            if (!active[p]) continue;
            const PatDesc &D = L.hdescs[p];
            for (int u = 0; u < D.n; ++u) {
                const bool w = wide && !((D.filter_mask >> u) & 1u);
                item_pu.push_back(((uint32_t)p << 8) | (uint32_t)u | (w ? dev::kWideItem : 0u));
                prefix.push_back(prefix.back() + (w ? (D.words[u] + 31) / 32 : D.words[u]));
            }
        }
        I.item_pu.ensure(item_pu.size());
        I.prefix.ensure(prefix.size());
        if (!item_pu.empty()) {
            I.stage.h2d(I.item_pu.p, item_pu.data(), item_pu.size() * 4, I.stream);
            I.stage.h2d(I.prefix.p, prefix.data(), prefix.size() * 8, I.stream);
            times_.h2d_bytes += item_pu.size() * 4 + prefix.size() * 8;
        }
    };
    // the batch's status records: DMA into page-locked memory, one synchronisation, then a copy
    auto land_status = [&]() {
        TFSM_CK(cudaMemcpyAsync(I.status_land.p, I.status.p, P * sizeof(PatStatus), cudaMemcpyDeviceToHost,
                                I.stream));
        TFSM_CK(cudaStreamSynchronize(I.stream));
        std::memcpy(I.hstatus.data(), I.status_land.p, P * sizeof(PatStatus));
        times_.d2h_bytes += P * sizeof(PatStatus);
    };
    auto read_status = [&]() { land_status(); };
    // end of a timed phase followed by a status read: one host round trip for both
    auto time_and_read_status = [&]() -> double {
        TFSM_CK(cudaEventRecord(I.ev1, I.stream));
        land_status();
        float ms = 0;
        TFSM_CK(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
        return ms;
    };

    phase(1);
    // ---- domain init and the first arc-consistency rounds: one launch sequence (a CUDA graph),
    // then one status read.  k_refine itself skips patterns that can no longer reach tau or that
    // the previous round left unchanged.
    std::vector<char> active(P, 0);
    for (size_t p = 0; p < P; ++p) active[p] = !trivial[p];
    // the first refinement rounds: every vertex, or (scoped) for a pattern that starts from its
    // parent's final domains only the two vertices of its newest edge (the rest were refined against
    // the same edges in the parent's call); express patterns always refine every vertex
    std::vector<uint32_t> ritem_pu;
    std::vector<uint64_t> rprefix(1, 0);
    {
        const bool scoped = opt.refine_scope != 0;
        for (size_t p = 0; p < P; ++p) {
            if (!active[p]) continue;
            const PatDesc &D = L.hdescs[p];
            const bool has_parent = p < parent.size() && parent[p].lvl != nullptr;
            const DfsCode &last = pats[p]->codes.back();
            for (int u = 0; u < D.n; ++u) {
                if (scoped && has_parent && !express[p] && u != last.from && u != last.to) continue;
                ritem_pu.push_back(((uint32_t)p << 8) | (uint32_t)u);
                rprefix.push_back(rprefix.back() + D.words[u]);
            }
        }
        I.ritem_pu.ensure(std::max<size_t>(1, ritem_pu.size()));
        I.rprefix.ensure(rprefix.size());
        if (!ritem_pu.empty()) {
            I.stage.h2d(I.ritem_pu.p, ritem_pu.data(), ritem_pu.size() * 4, I.stream);
            I.stage.h2d(I.rprefix.p, rprefix.data(), rprefix.size() * 8, I.stream);
            times_.h2d_bytes += ritem_pu.size() * 4 + rprefix.size() * 8;
        }
    }
    build_items(active, true);
    // refine_rounds 0: no arc consistency before the search (express patterns still run to their
    // fixpoint below: their domains are their result)
    const int fixed_refine = (int)std::min<uint32_t>(opt.refine_rounds, 32);
    if (!item_pu.empty()) {
        const uint32_t n_it = (uint32_t)item_pu.size();
        const uint64_t words = prefix.back();
        const uint32_t n_rit = (uint32_t)ritem_pu.size();
        const uint64_t rwords = rprefix.back();
        run_captured(I.stream, I.exec_init, [&]() {
            TFSM_CK(record_in_sequence(I.ev0, I.stream));
            TFSM_CK(dev::launch_domain_init(I.g, L.descs.p, I.status.p, I.item_pu.p, I.prefix.p, n_it, words, L.dom.p,
                                            L.found.p, L.failed.p, I.srcs.p, (uint32_t)srcs.size(), total,
                                            I.stream));
            TFSM_CK(record_in_sequence(I.ev_mid, I.stream));
            for (int r = 0; r < fixed_refine; ++r)
                TFSM_CK(dev::launch_refine(I.g, L.descs.p, I.status.p, I.ritem_pu.p, I.rprefix.p, n_rit, rwords,
                                           L.dom.p, total, r, tau, opt.exact, I.stream));
            TFSM_CK(record_in_sequence(I.ev1, I.stream));
        });
        read_status();
        float ms = 0;
        TFSM_CK(cudaEventElapsedTime(&ms, I.ev0, I.ev_mid));
        times_.init_ms += ms;
        TFSM_CK(cudaEventElapsedTime(&ms, I.ev_mid, I.ev1));
        times_.refine_ms += ms;
        times_.init_launches++;
        for (size_t p = 0; p < P; ++p)
            if (active[p])
                for (int u = 0; u < L.hdescs[p].n; ++u) times_.init_words += L.hdescs[p].words[u];
        times_.refine_launches += (uint64_t)fixed_refine;
        times_.refine_words += rwords * (uint64_t)fixed_refine;
    } else {
        read_status();
    }

    // ---- express patterns (distinct labels, acyclic) continue to the arc-consistency fixpoint,
    // whose domains are their MNI domains; one not settled after 32 rounds is searched instead.
    auto viable = [&](size_t p) {
        const PatDesc &D = L.hdescs[p];
        for (int u = 0; u < D.n; ++u) {
            const uint32_t ds = I.hstatus[p].dom_size[u];
            if (opt.exact ? ds == 0 : ds < tau) return false;
        }
        return true;
    };
    int last_round = fixed_refine - 1;
    for (int round = fixed_refine; round < 32; ++round) {
        for (size_t p = 0; p < P; ++p)
            active[p] = !trivial[p] && express[p] && viable(p) &&
                        (round == 0 || ((I.hstatus[p].changed >> (round - 1)) & 1u));
        if (std::find(active.begin(), active.end(), 1) == active.end()) break;
        build_items(active, false);
        TFSM_CK(cudaEventRecord(I.ev0, I.stream));
        TFSM_CK(dev::launch_refine(I.g, L.descs.p, I.status.p, I.item_pu.p, I.prefix.p, (uint32_t)item_pu.size(),
                                   prefix.back(), L.dom.p, total, round, tau, opt.exact, I.stream));
        times_.refine_ms += time_and_read_status();
        times_.refine_launches++;
        times_.refine_words += prefix.back();
        last_round = round;
    }
    if (last_round == 31)
        for (size_t p = 0; p < P; ++p)
            if (express[p] && ((I.hstatus[p].changed >> 31) & 1u)) express[p] = 0;

    phase(2);
    // ---- decisions from domain sizes; plans for the rest ----
    std::vector<char> need_search(P, 0);
    bool any_search = false;
    for (size_t p = 0; p < P; ++p) {
        PatDesc &D = L.hdescs[p];
        EvalResult &r = res[p];
        if (trivial[p]) {
            r.by_filter = true;
            continue;
        }
        const PatStatus &s = I.hstatus[p];
        uint32_t mn = UINT32_MAX;
        for (int u = 0; u < D.n; ++u) mn = std::min(mn, s.dom_size[u]);
        if (express[p]) {
            // an empty domain means no embedding at all; otherwise the arc-consistent domains
            // of a distinct-label tree are its MNI domains
            for (int u = 0; u < D.n; ++u) r.mni[(size_t)u] = mn == 0 ? 0 : s.dom_size[u];
            r.support = mn;
            r.frequent = mn >= tau;
            r.by_filter = true;
            continue;
        }
        if (opt.exact ? mn == 0 : mn < tau) {
            r.by_filter = true;
            continue;
        }
        need_search[p] = 1;
        any_search = true;
        for (int u = 0; u < D.n; ++u)
            if (D.rep[u] == u) {
                uint32_t bn[dev::kMaxN];
                gql_plan(*pats[p], s.dom_size, u, D.order[u], bn);
            }
    }
    if (!any_search) return;

    // ---- matching orders other than GQL (cost model / random for logging); record features ----
    struct Planned {
        uint32_t p;
        int u;
        std::array<float, costmodel::kFeatures> f;
    };
    std::vector<Planned> planned;
    if (opt.order_policy != 0 || opt.records) {
        const auto t_ord = std::chrono::steady_clock::now();
        std::mt19937_64 rng(opt.order_seed * 0x9E3779B97F4A7C15ull + times_.search_calls + 1);
        auto set_order = [](PatDesc &D, int u, const costmodel::Order &o) {
            for (int i = 0; i < D.n; ++i) D.order[u][i] = o[(size_t)i];
        };
        std::vector<float> X;                                       // model inputs, all candidates
        std::vector<std::pair<size_t, size_t>> span;                // per planned entry: [first, count)
        std::vector<std::vector<costmodel::Order>> cands;
        for (size_t p = 0; p < P; ++p) {
            if (!need_search[p]) continue;
            PatDesc &D = L.hdescs[p];
            for (int u = 0; u < D.n; ++u) {
                if (D.rep[u] != u) continue;
                costmodel::Order gq{};
                for (int i = 0; i < D.n; ++i) gq[(size_t)i] = D.order[u][i];
                std::vector<costmodel::Order> cand{gq};  // the GQL order first: it wins ties
                if (opt.order_policy != 0) {
                    std::vector<costmodel::Order> all;
                    costmodel::enumerate_orders(D, u, 128, all);
                    for (auto &o : all)
                        if (o != gq) cand.push_back(o);
                }
                if (opt.order_policy == 1) set_order(D, u, cand[rng() % cand.size()]);
                if (opt.order_policy == 2 && opt.cost_model) {
                    span.emplace_back(X.size() / costmodel::kFeatures, cand.size());
                    for (auto &o : cand) {
                        std::array<float, costmodel::kFeatures> f;
                        costmodel::order_features(D, I.hstatus[p].dom_size, tau, I.label_mean_deg.data(), o, f.data());
                        X.insert(X.end(), f.begin(), f.end());
                    }
                    cands.push_back(std::move(cand));
                }
                planned.push_back({(uint32_t)p, u, {}});
            }
        }
        if (opt.order_policy == 2 && opt.cost_model && !X.empty()) {
            std::vector<float> y(X.size() / costmodel::kFeatures);
            opt.cost_model->predict(X.data(), y.size(), y.data());
            for (size_t k = 0; k < planned.size(); ++k) {
                size_t best = 0;
                for (size_t j = 1; j < span[k].second; ++j)
                    if (y[span[k].first + j] < y[span[k].first + best]) best = j;
                PatDesc &D = L.hdescs[planned[k].p];
                set_order(D, planned[k].u, cands[k][best]);
                // The predicted cost of the chosen order also sets the hub-split span of its searches:
                // searches predicted to take 127 chunk steps or more split a hub's first depth above a
                // quarter of hub_span, searches predicted to take at most 3 never split it.
                const float c = y[span[k].first + best];  // log2(1 + chunk steps per search)
                D.hub_shift[planned[k].u] = c >= 7.f ? (int8_t)-2 : c <= 2.f ? dev::kNoHubSplit : (int8_t)0;
            }
        }
        for (auto &pl : planned) {
            const PatDesc &D = L.hdescs[pl.p];
            costmodel::Order o{};
            for (int i = 0; i < D.n; ++i) o[(size_t)i] = D.order[pl.u][i];
            costmodel::order_features(D, I.hstatus[pl.p].dom_size, tau, I.label_mean_deg.data(), o, pl.f.data());
        }
        times_.order_ms +=
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_ord).count();
    }
    I.stage.h2d(L.descs.p, L.hdescs.data(), P * sizeof(PatDesc), I.stream);
    times_.h2d_bytes += P * sizeof(PatDesc);

    phase(3);
    // ---- search items ----
    // Vertex-major, as the reference evaluates one pattern vertex after another
    // (parallel/comper.h:1181-1239): every pattern first searches its representative with the
    // smallest domain (an infrequent pattern usually dies there), then the next one, whose
    // candidates are by then largely marked found by the earlier embeddings.  Within one rank the
    // chunks of all patterns are interleaved so that every pattern progresses and early exit cuts
    // the rest.
    uint64_t n_items = 0;  // search items of the call (decoded on the device from its groups)
    uint32_t parts_log2 = 0;
    // lanes per search: teams of 8 when asked for, when the call has several patterns to search
    // (single-pattern calls measured faster with whole warps) and every one fits a team's state
    uint32_t team_lanes = 32;
    int max_n = 0, searched_pats = 0;
    for (size_t p = 0; p < P; ++p)
        if (need_search[p]) {
            max_n = std::max(max_n, L.hdescs[p].n);
            ++searched_pats;
        }
    if (opt.search_lanes == 8 && max_n <= 8 && searched_pats > 1) team_lanes = 8;
    // teams of 4 lanes: patterns of at most 5 vertices (at most 4 backward neighbours per depth)
    if (opt.search_lanes == 4 && searched_pats > 1) team_lanes = max_n <= 5 ? 4 : max_n <= 8 ? 8 : 32;
    const uint32_t cw = std::max<uint32_t>(1, opt.chunk_words);
    std::vector<dev::ItemGroup> igroups;
    std::vector<dev::ItemEntry> ientries;
    {
        // The search kernel claims items in order, so the order is the order in time.  With one
        // vertex-major order over a call of hundreds of patterns, a pattern's second vertex waits
        // until the first vertex of every pattern has been searched, although it is often the one
        // that shows the pattern infrequent and would have cut the first vertex's failing
        // searches: windows of `rank_window` patterns bound that wait (vertex-major inside each).
        // One item group per (window, rank): the rank-k representative of each of the window's
        // patterns, whose runs of words are interleaved round by round (dev::item_at).
        std::vector<uint32_t> searched;
        for (size_t p = 0; p < P; ++p)
            if (need_search[p]) searched.push_back((uint32_t)p);
        const size_t win = opt.rank_window ? opt.rank_window : std::max<size_t>(1, searched.size());
        std::vector<std::vector<dev::ItemEntry>> ranks;  // ranks[k]: the k-th smallest representative of each pattern
        for (size_t a = 0; a < searched.size(); a += win) {
            for (auto &r : ranks) r.clear();
            for (size_t i = a; i < std::min(searched.size(), a + win); ++i) {
                const uint32_t p = searched[i];
                const PatDesc &D = L.hdescs[p];
                std::vector<int> reps;
                for (int u = 0; u < D.n; ++u)
                    if (D.rep[u] == u) reps.push_back(u);
                const PatStatus &st = I.hstatus[p];
                std::stable_sort(reps.begin(), reps.end(),
                                 [&](int x, int y) { return st.dom_size[x] < st.dom_size[y]; });
                for (size_t k = 0; k < reps.size(); ++k) {
                    const uint32_t words = D.words[reps[k]];
                    if (!words) continue;
                    if (ranks.size() <= k) ranks.emplace_back();
                    dev::ItemEntry e;
                    std::memset(&e, 0, sizeof(e));
                    e.pat = p;
                    e.u = (uint16_t)reps[k];
                    e.words = words;
                    e.runs = (words + cw - 1) / cw;
                    ranks[k].push_back(e);
                }
            }
            for (auto &es : ranks) {
                if (es.empty()) continue;
                std::stable_sort(es.begin(), es.end(),
                                 [](const dev::ItemEntry &x, const dev::ItemEntry &y) { return x.runs > y.runs; });
                // before[i] = sum over j of min(runs[j], runs[i])
                const size_t m = es.size();
                uint64_t acc = 0;
                for (size_t i = m; i-- > 0;) {
                    const uint32_t below = i + 1 < m ? es[i + 1].runs : 0;
                    acc += (uint64_t)(i + 1) * (es[i].runs - below);
                    es[i].before = acc;
                }
                dev::ItemGroup gr;
                gr.first_item = n_items;
                gr.first_entry = (uint32_t)ientries.size();
                gr.n_entries = (uint32_t)m;
                igroups.push_back(gr);
                ientries.insert(ientries.end(), es.begin(), es.end());
                n_items += es[0].before;
            }
        }
        // Calls with few words (a level of a few patterns) split every item into interleaved parts
        // of its 32 candidates, so that enough warps search in parallel: about four items per
        // resident warp of the search kernel (152 SMs x 40 warps on GB300).
        const uint64_t want = 4ull * (uint64_t)dev::resident_search_warps() * (32u / team_lanes);
        while (parts_log2 < 5 && (n_items << parts_log2) < want) ++parts_log2;
    }
    if (n_items >= (1ull << 32) >> parts_log2) throw EngineError(6, "call has more than 2^32 search items");
    I.igroups.ensure(std::max<size_t>(1, igroups.size()));
    I.ientries.ensure(std::max<size_t>(1, ientries.size()));
    if (!igroups.empty()) {
        I.stage.h2d(I.igroups.p, igroups.data(), igroups.size() * sizeof(dev::ItemGroup), I.stream);
        I.stage.h2d(I.ientries.p, ientries.data(), ientries.size() * sizeof(dev::ItemEntry), I.stream);
    }
    times_.h2d_bytes += igroups.size() * sizeof(dev::ItemGroup) + ientries.size() * sizeof(dev::ItemEntry);
    dev::SearchParams prm;
    std::memset(&prm, 0, sizeof(prm));
    prm.tau = tau;
    prm.exact = opt.exact ? 1 : 0;
    prm.n_items = (uint32_t)n_items;
    prm.n_groups = (uint32_t)igroups.size();
    prm.chunk_words = cw;
    // patterns of more than kTaskMaxN vertices finish every search in place (split tasks hold
    // prefixes of at most kTaskMaxN vertices)
    prm.split = opt.split && opt.step_budget && max_n <= dev::kTaskMaxN ? 1 : 0;
    prm.max_n = (uint32_t)std::max(1, max_n);
    prm.split_slice = std::max<uint32_t>(1, opt.split_slice);
    prm.hub_span = opt.hub_span;
    prm.hub_parts = std::min<uint32_t>(std::max<uint32_t>(1, opt.hub_parts), 32);
    prm.isect_ratio = std::max<uint32_t>(1, opt.isect_ratio);
    prm.split_cap = (uint32_t)(I.splits.n / 2);
    prm.split_slack = prm.split_cap / 8;
    prm.search_fill = prm.split_cap / 2;
    prm.group_cap = (uint32_t)I.groups.n;
    prm.parts_log2 = parts_log2;
    prm.team_lanes = team_lanes;
    prm.n_pats = (uint32_t)P;
    prm.words = total;
    phase(4);
    // Passes.  In each, a search may take `budget` chunk steps before its unexplored remainder
    // becomes split tasks; split rounds then work those off, each task again with a budget (twice
    // the pass's, doubling per round up to 8x after the first `kFixedRounds`, none in the 64th
    // round).  The first rounds are launched with the search as one sequence (a CUDA graph); the
    // host launches further rounds while tasks remain.  Searches and tasks whose remainder found
    // no room are set aside (neither found nor failed) and retried by the next pass with 8x the
    // budgets; in the last pass they finish in place.
    constexpr int kFixedRounds = 2;
    const int n_passes = prm.split ? dev::kMaxPasses : 1;
    uint32_t hcnt[dev::kNumCounters];
    std::memset(hcnt, 0, sizeof(hcnt));
    TFSM_CK(cudaEventRecord(I.ev0, I.stream));
    uint64_t launches = 0;
    for (int pass = 0; pass < n_passes && n_items != 0; ++pass) {
        dev::SearchParams pk = prm;
        pk.step_budget = (uint32_t)std::min<uint64_t>((uint64_t)opt.step_budget << (3 * pass), 1u << 28);
        pk.last = pass + 1 == n_passes ? 1u : 0u;
        const uint32_t round_budget = (uint32_t)std::min<uint64_t>(2ull * pk.step_budget, 1u << 28);
        uint32_t *cnt = I.counters.p + (size_t)pass * dev::kNumCounters;
        const int fixed = prm.split ? kFixedRounds : 0;
        run_captured(I.stream, I.exec_search, [&]() {
            TFSM_CK(cudaMemsetAsync(cnt, 0, dev::kNumCounters * sizeof(uint32_t), I.stream));
            TFSM_CK(dev::launch_search(I.g, L.descs.p, I.status.p, I.igroups.p, I.ientries.p, pk, cnt, L.dom.p,
                                       L.found.p, L.failed.p, I.splits.p, I.groups.p, I.stream));
            for (int r = 0; r < fixed; ++r)
                TFSM_CK(dev::launch_split_round(I.g, L.descs.p, I.status.p, pk, cnt, r, round_budget, L.dom.p,
                                                L.found.p, L.failed.p, I.splits.p, I.groups.p, I.stream));
        });
        launches += 1 + (uint64_t)fixed;
        for (int r = fixed; prm.split && r < dev::kMaxRounds; ++r) {
            uint32_t pending = 0;
            TFSM_CK(cudaMemcpyAsync(&pending, cnt + 2 + r, sizeof(pending), cudaMemcpyDeviceToHost, I.stream));
            TFSM_CK(cudaStreamSynchronize(I.stream));
            times_.d2h_bytes += sizeof(pending);
            if (pending == 0) break;
            const uint32_t budget = round_budget << std::min(r - fixed + 1, 3);
            TFSM_CK(dev::launch_split_round(I.g, L.descs.p, I.status.p, pk, cnt, r, budget, L.dom.p, L.found.p,
                                            L.failed.p, I.splits.p, I.groups.p, I.stream));
            ++launches;
        }
        TFSM_CK(cudaMemcpyAsync(hcnt, cnt, sizeof(hcnt), cudaMemcpyDeviceToHost, I.stream));
        TFSM_CK(cudaStreamSynchronize(I.stream));
        times_.d2h_bytes += sizeof(hcnt);
        times_.search_passes++;
        times_.split_groups += std::min<uint32_t>(hcnt[1], prm.group_cap);
        for (int r = 0; r < dev::kMaxRounds; ++r) times_.split_tasks += std::min(hcnt[2 + r], prm.split_cap);
        times_.abandoned += hcnt[dev::kCntAbandoned];
        if (hcnt[dev::kCntAbandoned] == 0) break;
    }
    TFSM_CK(cudaEventRecord(I.ev1, I.stream));
    land_status();
    {
        float ms = 0;
        TFSM_CK(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
        times_.search_ms += ms;
    }
    times_.search_launches += launches;
    times_.search_calls++;
    {
        unsigned long long rec[4];
        if (dev::read_bounds_check(rec))
            throw EngineError(12, "bounds check failed in the search kernels: site " + std::to_string(rec[1]) +
                                      " index " + std::to_string(rec[2]) + " bound " + std::to_string(rec[3]) +
                                      " (" + std::to_string(rec[0]) + " violations)");
    }

    phase(5);
    if (opt.records)
        for (auto &pl : planned) {
            const PatStatus &s = I.hstatus[pl.p];
            if (!s.searches_u[pl.u]) continue;  // nothing was searched with this order
            opt.records->insert(opt.records->end(), pl.f.begin(), pl.f.end());
            opt.records->push_back(
                (float)std::log2(1.0 + (double)s.steps_u[pl.u] / (double)s.searches_u[pl.u]));
        }

    for (size_t p = 0; p < P; ++p) {
        if (!need_search[p]) continue;
        const PatDesc &D = L.hdescs[p];
        const PatStatus &s = I.hstatus[p];
        EvalResult &r = res[p];
        r.searches = s.searches;
        r.steps = s.steps;
        r.max_steps = s.max_steps;
        times_.search_bytes += s.bytes;
        times_.isects += s.isects;
        uint32_t mn = UINT32_MAX;
        bool all_reps = true;
        for (int u = 0; u < D.n; ++u) {
            r.mni[(size_t)u] = s.found_cnt[u];
            mn = std::min(mn, s.found_cnt[u]);
            if (D.rep[u] == u && s.found_cnt[u] < tau) all_reps = false;
        }
        r.support = mn;
        if (opt.exact) r.frequent = mn >= tau;
        else r.frequent = s.state == dev::kFrequent || (s.state == dev::kRunning && all_reps);
    }
    phase(6);
}

}  // namespace tfsm
