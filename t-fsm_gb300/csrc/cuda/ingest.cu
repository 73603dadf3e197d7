// GPU ingestion of the data graph (what each phase restates: ingest.hpp).
//
// Phases, all on one stream (n input vertices, m input edges, N / M after pruning):
//   .lg only   newline positions (one select over the bytes), per-line kinds and the first
//              malformed line (one thread per line), vertex / edge positions (two scans), values
//   labels     distinct vertex / edge labels with counts (radix sort + run-length encode); the
//              host keeps those with count >= tau (the only round trip before the CSR)
//   prune      dense label per vertex, pruned ids (scan), kept edges and degrees (atomics), kept
//              edge positions (scan)
//   renumber   (label, -degree, pruned id) sort: internal id = label start + the rank's position
//              in the column-major fill of the label's bitmap words
//   CSR        both directions of every kept edge as one (row, neighbour, edge label) key, one
//              radix sort, unpacked into col / elab; row offsets by a scan of the degrees
//   tables     per (vertex, label): first position of the label's neighbours (binary search in the
//              sorted row) and the edge labels present (1-edge pattern endpoint counts, atomics)
// The radix sorts, scans and run-length encodes are CUB's; every other step is a kernel below.
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "cuda/dev_common.cuh"
#include "cuda/ingest.hpp"
#include "cuda/ingest_rules.cuh"
#include "engine.hpp"

namespace tfsm {

DevOwned::~DevOwned() {
    if (p) cudaFree(p);
}

namespace {

#define ING_CK(x)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) throw EngineError(10, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr uint8_t kDrop = 0xff;  // dense label of a pruned vertex or edge
constexpr unsigned long long kNone = ~0ull;

struct Scratch {
    void *p = nullptr;
    Scratch() = default;
    explicit Scratch(size_t bytes) { alloc(bytes); }
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    ~Scratch() {
        if (p) cudaFree(p);
    }
    void alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        ING_CK(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
};

const uint32_t *u32(const DevOwned &o) { return static_cast<const uint32_t *>(o.p); }

void own(DevOwned &o, size_t bytes) {
    if (o.p) cudaFree(o.p);
    o.p = nullptr;
    ING_CK(cudaMalloc(&o.p, std::max<size_t>(bytes, 16)));
    o.bytes = bytes;
}

unsigned grid_for(uint64_t items, unsigned threads = 256) {
    const uint64_t b = (items + threads - 1) / threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 152ull * 16));
}

struct Ctx {
    cudaStream_t s;
    Scratch tmp;
    size_t tmp_bytes = 0;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    std::string *log;
    // a CUB device algorithm: size query, then the run on a temp buffer kept between calls
    template <class F>
    void cub(F f) {
        size_t b = 0;
        ING_CK(f(nullptr, b));
        if (b > tmp_bytes) {
            ING_CK(cudaStreamSynchronize(s));
            tmp.alloc(b);
            tmp_bytes = b;
        }
        ING_CK(f(tmp.p, b));
    }
    template <class T>
    T read(const T *dev) {
        T v;
        ING_CK(cudaMemcpyAsync(&v, dev, sizeof(T), cudaMemcpyDeviceToHost, s));
        ING_CK(cudaStreamSynchronize(s));
        return v;
    }
    void mark(const char *what) {
        const auto now = std::chrono::steady_clock::now();
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%s%s %.2f", log->empty() ? "" : ", ", what,
                      std::chrono::duration<double, std::milli>(now - t).count());
        *log += buf;
        t = now;
    }
};

// ---- .lg text ----------------------------------------------------------------------------------

struct IsNewline {
    const char *buf;
    __host__ __device__ bool operator()(uint64_t i) const { return buf[i] == '\n'; }
};
struct NewlineCount {
    const char *buf;
    __host__ __device__ uint64_t operator()(uint64_t i) const { return buf[i] == '\n' ? 1u : 0u; }
};

template <uint8_t K>
struct KindIs {
    __host__ __device__ uint64_t operator()(uint8_t k) const { return k == K ? 1u : 0u; }
};

__device__ __forceinline__ void line_bounds(const uint64_t *nl, uint64_t k, uint64_t &ls, uint64_t &le) {
    ls = k ? nl[k - 1] + 1 : 0;
    le = nl[k];
}

__global__ void k_line_kinds(const char *__restrict__ buf, uint64_t size, const uint64_t *__restrict__ nl,
                             uint64_t lines, uint8_t *__restrict__ kind, unsigned long long *err_line) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lines; k += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t ls, le;
        line_bounds(nl, k, ls, le);
        const lgparse::Line L = lgparse::parse_line(buf, size, ls, le);
        kind[k] = L.kind;
        if (L.kind >= lgparse::kBadVertex) atomicMin(err_line, (unsigned long long)k);
    }
}

__global__ void k_line_values(const char *__restrict__ buf, uint64_t size, const uint64_t *__restrict__ nl,
                              uint64_t lines, const uint8_t *__restrict__ kind, const uint64_t *__restrict__ vpos,
                              const uint64_t *__restrict__ epos, uint64_t n, int32_t *__restrict__ vlabel,
                              uint32_t *__restrict__ src, uint32_t *__restrict__ dst, int32_t *__restrict__ elab,
                              unsigned long long *bad_vertex, unsigned int *bad_edge) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lines; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t kd = kind[k];
        if (kd != lgparse::kVertex && kd != lgparse::kEdge) continue;
        uint64_t ls, le;
        line_bounds(nl, k, ls, le);
        const lgparse::Line L = lgparse::parse_line(buf, size, ls, le);
        if (kd == lgparse::kVertex) {
            const uint64_t i = vpos[k];
            vlabel[i] = (int32_t)(uint32_t)(uint64_t)L.v[1];
            if (L.v[0] != (int64_t)i) atomicMin(bad_vertex, (unsigned long long)i);
        } else {
            const uint64_t j = epos[k];
            const uint32_t a = (uint32_t)(uint64_t)L.v[0], b = (uint32_t)(uint64_t)L.v[1];
            src[j] = a;
            dst[j] = b;
            elab[j] = (int32_t)(uint32_t)(uint64_t)L.v[2];
            if (a >= n || b >= n) atomicOr(bad_edge, 1u);
        }
    }
}

// the line of vertex `i` (the vertex lines' positions are unique)
__global__ void k_vertex_line(const uint8_t *__restrict__ kind, const uint64_t *__restrict__ vpos, uint64_t lines,
                              uint64_t i, unsigned long long *line) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lines; k += (uint64_t)gridDim.x * blockDim.x)
        if (kind[k] == lgparse::kVertex && vpos[k] == i) *line = k;
}

// ---- edge arrays -------------------------------------------------------------------------------

__global__ void k_check_endpoints(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                                  uint64_t n, unsigned int *bad) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x)
        if (src[k] >= n || dst[k] >= n) atomicOr(bad, 1u);
}

// ---- pruning, renumbering, CSR -----------------------------------------------------------------

// index of `x` in the ascending table, or -1
__device__ __forceinline__ int table_index(const int32_t *__restrict__ t, int nt, int32_t x) {
    int lo = 0, hi = nt;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo < nt && t[lo] == x ? lo : -1;
}

__global__ void k_vertex_dense(const int32_t *__restrict__ vlabel, uint64_t n, const int32_t *__restrict__ freq_v,
                               int nv, uint8_t *__restrict__ dl_in) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int d = table_index(freq_v, nv, vlabel[i]);
        dl_in[i] = d < 0 ? kDrop : (uint8_t)min(d, 254);
    }
}

struct NotDropped {
    __host__ __device__ uint32_t operator()(uint8_t d) const { return d != kDrop ? 1u : 0u; }
};

__global__ void k_vertex_compact(const uint8_t *__restrict__ dl_in, const uint32_t *__restrict__ id_map, uint64_t n,
                                 uint8_t *__restrict__ dl) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (dl_in[i] != kDrop) dl[id_map[i]] = dl_in[i];
}

__global__ void k_edge_keep(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst,
                            const int32_t *__restrict__ elab, uint64_t m, const uint8_t *__restrict__ dl_in,
                            const uint32_t *__restrict__ id_map, const int32_t *__restrict__ freq_e, int ne,
                            uint8_t *__restrict__ edl, uint32_t *__restrict__ deg) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = src[k], b = dst[k];
        const int e = table_index(freq_e, ne, elab[k]);
        const bool keep = e >= 0 && dl_in[a] != kDrop && dl_in[b] != kDrop;
        edl[k] = keep ? (uint8_t)min(e, 254) : kDrop;
        if (keep) {
            atomicAdd(&deg[id_map[a]], 1u);
            atomicAdd(&deg[id_map[b]], 1u);
        }
    }
}

__global__ void k_rank_keys(const uint8_t *__restrict__ dl, const uint32_t *__restrict__ deg, uint32_t n,
                            uint64_t *__restrict__ key, uint32_t *__restrict__ val) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        key[v] = ((uint64_t)dl[v] << 32) | (uint64_t)(~deg[v]);
        val[v] = v;
    }
}

__global__ void k_assign_ids(const uint64_t *__restrict__ key_sorted, const uint32_t *__restrict__ perm, uint32_t n,
                             const uint32_t *__restrict__ lstart, const uint32_t *__restrict__ deg,
                             uint32_t *__restrict__ to_int, uint32_t *__restrict__ deg_int,
                             uint8_t *__restrict__ lab_int) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const uint32_t L = (uint32_t)(key_sorted[s] >> 32);
        const uint32_t v = perm[s];
        const uint32_t x = lstart[L] + rank_to_local(s - lstart[L], lstart[L + 1] - lstart[L]);
        to_int[v] = x;
        deg_int[x] = deg[v];
        lab_int[x] = (uint8_t)L;
    }
}

// (row, neighbour, edge label) packed with `b` bits per vertex id
__global__ void k_entries(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                          const uint8_t *__restrict__ edl, const uint32_t *__restrict__ epos,
                          const uint32_t *__restrict__ id_map, const uint32_t *__restrict__ to_int, int b,
                          uint64_t *__restrict__ key) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t e = edl[k];
        if (e == kDrop) continue;
        const uint64_t x = to_int[id_map[src[k]]], y = to_int[id_map[dst[k]]];
        const uint64_t j = (uint64_t)epos[k] * 2;
        key[j] = (x << (b + 8)) | (y << 8) | e;
        key[j + 1] = (y << (b + 8)) | (x << 8) | e;
    }
}

// Wide ids (b > 28): (row << 32 | neighbour) keys with the edge label as value, sorted in two
// stable passes (edge label, then the key).
__global__ void k_entries_wide(const uint32_t *__restrict__ src, const uint32_t *__restrict__ dst, uint64_t m,
                               const uint8_t *__restrict__ edl, const uint32_t *__restrict__ epos,
                               const uint32_t *__restrict__ id_map, const uint32_t *__restrict__ to_int,
                               uint64_t *__restrict__ key, uint8_t *__restrict__ el) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t e = edl[k];
        if (e == kDrop) continue;
        const uint64_t x = to_int[id_map[src[k]]], y = to_int[id_map[dst[k]]];
        const uint64_t j = (uint64_t)epos[k] * 2;
        key[j] = (x << 32) | y;
        key[j + 1] = (y << 32) | x;
        el[j] = el[j + 1] = e;
    }
}

__global__ void k_unpack(const uint64_t *__restrict__ key, uint64_t m2, int b, uint32_t *__restrict__ col,
                         uint8_t *__restrict__ el) {
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m2; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = key[i];
        col[i] = (uint32_t)((k >> 8) & mask);
        el[i] = (uint8_t)(k & 0xffu);
    }
}

__global__ void k_unpack_wide(const uint64_t *__restrict__ key, uint64_t m2, uint32_t *__restrict__ col) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m2; i += (uint64_t)gridDim.x * blockDim.x)
        col[i] = (uint32_t)key[i];
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *__restrict__ a, uint32_t lo, uint32_t hi,
                                                    uint32_t x) {
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One thread per (label L <= NL, vertex x), x fastest: the label-offset entry (label-major), and
// for L < NL the edge labels of x's neighbours with label L, counted once per (x, edge label, L)
// into the 1-edge pattern cell (min label, edge label, max label) on x's side.
__global__ void k_label_tables(const uint32_t *__restrict__ row_off, const uint32_t *__restrict__ col,
                               const uint8_t *__restrict__ el, uint32_t n, const uint32_t *__restrict__ lstart, int nl,
                               int ne, const uint8_t *__restrict__ lab_int, uint32_t *__restrict__ lab_off,
                               uint32_t *__restrict__ cnt_a, uint32_t *__restrict__ cnt_b) {
    const uint64_t total = (uint64_t)n * ((uint64_t)nl + 1);
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const int L = (int)(t / n);
        const uint32_t x = (uint32_t)(t % n);
        const uint32_t b = row_off[x], e = row_off[x + 1];
        if (L == nl) {
            lab_off[t] = e;
            continue;
        }
        const uint32_t lo = lower_bound_u32(col, b, e, lstart[L]);
        lab_off[t] = lo;
        const uint32_t hi = lower_bound_u32(col, lo, e, lstart[L + 1]);
        if (hi == lo) continue;
        uint32_t mask[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (ne <= 32) {
            for (uint32_t i = lo; i < hi; ++i) mask[0] |= 1u << el[i];
        } else {
            for (uint32_t i = lo; i < hi; ++i) mask[el[i] >> 5] |= 1u << (el[i] & 31);
        }
        const uint32_t la = lab_int[x], lb = (uint32_t)L;
        const bool side_a = la <= lb;
        const uint64_t lo_l = side_a ? la : lb, hi_l = side_a ? lb : la;
        for (int w = 0; w < 8; ++w) {
            uint32_t bits = mask[w];
            while (bits) {
                const int bit = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint64_t cell = (lo_l * (uint64_t)ne + (uint64_t)(w * 32 + bit)) * (uint64_t)nl + hi_l;
                atomicAdd(side_a ? &cnt_a[cell] : &cnt_b[cell], 1u);
            }
        }
    }
}

struct EdgeCell {
    uint64_t cell;
    uint32_t ca, cb;
};

__global__ void k_edge_cells(const uint32_t *__restrict__ cnt_a, const uint32_t *__restrict__ cnt_b, uint64_t cells,
                             int nl, int ne, int64_t tau, EdgeCell *__restrict__ out, unsigned long long *count) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = cnt_a[c], b = cnt_b[c];
        if (!a && !b) continue;
        const uint64_t la = c / ((uint64_t)ne * nl), lb = c % (uint64_t)nl;
        const uint32_t cb = la == lb ? a : b;
        if ((int64_t)a >= tau && (int64_t)cb >= tau) out[atomicAdd(count, 1ull)] = EdgeCell{c, a, cb};
    }
}

int id_bits(uint32_t n) {
    int b = 1;
    while (b < 32 && ((uint64_t)1 << b) < (uint64_t)n) ++b;
    return b;
}

// The pruned graph of device arrays vlabel [n_in], src / dst / elab [m_in] (endpoints checked).
void build_graph(Ctx &C, const int32_t *vlabel, uint64_t n_in, const uint32_t *src, const uint32_t *dst,
                 const int32_t *elab, uint64_t m_in, int tau, DeviceGraphBuild &out) {
    cudaStream_t s = C.s;
    LgGraph &g = out.summary;
    g.input_vertices = n_in;
    g.input_edges = m_in;
    if (m_in >= (1ull << 32)) throw LgError(5, "more than 2^32 - 1 edges");
    const uint64_t need = (uint64_t)std::max(tau, 0);
    // ---- distinct labels with counts ----
    auto distinct = [&](const int32_t *in, uint64_t cnt, std::vector<int> &vals, std::vector<uint32_t> &counts) {
        vals.clear();
        counts.clear();
        if (!cnt) return;
        Scratch sorted(cnt * 4), uniq(cnt * 4), num(cnt * 4), runs(8);
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceRadixSort::SortKeys(t, b, in, sorted.as<int32_t>(), (int64_t)cnt, 0, 32, s);
        });
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceRunLengthEncode::Encode(t, b, sorted.as<int32_t>(), uniq.as<int32_t>(),
                                                      num.as<uint32_t>(), runs.as<uint64_t>(), (int64_t)cnt, s);
        });
        const uint64_t r = C.read(runs.as<uint64_t>());
        vals.resize(r);
        counts.resize(r);
        ING_CK(cudaMemcpyAsync(vals.data(), uniq.p, r * 4, cudaMemcpyDeviceToHost, s));
        ING_CK(cudaMemcpyAsync(counts.data(), num.p, r * 4, cudaMemcpyDeviceToHost, s));
        ING_CK(cudaStreamSynchronize(s));
    };
    std::vector<int> vl, ell;
    std::vector<uint32_t> vc, ec;
    distinct(vlabel, n_in, vl, vc);
    distinct(elab, m_in, ell, ec);
    std::vector<uint32_t> fcount;  // vertices per frequent vertex label
    for (size_t k = 0; k < vl.size(); ++k)
        if (vc[k] >= need) {
            g.freq_vlabels.push_back(vl[k]);
            fcount.push_back(vc[k]);
            g.max_label_freq = std::max(g.max_label_freq, vc[k]);
        }
    for (size_t k = 0; k < ell.size(); ++k)
        if (ec[k] >= need) g.freq_elabels.push_back(ell[k]);
    const int NL = (int)g.freq_vlabels.size(), NE = (int)g.freq_elabels.size();
    C.mark("labels");
    // ---- pruning ----
    Scratch freq_v((size_t)NL * 4), freq_e((size_t)NE * 4);
    if (NL) ING_CK(cudaMemcpyAsync(freq_v.p, g.freq_vlabels.data(), (size_t)NL * 4, cudaMemcpyHostToDevice, s));
    if (NE) ING_CK(cudaMemcpyAsync(freq_e.p, g.freq_elabels.data(), (size_t)NE * 4, cudaMemcpyHostToDevice, s));
    out.h2d_bytes += (uint64_t)(NL + NE) * 4;
    Scratch dl_in(n_in), id_map((n_in + 1) * 4);
    uint32_t n = 0;
    if (n_in) {
        k_vertex_dense<<<grid_for(n_in), 256, 0, s>>>(vlabel, n_in, freq_v.as<int32_t>(), NL, dl_in.as<uint8_t>());
        ING_CK(cudaGetLastError());
        auto kept = thrust::make_transform_iterator(dl_in.as<uint8_t>(), NotDropped());
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceScan::ExclusiveSum(t, b, kept, id_map.as<uint32_t>(), (int64_t)n_in, s);
        });
        const uint32_t last = C.read(id_map.as<uint32_t>() + n_in - 1);
        const uint8_t last_dl = C.read(dl_in.as<uint8_t>() + n_in - 1);
        n = last + (last_dl != kDrop ? 1u : 0u);
    }
    g.n = n;
    Scratch dl((size_t)n + 1), deg(((size_t)n + 1) * 4);
    ING_CK(cudaMemsetAsync(deg.p, 0, ((size_t)n + 1) * 4, s));
    if (n_in) {
        k_vertex_compact<<<grid_for(n_in), 256, 0, s>>>(dl_in.as<uint8_t>(), id_map.as<uint32_t>(), n_in, dl.as<uint8_t>());
        ING_CK(cudaGetLastError());
    }
    Scratch edl(m_in), epos((m_in + 1) * 4);
    uint64_t m = 0;
    if (m_in) {
        k_edge_keep<<<grid_for(m_in), 256, 0, s>>>(src, dst, elab, m_in, dl_in.as<uint8_t>(), id_map.as<uint32_t>(),
                                                   freq_e.as<int32_t>(), NE, edl.as<uint8_t>(), deg.as<uint32_t>());
        ING_CK(cudaGetLastError());
        auto kept = thrust::make_transform_iterator(edl.as<uint8_t>(), NotDropped());
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceScan::ExclusiveSum(t, b, kept, epos.as<uint32_t>(), (int64_t)m_in, s);
        });
        const uint32_t last = C.read(epos.as<uint32_t>() + m_in - 1);
        const uint8_t last_e = C.read(edl.as<uint8_t>() + m_in - 1);
        m = (uint64_t)last + (last_e != kDrop ? 1u : 0u);
    }
    g.m = m;
    const uint64_t m2 = 2 * m;
    // the engine's limits, in the order its host-built path checks them
    if (m2 >= (1ull << 32)) throw EngineError(5, "graph has >= 2^32 adjacency entries");
    if (NE > 250) throw EngineError(5, "more than 250 frequent edge labels");
    if (NL > 250) throw EngineError(5, "more than 250 frequent vertex labels");
    const uint64_t stride = (uint64_t)NL + 1;
    if ((uint64_t)n * stride >= (1ull << 34)) throw EngineError(5, "label-offset table too large");
    C.mark("prune");
    // ---- label-grouped, degree-ranked internal ids ----
    out.lstart.assign((size_t)NL + 1, 0);
    for (int L = 0; L < NL; ++L) out.lstart[(size_t)L + 1] = out.lstart[(size_t)L] + fcount[(size_t)L];
    own(out.label_start, stride * 4);
    ING_CK(cudaMemcpyAsync(out.label_start.p, out.lstart.data(), stride * 4, cudaMemcpyHostToDevice, s));
    out.h2d_bytes += stride * 4;
    Scratch key_v((size_t)n * 8), key_s((size_t)n * 8), val_v((size_t)n * 4), perm((size_t)n * 4);
    Scratch to_int((size_t)n * 4), deg_int(((size_t)n + 1) * 4), lab_int((size_t)n + 1);
    ING_CK(cudaMemsetAsync(deg_int.p, 0, ((size_t)n + 1) * 4, s));
    if (n) {
        k_rank_keys<<<grid_for(n), 256, 0, s>>>(dl.as<uint8_t>(), deg.as<uint32_t>(), n, key_v.as<uint64_t>(),
                                                val_v.as<uint32_t>());
        ING_CK(cudaGetLastError());
        int lbits = 1;
        while ((1 << lbits) < NL) ++lbits;
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceRadixSort::SortPairs(t, b, key_v.as<uint64_t>(), key_s.as<uint64_t>(), val_v.as<uint32_t>(),
                                                   perm.as<uint32_t>(), (int64_t)n, 0, 32 + lbits, s);
        });
        k_assign_ids<<<grid_for(n), 256, 0, s>>>(key_s.as<uint64_t>(), perm.as<uint32_t>(), n,
                                                 u32(out.label_start), deg.as<uint32_t>(), to_int.as<uint32_t>(),
                                                 deg_int.as<uint32_t>(), lab_int.as<uint8_t>());
        ING_CK(cudaGetLastError());
    }
    // per-label degree sums (2m < 2^32 bounds every sum) and the largest degree
    std::vector<uint32_t> dsum((size_t)NL, 0);
    Scratch dsum_d((size_t)NL * 4 + 4), maxdeg(4);
    if (n) {
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceSegmentedReduce::Sum(t, b, deg_int.as<uint32_t>(), dsum_d.as<uint32_t>(), (int64_t)NL,
                                                   u32(out.label_start), u32(out.label_start) + 1, s);
        });
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceReduce::Max(t, b, deg_int.as<uint32_t>(), maxdeg.as<uint32_t>(), (int64_t)n, s);
        });
        ING_CK(cudaMemcpyAsync(dsum.data(), dsum_d.p, (size_t)NL * 4, cudaMemcpyDeviceToHost, s));
        g.max_degree = C.read(maxdeg.as<uint32_t>());
    }
    out.label_mean_deg.assign((size_t)NL, 0.f);
    for (int L = 0; L < NL; ++L)
        if (fcount[(size_t)L]) out.label_mean_deg[(size_t)L] = (float)((double)dsum[(size_t)L] / fcount[(size_t)L]);
    // ---- CSR: row offsets, then the sorted (row, neighbour, edge label) entries ----
    own(out.row_off, ((size_t)n + 1) * 4);
    C.cub([&](void *t, size_t &b) {
        return cub::DeviceScan::ExclusiveSum(t, b, deg_int.as<uint32_t>(), (uint32_t *)out.row_off.p, (int64_t)n + 1, s);
    });
    own(out.col, (m2 + dev::kColPad) * 4);
    own(out.elab, m2);
    ING_CK(cudaMemsetAsync((uint32_t *)out.col.p + m2, 0xff, dev::kColPad * 4, s));
    out.m2 = m2;
    C.mark("renumber");
    if (m2) {
        const int b = id_bits(n);
        Scratch keys(m2 * 8), keys2(m2 * 8);
        // TFSM_INGEST_WIDE_IDS=1 takes the two-pass sort of graphs over 2^28 vertices on any graph
        // (tests compare both forms)
        const char *wide_env = std::getenv("TFSM_INGEST_WIDE_IDS");
        const bool wide = 2 * b + 8 > 64 || (wide_env && wide_env[0] == '1');
        if (!wide) {
            k_entries<<<grid_for(m_in), 256, 0, s>>>(src, dst, m_in, edl.as<uint8_t>(), epos.as<uint32_t>(),
                                                     id_map.as<uint32_t>(), to_int.as<uint32_t>(), b,
                                                     keys.as<uint64_t>());
            ING_CK(cudaGetLastError());
            C.cub([&](void *t, size_t &bb) {
                return cub::DeviceRadixSort::SortKeys(t, bb, keys.as<uint64_t>(), keys2.as<uint64_t>(), (int64_t)m2, 0,
                                                      2 * b + 8, s);
            });
            k_unpack<<<grid_for(m2), 256, 0, s>>>(keys2.as<uint64_t>(), m2, b, (uint32_t *)out.col.p,
                                                  (uint8_t *)out.elab.p);
            ING_CK(cudaGetLastError());
        } else {
            Scratch el1(m2), el2(m2);
            k_entries_wide<<<grid_for(m_in), 256, 0, s>>>(src, dst, m_in, edl.as<uint8_t>(), epos.as<uint32_t>(),
                                                          id_map.as<uint32_t>(), to_int.as<uint32_t>(),
                                                          keys.as<uint64_t>(), el1.as<uint8_t>());
            ING_CK(cudaGetLastError());
            // stable passes: by edge label, then by (row, neighbour)
            C.cub([&](void *t, size_t &bb) {
                return cub::DeviceRadixSort::SortPairs(t, bb, el1.as<uint8_t>(), el2.as<uint8_t>(), keys.as<uint64_t>(),
                                                       keys2.as<uint64_t>(), (int64_t)m2, 0, 8, s);
            });
            C.cub([&](void *t, size_t &bb) {
                return cub::DeviceRadixSort::SortPairs(t, bb, keys2.as<uint64_t>(), keys.as<uint64_t>(), el2.as<uint8_t>(),
                                                       (uint8_t *)out.elab.p, (int64_t)m2, 0, 64, s);
            });
            k_unpack_wide<<<grid_for(m2), 256, 0, s>>>(keys.as<uint64_t>(), m2, (uint32_t *)out.col.p);
            ING_CK(cudaGetLastError());
        }
        ING_CK(cudaStreamSynchronize(s));
    }
    C.mark("csr");
    // ---- label offsets and 1-edge pattern endpoint counts ----
    own(out.lab_off, (size_t)n * stride * 4);
    const uint64_t cells = (uint64_t)NL * (uint64_t)NE * (uint64_t)NL;
    Scratch cnt_a(cells * 4), cnt_b(cells * 4);
    if (cells) {
        ING_CK(cudaMemsetAsync(cnt_a.p, 0, cells * 4, s));
        ING_CK(cudaMemsetAsync(cnt_b.p, 0, cells * 4, s));
    }
    if (n) {
        k_label_tables<<<grid_for((uint64_t)n * stride), 256, 0, s>>>(
            (const uint32_t *)out.row_off.p, (const uint32_t *)out.col.p, (const uint8_t *)out.elab.p, n,
            u32(out.label_start), NL, NE, lab_int.as<uint8_t>(), (uint32_t *)out.lab_off.p, cnt_a.as<uint32_t>(),
            cnt_b.as<uint32_t>());
        ING_CK(cudaGetLastError());
    }
    if (cells) {
        Scratch cell_out(cells * sizeof(EdgeCell)), ncell(8);
        ING_CK(cudaMemsetAsync(ncell.p, 0, 8, s));
        k_edge_cells<<<grid_for(cells), 256, 0, s>>>(cnt_a.as<uint32_t>(), cnt_b.as<uint32_t>(), cells, NL, NE,
                                                     (int64_t)tau, cell_out.as<EdgeCell>(),
                                                     ncell.as<unsigned long long>());
        ING_CK(cudaGetLastError());
        const uint64_t k = C.read(ncell.as<unsigned long long>());
        std::vector<EdgeCell> hc(k);
        if (k) ING_CK(cudaMemcpyAsync(hc.data(), cell_out.p, k * sizeof(EdgeCell), cudaMemcpyDeviceToHost, s));
        ING_CK(cudaStreamSynchronize(s));
        std::sort(hc.begin(), hc.end(), [](const EdgeCell &a, const EdgeCell &b) { return a.cell < b.cell; });
        for (const EdgeCell &c : hc) {
            const size_t la = (size_t)(c.cell / ((uint64_t)NE * NL)), el = (size_t)((c.cell / NL) % NE),
                         lb = (size_t)(c.cell % NL);
            g.edge_pairs.push_back({g.freq_vlabels[la], g.freq_elabels[el], g.freq_vlabels[lb], c.ca, c.cb});
        }
    }
    ING_CK(cudaStreamSynchronize(s));
    C.mark("tables");
}

// The file's bytes, mapped read-only (a private mapping of the page cache).
struct MappedFile {
    int fd = -1;
    void *p = nullptr;
    size_t size = 0;
    ~MappedFile() {
        if (p) munmap(p, size);
        if (fd >= 0) close(fd);
    }
};

}  // namespace

void ingest_lg_file(const std::string &path, int tau, CUstream_st *stream, DeviceGraphBuild &out) {
    Ctx C{stream};
    C.log = &out.breakdown;
    MappedFile f;
    f.fd = open(path.c_str(), O_RDONLY);
    if (f.fd < 0) throw LgError(2, "cannot open graph file " + path);
    struct stat st;
    if (fstat(f.fd, &st) != 0) throw LgError(2, "cannot open graph file " + path);
    f.size = (size_t)st.st_size;
    if (f.size) {
        f.p = mmap(nullptr, f.size, PROT_READ, MAP_PRIVATE | MAP_POPULATE, f.fd, 0);
        if (f.p == MAP_FAILED) {
            f.p = nullptr;
            throw LgError(2, "cannot read graph file " + path);
        }
    }
    cudaStream_t s = C.s;
    // the bytes plus a final newline (the host loader appends one as well)
    const uint64_t size = f.size + 1;
    Scratch buf(size);
    if (f.size) ING_CK(cudaMemcpyAsync(buf.p, f.p, f.size, cudaMemcpyHostToDevice, s));
    out.h2d_bytes += f.size;
    ING_CK(cudaMemsetAsync(buf.as<char>() + f.size, '\n', 1, s));
    C.mark("read+copy");
    // newline positions = line ends
    Scratch nl, nlines(8);
    {
        // count first to size the position array
        uint64_t lines = 0;
        {
            Scratch cnt(8);
            auto flags = thrust::make_transform_iterator(thrust::counting_iterator<uint64_t>(0),
                                                         NewlineCount{buf.as<char>()});
            C.cub([&](void *t, size_t &b) {
                return cub::DeviceReduce::Sum(t, b, flags, cnt.as<uint64_t>(), (int64_t)size, s);
            });
            lines = C.read(cnt.as<uint64_t>());
        }
        nl.alloc(lines * 8);
        C.cub([&](void *t, size_t &b) {
            return cub::DeviceSelect::If(t, b, thrust::counting_iterator<uint64_t>(0), nl.as<uint64_t>(),
                                         nlines.as<uint64_t>(), (int64_t)size, IsNewline{buf.as<char>()}, s);
        });
    }
    const uint64_t lines = C.read(nlines.as<uint64_t>());
    Scratch kind(lines), vpos(lines * 8), epos(lines * 8), err(8);
    ING_CK(cudaMemsetAsync(err.p, 0xff, 8, s));
    k_line_kinds<<<grid_for(lines), 256, 0, s>>>(buf.as<char>(), size, nl.as<uint64_t>(), lines, kind.as<uint8_t>(),
                                                  err.as<unsigned long long>());
    ING_CK(cudaGetLastError());
    const unsigned long long bad_line = C.read(err.as<unsigned long long>());
    if (bad_line != kNone) {
        const uint8_t k = C.read(kind.as<uint8_t>() + bad_line);
        const std::string what = k == lgparse::kBadVertex ? "malformed vertex line "
                                 : k == lgparse::kBadEdge ? "malformed edge line "
                                                          : "unknown line kind at line ";
        throw LgError(3, what + std::to_string(bad_line + 1));
    }
    auto is_v = thrust::make_transform_iterator(kind.as<uint8_t>(), KindIs<lgparse::kVertex>());
    auto is_e = thrust::make_transform_iterator(kind.as<uint8_t>(), KindIs<lgparse::kEdge>());
    C.cub([&](void *t, size_t &b) { return cub::DeviceScan::ExclusiveSum(t, b, is_v, vpos.as<uint64_t>(), (int64_t)lines, s); });
    C.cub([&](void *t, size_t &b) { return cub::DeviceScan::ExclusiveSum(t, b, is_e, epos.as<uint64_t>(), (int64_t)lines, s); });
    const uint8_t last_kind = C.read(kind.as<uint8_t>() + lines - 1);
    const uint64_t n_in = C.read(vpos.as<uint64_t>() + lines - 1) + (last_kind == lgparse::kVertex ? 1 : 0);
    const uint64_t m_in = C.read(epos.as<uint64_t>() + lines - 1) + (last_kind == lgparse::kEdge ? 1 : 0);
    if (n_in >= (1ull << 32)) throw LgError(5, "more than 2^32 - 1 vertices");
    Scratch vlabel(n_in * 4), src(m_in * 4), dst(m_in * 4), elab(m_in * 4), bad_v(8), bad_e(4);
    ING_CK(cudaMemsetAsync(bad_v.p, 0xff, 8, s));
    ING_CK(cudaMemsetAsync(bad_e.p, 0, 4, s));
    k_line_values<<<grid_for(lines), 256, 0, s>>>(buf.as<char>(), size, nl.as<uint64_t>(), lines, kind.as<uint8_t>(),
                                                  vpos.as<uint64_t>(), epos.as<uint64_t>(), n_in, vlabel.as<int32_t>(),
                                                  src.as<uint32_t>(), dst.as<uint32_t>(), elab.as<int32_t>(),
                                                  bad_v.as<unsigned long long>(), bad_e.as<unsigned int>());
    ING_CK(cudaGetLastError());
    const unsigned long long bad_vertex = C.read(bad_v.as<unsigned long long>());
    if (bad_vertex != kNone) {
        // the message names the line's id: find the vertex's line and parse it here
        Scratch line(8);
        k_vertex_line<<<grid_for(lines), 256, 0, s>>>(kind.as<uint8_t>(), vpos.as<uint64_t>(), lines, bad_vertex,
                                                       line.as<unsigned long long>());
        ING_CK(cudaGetLastError());
        const uint64_t k = C.read(line.as<unsigned long long>());
        const uint64_t le = C.read(nl.as<uint64_t>() + k);
        const uint64_t ls = k ? C.read(nl.as<uint64_t>() + k - 1) + 1 : 0;
        // le < f.size: the line's newline is one of the file's own (a vertex line is never the
        // appended last line unless the file lacks a final newline; then le == f.size)
        std::string text((const char *)f.p + ls, (const char *)f.p + std::min<uint64_t>(le, f.size));
        text.push_back('\n');
        const lgparse::Line L = lgparse::parse_line(text.data(), text.size(), 0, text.size() - 1);
        throw LgError(3, "vertex ids must be 0..N-1 in order (line for id " + std::to_string(L.v[0]) + ")");
    }
    if (C.read(bad_e.as<unsigned int>())) throw LgError(3, "edge endpoint out of range");
    C.mark("parse");
    build_graph(C, vlabel.as<int32_t>(), n_in, src.as<uint32_t>(), dst.as<uint32_t>(), elab.as<int32_t>(), m_in, tau,
                out);
}

void ingest_edge_arrays(uint32_t n, const int32_t *vlabel, uint64_t m, const uint32_t *src, const uint32_t *dst,
                        const int32_t *elabel, int tau, CUstream_st *stream, DeviceGraphBuild &out) {
    Ctx C{stream};
    C.log = &out.breakdown;
    cudaStream_t s = C.s;
    Scratch dv((size_t)n * 4), ds(m * 4), dd(m * 4), de(m * 4), bad(4);
    if (n) ING_CK(cudaMemcpyAsync(dv.p, vlabel, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    if (m) {
        ING_CK(cudaMemcpyAsync(ds.p, src, m * 4, cudaMemcpyHostToDevice, s));
        ING_CK(cudaMemcpyAsync(dd.p, dst, m * 4, cudaMemcpyHostToDevice, s));
        ING_CK(cudaMemcpyAsync(de.p, elabel, m * 4, cudaMemcpyHostToDevice, s));
    }
    out.h2d_bytes += (uint64_t)n * 4 + m * 12;
    ING_CK(cudaMemsetAsync(bad.p, 0, 4, s));
    if (m) {
        k_check_endpoints<<<grid_for(m), 256, 0, s>>>(ds.as<uint32_t>(), dd.as<uint32_t>(), m, n, bad.as<unsigned int>());
        ING_CK(cudaGetLastError());
    }
    if (C.read(bad.as<unsigned int>())) throw LgError(3, "edge endpoint out of range");
    C.mark("copy");
    build_graph(C, dv.as<int32_t>(), n, ds.as<uint32_t>(), dd.as<uint32_t>(), de.as<int32_t>(), m, tau, out);
}

}  // namespace tfsm
