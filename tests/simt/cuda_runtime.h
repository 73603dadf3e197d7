// TEST INFRASTRUCTURE ONLY — host-side SIMT emulation of the CUDA subset used by the kernels of
// t-fsm_gb300/csrc/cuda/kernels.cu and the engine, so that the exact kernel sources can run on the
// CPU under AddressSanitizer / UndefinedBehaviorSanitizer / ThreadSanitizer.
//
// Model: a launch runs its blocks, and the warps of a block, one after another on 32 persistent workers;
// each group of 32 threads is a warp whose collectives (__syncwarp, __ballot_sync, __any_sync,
// __shfl_sync, __shfl_xor_sync, __reduce_add_sync) are rendezvous on a std::barrier, which also
// orders memory like bar.warp.sync.  __shared__ variables become static storage (one block at a
// time).  Atomics are GCC __atomic builtins; __ldcg is a relaxed atomic load.  Device memory is
// host memory.  Masks: the full warp, or an aligned group of 4, 8 or 16 lanes (a team of lanes that
// runs its own search); each group has its own rendezvous, so groups of a warp proceed independently.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__ static
#define __align__(n) __attribute__((aligned(n)))

struct dim3 {
    unsigned x = 1, y = 1, z = 1;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

namespace tfsm_emu {

// Warp rendezvous (sense-reversing, spin + yield) with a watchdog: a lane that waits more than
// 20 s reports, per lane, the source line of the collective it is blocked in (divergent
// collectives are a kernel bug).
struct Barrier {
    std::atomic<unsigned> arrived{0};
    std::atomic<unsigned long long> generation{0};
    std::atomic<int> line[32];
    unsigned count = 32;  // lanes that meet here
    Barrier() {
        for (auto &l : line) l.store(0);
    }
    void arrive_and_wait(unsigned lane, int at) {
        line[lane].store(at, std::memory_order_relaxed);
        const unsigned long long gen = generation.load(std::memory_order_acquire);
        if (arrived.fetch_add(1, std::memory_order_acq_rel) == count - 1) {
            arrived.store(0, std::memory_order_relaxed);
            generation.fetch_add(1, std::memory_order_acq_rel);
            return;
        }
        const auto t0 = std::chrono::steady_clock::now();
        unsigned spins = 0;
        while (generation.load(std::memory_order_acquire) == gen) {
            if (++spins > 64) {
                std::this_thread::yield();
                if ((spins & 0xffff) == 0 &&
                    std::chrono::steady_clock::now() - t0 > std::chrono::seconds(20)) {
                    std::fprintf(stderr, "emulation: warp collective deadlock; lane:line =");
                    for (unsigned l = 0; l < 32; ++l) std::fprintf(stderr, " %u:%d", l, line[l].load());
                    std::fprintf(stderr, "\n");
                    std::abort();
                }
            }
        }
    }
};

struct Warp {
    Barrier bar;
    Barrier g4[8], g8[4], g16[2];  // aligned lane groups
    uint64_t vals[32];
    Warp() {
        for (auto &b : g4) b.count = 4;
        for (auto &b : g8) b.count = 8;
        for (auto &b : g16) b.count = 16;
    }
    Barrier &of(unsigned mask) {
        if (mask == 0xffffffffu) return bar;
        const unsigned base = (unsigned)__builtin_ctz(mask), size = (unsigned)__builtin_popcount(mask);
        const bool aligned = (size == 4 || size == 8 || size == 16) && base % size == 0 &&
                             mask == (((1u << size) - 1) << base);
        if (!aligned) {
            std::fprintf(stderr, "emulation: unsupported collective mask %08x\n", mask);
            std::abort();
        }
        return size == 4 ? g4[base / 4] : size == 8 ? g8[base / 8] : g16[base / 16];
    }
};

inline thread_local dim3 tl_threadIdx, tl_blockIdx;
inline dim3 g_blockDim, g_gridDim;
inline thread_local Warp *tl_warp = nullptr;

// Persistent workers: thread t of every emulated block runs on worker t.
struct Pool {
    std::vector<std::thread> th;
    std::mutex mu;
    std::condition_variable cv_go, cv_done;
    std::function<void(unsigned)> job;
    unsigned active = 0, remaining = 0;
    unsigned long long epoch = 0;
    bool quit = false;
    explicit Pool(unsigned n) {
        for (unsigned i = 0; i < n; ++i)
            th.emplace_back([this, i]() {
                unsigned long long seen = 0;
                for (;;) {
                    std::function<void(unsigned)> j;
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv_go.wait(lk, [&] { return quit || epoch != seen; });
                        if (quit) return;
                        seen = epoch;
                        if (i >= active) continue;
                        j = job;
                    }
                    j(i);
                    std::lock_guard<std::mutex> lk(mu);
                    if (--remaining == 0) cv_done.notify_all();
                }
            });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv_go.notify_all();
        for (auto &t : th) t.join();
    }
    void run(unsigned n, std::function<void(unsigned)> f) {
        std::unique_lock<std::mutex> lk(mu);
        job = std::move(f);
        active = remaining = n;
        ++epoch;
        cv_go.notify_all();
        cv_done.wait(lk, [&] { return remaining == 0; });
    }
};

inline Pool &pool() {
    static Pool p(32);
    return p;
}

template <class F>
void launch(unsigned grid, unsigned block, F &&fn) {
    if (block % 32 != 0 || block > 1024) {
        std::fprintf(stderr, "emulation: block size must be a multiple of 32, at most 1024\n");
        std::abort();
    }
    g_gridDim = dim3(grid);
    g_blockDim = dim3(block);
    static const bool trace = std::getenv("TFSM_EMU_TRACE") != nullptr;
    if (trace) std::fprintf(stderr, "emu launch grid %u block %u\n", grid, block);
    // The kernels never make one warp wait for another (warps share only global atomics and
    // their own shared-memory slots), so the warps of a block may run one after another.
    Warp warp;
    for (unsigned b = 0; b < grid; ++b) {
        for (unsigned w = 0; w < block / 32; ++w) {
            pool().run(32, [&, b, w](unsigned t) {
                tl_threadIdx = dim3(w * 32 + t);
                tl_blockIdx = dim3(b);
                tl_warp = &warp;
                fn();
            });
        }
    }
}

inline unsigned lane() { return tl_threadIdx.x & 31; }

// the lanes of `mask` publish a value, then read the published values
template <class R>
R collective(unsigned mask, uint64_t mine, R (*combine)(const uint64_t *, unsigned, unsigned, uint64_t), uint64_t arg,
             int at) {
    Warp &w = *tl_warp;
    Barrier &b = w.of(mask);
    w.vals[lane()] = mine;
    b.arrive_and_wait(lane(), at);
    R r = combine(w.vals, lane(), mask, arg);
    b.arrive_and_wait(lane(), -at);
    return r;
}

}  // namespace tfsm_emu

#define threadIdx (tfsm_emu::tl_threadIdx)
#define blockIdx (tfsm_emu::tl_blockIdx)
#define blockDim (tfsm_emu::g_blockDim)
#define gridDim (tfsm_emu::g_gridDim)

inline void __syncwarp(unsigned mask = 0xffffffffu, int at = __builtin_LINE()) {
    tfsm_emu::tl_warp->of(mask).arrive_and_wait(tfsm_emu::lane(), at);
}

inline unsigned __ballot_sync(unsigned mask, int pred, int at = __builtin_LINE()) {
    return tfsm_emu::collective<unsigned>(
        mask, pred ? 1u : 0u,
        [](const uint64_t *v, unsigned, unsigned m, uint64_t) -> unsigned {
            unsigned r = 0;
            for (unsigned l = 0; l < 32; ++l)
                if (((m >> l) & 1u) && v[l]) r |= 1u << l;
            return r;
        },
        0, at);
}

inline int __any_sync(unsigned m, int pred, int at = __builtin_LINE()) { return __ballot_sync(m, pred, at) != 0; }

// Source lanes follow CUDA: `src` (or lane ^ laneMask) inside the caller's segment of `width`
// lanes.  The argument packs (width << 8 | src).
template <class T>
T __shfl_sync(unsigned mask, T v, int src, int width = 32, int at = __builtin_LINE()) {
    static_assert(sizeof(T) <= 8, "shuffle of at most 8 bytes");
    uint64_t bits = 0;
    std::memcpy(&bits, &v, sizeof(T));
    const uint64_t got = tfsm_emu::collective<uint64_t>(
        mask, bits,
        [](const uint64_t *vals, unsigned ln, unsigned, uint64_t a) -> uint64_t {
            const unsigned w = (unsigned)(a >> 8), s = (unsigned)(a & 0xff);
            return vals[(ln & ~(w - 1)) + (s & (w - 1))];
        },
        ((uint64_t)width << 8) | (uint64_t)(src & 0xff), at);
    T r;
    std::memcpy(&r, &got, sizeof(T));
    return r;
}

template <class T>
T __shfl_xor_sync(unsigned mask, T v, int lane_mask, int width = 32, int at = __builtin_LINE()) {
    uint64_t bits = 0;
    std::memcpy(&bits, &v, sizeof(T));
    const uint64_t got = tfsm_emu::collective<uint64_t>(
        mask, bits,
        [](const uint64_t *vals, unsigned ln, unsigned, uint64_t a) -> uint64_t {
            const unsigned w = (unsigned)(a >> 8), m = (unsigned)(a & 0xff);
            const unsigned t = ln ^ m;
            return vals[((t & ~(w - 1)) == (ln & ~(w - 1))) ? t : ln];
        },
        ((uint64_t)width << 8) | (uint64_t)(lane_mask & 0xff), at);
    T r;
    std::memcpy(&r, &got, sizeof(T));
    return r;
}

inline unsigned __reduce_add_sync(unsigned mask, unsigned v, int at = __builtin_LINE()) {
    return tfsm_emu::collective<unsigned>(
        mask, v,
        [](const uint64_t *vals, unsigned, unsigned m, uint64_t) -> unsigned {
            unsigned s = 0;
            for (unsigned l = 0; l < 32; ++l)
                if ((m >> l) & 1u) s += (unsigned)vals[l];
            return s;
        },
        0, at);
}

inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
struct alignas(16) uint4 {
    unsigned x, y, z, w;
};
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }

template <class T>
inline T __ldg(const T *p) {
    return *p;
}
template <class T>
inline T __ldcg(const T *p) {
    return __atomic_load_n(p, __ATOMIC_RELAXED);
}
inline void __threadfence() { std::atomic_thread_fence(std::memory_order_seq_cst); }

inline unsigned atomicAdd(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v) {
    return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}
inline unsigned atomicSub(unsigned *p, unsigned v) { return __atomic_fetch_sub(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicOr(unsigned *p, unsigned v) { return __atomic_fetch_or(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicAnd(unsigned *p, unsigned v) { return __atomic_fetch_and(p, v, __ATOMIC_RELAXED); }
inline unsigned long long atomicMax(unsigned long long *p, unsigned long long v) {
    unsigned long long cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
    return cur;
}
inline unsigned atomicCAS(unsigned *p, unsigned cmp, unsigned val) {
    __atomic_compare_exchange_n(p, &cmp, val, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
    return cmp;
}
inline unsigned atomicExch(unsigned *p, unsigned v) { return __atomic_exchange_n(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicMax(unsigned *p, unsigned v) {
    unsigned cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
    return cur;
}
// __nanosleep of a team waiting for work: let the other emulated lanes run
inline void tfsm_emu_nap(unsigned) { std::this_thread::yield(); }

// ---------------- runtime API subset ----------------
typedef int cudaError_t;
enum : int { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2, cudaErrorNoDevice = 100 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount = 16 };
#define cudaStreamNonBlocking 0x01
struct CUstream_st {};  // the runtime's stream type (engine.hpp names it)
struct EmuEvent {
    std::chrono::steady_clock::time_point t;
};
typedef CUstream_st *cudaStream_t;
typedef EmuEvent *cudaEvent_t;

inline const char *cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "emulated error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int *n) {
    *n = 1;
    return cudaSuccess;
}
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaMemGetInfo(size_t *f, size_t *t) {
    *f = *t = 0;
    return cudaSuccess;
}
inline cudaError_t cudaGetDevice(int *d) {
    *d = 0;
    return cudaSuccess;
}
inline cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr, int) {
    *v = 1;
    return cudaSuccess;
}
template <class F>
inline cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int *n, F, int, size_t) {
    *n = 1;
    return cudaSuccess;
}
inline cudaError_t cudaMalloc(void **p, size_t n) {
    *p = std::calloc(1, n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void *p) {
    std::free(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind, cudaStream_t = nullptr) {
    if (n) std::memcpy(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind k) { return cudaMemcpyAsync(d, s, n, k); }
inline cudaError_t cudaMemsetAsync(void *d, int v, size_t n, cudaStream_t = nullptr) {
    if (n) std::memset(d, v, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaGetSymbolAddress(void **p, const T &sym) {
    *p = (void *)&sym;
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyFromSymbol(void *dst, const T &sym, size_t n) {
    std::memcpy(dst, &sym, n);
    return cudaSuccess;
}
inline cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned) {
    *s = new CUstream_st;
    return cudaSuccess;
}
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaStreamDestroy(cudaStream_t s) {
    delete s;
    return cudaSuccess;
}
inline cudaError_t cudaEventCreate(cudaEvent_t *e) {
    *e = new EmuEvent;
    return cudaSuccess;
}
inline cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t = nullptr) {
    e->t = std::chrono::steady_clock::now();
    return cudaSuccess;
}
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
    return cudaSuccess;
}
// page-locked host memory: plain host memory here
#define cudaHostAllocDefault 0u
inline cudaError_t cudaHostAlloc(void **p, size_t bytes, unsigned) {
    *p = std::malloc(bytes ? bytes : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFreeHost(void *p) {
    std::free(p);
    return cudaSuccess;
}
// CUDA graphs: the emulated engine launches directly, only the handle type and its release exist
typedef struct EmuGraphExec *cudaGraphExec_t;
inline cudaError_t cudaGraphExecDestroy(cudaGraphExec_t) { return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t e) {
    delete e;
    return cudaSuccess;
}
