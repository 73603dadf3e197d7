// Cost-model MLP kernels: forward (inference), forward + backward (training), Adam.
//
// One warp owns 16 records.  Every product is a warp-level BF16 tensor-core MMA
// (mma.sync.m16n8k16, FP32 accumulation) on operands staged in shared memory:
//   forward          Z1 = X W1, Z2 = H1 W2          (A: records x features, B: weights)
//   backward, data   dH1 = dZ2 W2^T                 (B read transposed)
//   backward, weight dW2 = H1^T dZ2, dW1 = X^T dZ1  (A read transposed; K = the 16 records)
// The last layer (64 -> 1) and the bias gradients are FP32 dot products and warp reductions.
// The weight gradients of a warp are added to FP32 global accumulators with atomics; an Adam
// kernel then updates the FP32 master weights and rewrites their BF16 copies.
//
// The network is 6 337 parameters and about 12 KFLOP per record forward: tensor-core
// throughput is irrelevant here and the warp-level MMA keeps the kernels short.  Rounding points
// (what the CPU checker replicates): X, W1, W2, H1, dZ2 and dZ1 enter the MMAs as BF16
// (round to nearest even); W3 is BF16; everything else is FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>

#include "mlp.hpp"

namespace tfsm {

namespace {

constexpr int kIn = CostModel::kIn, kH = CostModel::kHidden;
constexpr int kWarps = 4;  // warps per block; each owns 16 records
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + (size_t)kIn * kH, kOffW2 = kOffB1 + kH,
                 kOffB2 = kOffW2 + (size_t)kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH;
static_assert(kOffB3 + 1 == CostModel::kParams, "parameter layout");

#define MLP_CK(x)                                                                                      \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct DevParams {
    const __nv_bfloat16 *w1, *w2, *w3;  // BF16 copies
    const float *b1, *b2, *b3;          // FP32 (inside the master vector)
};

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 inputs, FP32 accumulators.
__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragments of the m16n8k16 operands (PTX ISA, warp-level matrix fragments): with g = lane / 4
// and q = lane % 4, A holds rows g and g + 8 at columns 2q, 2q + 1, 2q + 8, 2q + 9; B holds rows
// (k) 2q, 2q + 1, 2q + 8, 2q + 9 of column (n) g; C/D holds rows g, g + 8 at columns 2q, 2q + 1.
template <class F>
__device__ __forceinline__ void frag_a(F at, uint32_t lane, uint32_t a[4]) {
    const int g = (int)(lane >> 2), q = (int)(lane & 3);
    a[0] = pack2(at(g, 2 * q), at(g, 2 * q + 1));
    a[1] = pack2(at(g + 8, 2 * q), at(g + 8, 2 * q + 1));
    a[2] = pack2(at(g, 2 * q + 8), at(g, 2 * q + 9));
    a[3] = pack2(at(g + 8, 2 * q + 8), at(g + 8, 2 * q + 9));
}
template <class F>
__device__ __forceinline__ void frag_b(F at, uint32_t lane, uint32_t b[2]) {
    const int g = (int)(lane >> 2), q = (int)(lane & 3);
    b[0] = pack2(at(2 * q, g), at(2 * q + 1, g));
    b[1] = pack2(at(2 * q + 8, g), at(2 * q + 9, g));
}

struct WarpSmem {
    __nv_bfloat16 x[16][kIn];
    __nv_bfloat16 h1[16][kH];
    __nv_bfloat16 dz2[16][kH];
    __nv_bfloat16 dz1[16][kH];
};
struct BlockSmem {
    __nv_bfloat16 w1[kIn][kH];
    __nv_bfloat16 w2[kH][kH];
    WarpSmem warp[kWarps];
};

// Loads the weights into shared memory and the warp's 16 records (rows >= n are zero).
__device__ void stage(BlockSmem &sm, const DevParams &P, const float *__restrict__ x, size_t row0, size_t n) {
    for (int i = threadIdx.x; i < kIn * kH; i += blockDim.x) sm.w1[i / kH][i % kH] = P.w1[i];
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) sm.w2[i / kH][i % kH] = P.w2[i];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpSmem &W = sm.warp[wid];
    for (int i = (int)lane; i < 16 * kIn; i += 32) {
        const size_t r = row0 + (size_t)(i / kIn);
        W.x[i / kIn][i % kIn] = __float2bfloat16_rn(r < n ? x[r * kIn + (size_t)(i % kIn)] : 0.f);
    }
    __syncthreads();
}

// Forward pass of the warp's 16 records.  z1 / h2 hold the C fragments of Z1 (pre-activation)
// and H2 = relu(Z2) for the 8 column tiles; y_g / y_g8 are the outputs of rows g and g + 8.
__device__ void forward(BlockSmem &sm, const DevParams &P, uint32_t lane, float z1[8][4], float z2[8][4],
                        float &y_g, float &y_g8) {
    WarpSmem &W = sm.warp[threadIdx.x >> 5];
    const int g = (int)(lane >> 2), q = (int)(lane & 3);
    // Z1 = X W1 + b1
    for (int nt = 0; nt < 8; ++nt) {
        for (int c = 0; c < 4; ++c) z1[nt][c] = 0.f;
        for (int kt = 0; kt < kIn / 16; ++kt) {
            uint32_t a[4], b[2];
            frag_a([&](int r, int c) { return W.x[r][kt * 16 + c]; }, lane, a);
            frag_b([&](int k, int c) { return sm.w1[kt * 16 + k][nt * 8 + c]; }, lane, b);
            mma_bf16(z1[nt], a, b);
        }
        const float bias0 = P.b1[nt * 8 + 2 * q], bias1 = P.b1[nt * 8 + 2 * q + 1];
        z1[nt][0] += bias0;
        z1[nt][1] += bias1;
        z1[nt][2] += bias0;
        z1[nt][3] += bias1;
        W.h1[g][nt * 8 + 2 * q] = __float2bfloat16_rn(fmaxf(z1[nt][0], 0.f));
        W.h1[g][nt * 8 + 2 * q + 1] = __float2bfloat16_rn(fmaxf(z1[nt][1], 0.f));
        W.h1[g + 8][nt * 8 + 2 * q] = __float2bfloat16_rn(fmaxf(z1[nt][2], 0.f));
        W.h1[g + 8][nt * 8 + 2 * q + 1] = __float2bfloat16_rn(fmaxf(z1[nt][3], 0.f));
    }
    __syncwarp();
    // Z2 = H1 W2 + b2; y = relu(Z2) . W3 + b3
    float yg = 0.f, yg8 = 0.f;
    for (int nt = 0; nt < 8; ++nt) {
        for (int c = 0; c < 4; ++c) z2[nt][c] = 0.f;
        for (int kt = 0; kt < kH / 16; ++kt) {
            uint32_t a[4], b[2];
            frag_a([&](int r, int c) { return W.h1[r][kt * 16 + c]; }, lane, a);
            frag_b([&](int k, int c) { return sm.w2[kt * 16 + k][nt * 8 + c]; }, lane, b);
            mma_bf16(z2[nt], a, b);
        }
        const int c0 = nt * 8 + 2 * q;
        const float bias0 = P.b2[c0], bias1 = P.b2[c0 + 1];
        z2[nt][0] += bias0;
        z2[nt][1] += bias1;
        z2[nt][2] += bias0;
        z2[nt][3] += bias1;
        const float w0 = __bfloat162float(P.w3[c0]), w1 = __bfloat162float(P.w3[c0 + 1]);
        yg += fmaxf(z2[nt][0], 0.f) * w0 + fmaxf(z2[nt][1], 0.f) * w1;
        yg8 += fmaxf(z2[nt][2], 0.f) * w0 + fmaxf(z2[nt][3], 0.f) * w1;
    }
    // the four lanes of a quad hold the columns of the same two rows
    yg += __shfl_xor_sync(0xffffffffu, yg, 1);
    yg += __shfl_xor_sync(0xffffffffu, yg, 2);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 1);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 2);
    y_g = yg + P.b3[0];
    y_g8 = yg8 + P.b3[0];
}

__global__ void __launch_bounds__(kWarps * 32) k_mlp_predict(DevParams P, const float *__restrict__ x, size_t n,
                                                             float *__restrict__ y) {
    __shared__ BlockSmem sm;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t row0 = ((size_t)blockIdx.x * kWarps + wid) * 16;
    stage(sm, P, x, row0, n);
    float z1[8][4], z2[8][4], yg, yg8;
    forward(sm, P, lane, z1, z2, yg, yg8);
    const int g = (int)(lane >> 2);
    if ((lane & 3) == 0) {
        if (row0 + g < n) y[row0 + g] = yg;
        if (row0 + g + 8 < n) y[row0 + g + 8] = yg8;
    }
}

// Sum over the 8 groups (lanes with equal lane % 4) of a per-column value; result in every lane.
__device__ __forceinline__ float sum_over_groups(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

// Gradient of  mean over the batch (`scale` = 1 / batch size) of (y - t)^2  for the records
// idx[row0 ..] (or rows row0.. when idx is null), added into grad (FP32, parameter layout).
__global__ void __launch_bounds__(kWarps * 32) k_mlp_grad(DevParams P, const float *__restrict__ x,
                                                          const float *__restrict__ t, size_t n, float scale,
                                                          float *__restrict__ grad, float *__restrict__ loss) {
    __shared__ BlockSmem sm;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpSmem &W = sm.warp[wid];
    const size_t row0 = ((size_t)blockIdx.x * kWarps + wid) * 16;
    stage(sm, P, x, row0, n);
    float z1[8][4], z2[8][4], yg, yg8;
    forward(sm, P, lane, z1, z2, yg, yg8);
    const int g = (int)(lane >> 2), q = (int)(lane & 3);
    const bool vg = row0 + g < n, vg8 = row0 + g + 8 < n;
    const float eg = vg ? yg - t[row0 + g] : 0.f, eg8 = vg8 ? yg8 - t[row0 + g + 8] : 0.f;
    const float dyg = 2.f * eg * scale, dyg8 = 2.f * eg8 * scale;
    {
        const float l = sum_over_groups(q == 0 ? eg * eg + eg8 * eg8 : 0.f);  // the quad's lanes hold equal rows
        if (lane == 0) atomicAdd(loss, l);
    }
    // last layer: dW3 = sum_r H2 dy, db3 = sum_r dy; dZ2 = dy W3 (Z2 > 0)
    float db3 = dyg + dyg8;
    db3 += __shfl_xor_sync(0xffffffffu, db3, 4);
    db3 += __shfl_xor_sync(0xffffffffu, db3, 8);
    db3 += __shfl_xor_sync(0xffffffffu, db3, 16);
    if (lane == 0) atomicAdd(grad + kOffB3, db3);
    for (int nt = 0; nt < 8; ++nt) {
        for (int h = 0; h < 2; ++h) {
            const int c = nt * 8 + 2 * q + h;
            const float zg = z2[nt][h], zg8 = z2[nt][2 + h];
            const float dw3 = sum_over_groups(fmaxf(zg, 0.f) * dyg + fmaxf(zg8, 0.f) * dyg8);
            const float w3 = __bfloat162float(P.w3[c]);
            const float dzg = zg > 0.f ? dyg * w3 : 0.f, dzg8 = zg8 > 0.f ? dyg8 * w3 : 0.f;
            const float db2 = sum_over_groups(dzg + dzg8);
            if (g == 0) {
                atomicAdd(grad + kOffW3 + c, dw3);
                atomicAdd(grad + kOffB2 + c, db2);
            }
            W.dz2[g][c] = __float2bfloat16_rn(dzg);
            W.dz2[g + 8][c] = __float2bfloat16_rn(dzg8);
        }
    }
    __syncwarp();
    // dW2[i][j] = sum_r H1[r][i] dZ2[r][j]: A = H1^T (64 x 16 records), B = dZ2 (16 x 64)
    for (int mt = 0; mt < kH / 16; ++mt)
        for (int nt = 0; nt < 8; ++nt) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t a[4], b[2];
            frag_a([&](int r, int c) { return W.h1[c][mt * 16 + r]; }, lane, a);
            frag_b([&](int k, int c) { return W.dz2[k][nt * 8 + c]; }, lane, b);
            mma_bf16(acc, a, b);
            float *dst = grad + kOffW2;
            atomicAdd(dst + (size_t)(mt * 16 + g) * kH + nt * 8 + 2 * q, acc[0]);
            atomicAdd(dst + (size_t)(mt * 16 + g) * kH + nt * 8 + 2 * q + 1, acc[1]);
            atomicAdd(dst + (size_t)(mt * 16 + g + 8) * kH + nt * 8 + 2 * q, acc[2]);
            atomicAdd(dst + (size_t)(mt * 16 + g + 8) * kH + nt * 8 + 2 * q + 1, acc[3]);
        }
    // dH1 = dZ2 W2^T; dZ1 = dH1 (Z1 > 0); db1 = sum_r dZ1
    for (int nt = 0; nt < 8; ++nt) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int kt = 0; kt < kH / 16; ++kt) {
            uint32_t a[4], b[2];
            frag_a([&](int r, int c) { return W.dz2[r][kt * 16 + c]; }, lane, a);
            frag_b([&](int k, int c) { return sm.w2[nt * 8 + c][kt * 16 + k]; }, lane, b);
            mma_bf16(acc, a, b);
        }
        for (int h = 0; h < 2; ++h) {
            const int c = nt * 8 + 2 * q + h;
            const float dzg = z1[nt][h] > 0.f ? acc[h] : 0.f, dzg8 = z1[nt][2 + h] > 0.f ? acc[2 + h] : 0.f;
            const float db1 = sum_over_groups(dzg + dzg8);
            if (g == 0) atomicAdd(grad + kOffB1 + c, db1);
            W.dz1[g][c] = __float2bfloat16_rn(dzg);
            W.dz1[g + 8][c] = __float2bfloat16_rn(dzg8);
        }
    }
    __syncwarp();
    // dW1[k][i] = sum_r X[r][k] dZ1[r][i]: A = X^T (32 x 16 records), B = dZ1 (16 x 64)
    for (int mt = 0; mt < kIn / 16; ++mt)
        for (int nt = 0; nt < 8; ++nt) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t a[4], b[2];
            frag_a([&](int r, int c) { return W.x[c][mt * 16 + r]; }, lane, a);
            frag_b([&](int k, int c) { return W.dz1[k][nt * 8 + c]; }, lane, b);
            mma_bf16(acc, a, b);
            float *dst = grad + kOffW1;
            atomicAdd(dst + (size_t)(mt * 16 + g) * kH + nt * 8 + 2 * q, acc[0]);
            atomicAdd(dst + (size_t)(mt * 16 + g) * kH + nt * 8 + 2 * q + 1, acc[1]);
            atomicAdd(dst + (size_t)(mt * 16 + g + 8) * kH + nt * 8 + 2 * q, acc[2]);
            atomicAdd(dst + (size_t)(mt * 16 + g + 8) * kH + nt * 8 + 2 * q + 1, acc[3]);
        }
}

// Adam step on the FP32 master weights; refreshes the BF16 copies and clears the gradient.
__global__ void k_mlp_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                           float *__restrict__ grad, __nv_bfloat16 *__restrict__ w1b, __nv_bfloat16 *__restrict__ w2b,
                           __nv_bfloat16 *__restrict__ w3b, float lr, float bc1, float bc2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= CostModel::kParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    grad[i] = 0.f;
    if (i < kOffB1) w1b[i - kOffW1] = __float2bfloat16_rn(wi);
    else if (i >= kOffW2 && i < kOffB2) w2b[i - kOffW2] = __float2bfloat16_rn(wi);
    else if (i >= kOffW3 && i < kOffB3) w3b[i - kOffW3] = __float2bfloat16_rn(wi);
}

__global__ void k_mlp_refresh_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ w1b,
                                   __nv_bfloat16 *__restrict__ w2b, __nv_bfloat16 *__restrict__ w3b) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (size_t)kIn * kH) w1b[i] = __float2bfloat16_rn(w[kOffW1 + i]);
    if (i < (size_t)kH * kH) w2b[i] = __float2bfloat16_rn(w[kOffW2 + i]);
    if (i < (size_t)kH) w3b[i] = __float2bfloat16_rn(w[kOffW3 + i]);
}

template <class T>
struct Buf {
    T *p = nullptr;
    size_t n = 0;
    ~Buf() {
        if (p) cudaFree(p);
    }
    void ensure(size_t k) {
        if (k <= n && p) return;
        if (p) cudaFree(p);
        p = nullptr;
        MLP_CK(cudaMalloc((void **)&p, sizeof(T) * std::max<size_t>(k, 1)));
        n = std::max<size_t>(k, 1);
    }
};

}  // namespace

struct CostModel::Impl {
    int device = 0;
    cudaStream_t s = nullptr;
    Buf<float> w, m, v, grad, loss;
    Buf<__nv_bfloat16> w1b, w2b, w3b;
    mutable Buf<float> x, t, y;
    uint64_t adam_t = 0;

    DevParams params() const {
        return DevParams{w1b.p, w2b.p, w3b.p, w.p + kOffB1, w.p + kOffB2, w.p + kOffB3};
    }
    void refresh() {
        k_mlp_refresh_bf16<<<(kH * kH + 255) / 256, 256, 0, s>>>(w.p, w1b.p, w2b.p, w3b.p);
        MLP_CK(cudaGetLastError());
    }
    unsigned blocks(size_t n) const { return (unsigned)((n + 16 * kWarps - 1) / (16 * kWarps)); }
};

CostModel::CostModel(uint64_t seed, int device) : impl_(new Impl) {
    Impl &I = *impl_;
    I.device = device;
    MLP_CK(cudaSetDevice(device));
    MLP_CK(cudaStreamCreateWithFlags(&I.s, cudaStreamNonBlocking));
    I.w.ensure(kParams);
    I.m.ensure(kParams);
    I.v.ensure(kParams);
    I.grad.ensure(kParams);
    I.loss.ensure(1);
    I.w1b.ensure((size_t)kIn * kH);
    I.w2b.ensure((size_t)kH * kH);
    I.w3b.ensure(kH);
    // He-uniform weights, zero biases
    std::mt19937_64 rng(seed);
    std::vector<float> p(kParams, 0.f);
    auto fill = [&](size_t off, size_t count, int fan_in) {
        const float lim = std::sqrt(6.f / (float)fan_in);
        std::uniform_real_distribution<float> U(-lim, lim);
        for (size_t i = 0; i < count; ++i) p[off + i] = U(rng);
    };
    fill(kOffW1, (size_t)kIn * kH, kIn);
    fill(kOffW2, (size_t)kH * kH, kH);
    fill(kOffW3, kH, kH);
    set_params(p.data());
}

CostModel::~CostModel() {
    if (impl_ && impl_->s) {
        cudaStreamSynchronize(impl_->s);
        cudaStreamDestroy(impl_->s);
    }
}

void CostModel::set_params(const float *p) {
    Impl &I = *impl_;
    MLP_CK(cudaSetDevice(I.device));
    MLP_CK(cudaMemcpyAsync(I.w.p, p, kParams * sizeof(float), cudaMemcpyHostToDevice, I.s));
    MLP_CK(cudaMemsetAsync(I.m.p, 0, kParams * sizeof(float), I.s));
    MLP_CK(cudaMemsetAsync(I.v.p, 0, kParams * sizeof(float), I.s));
    MLP_CK(cudaMemsetAsync(I.grad.p, 0, kParams * sizeof(float), I.s));
    I.refresh();
    MLP_CK(cudaStreamSynchronize(I.s));
    I.adam_t = 0;
}

std::vector<float> CostModel::params() const {
    const Impl &I = *impl_;
    std::vector<float> p(kParams);
    MLP_CK(cudaSetDevice(I.device));
    MLP_CK(cudaMemcpyAsync(p.data(), I.w.p, kParams * sizeof(float), cudaMemcpyDeviceToHost, I.s));
    MLP_CK(cudaStreamSynchronize(I.s));
    return p;
}

void CostModel::predict(const float *x, size_t n, float *y) const {
    const Impl &I = *impl_;
    if (n == 0) return;
    MLP_CK(cudaSetDevice(I.device));
    I.x.ensure(n * kIn);
    I.y.ensure(n);
    MLP_CK(cudaMemcpyAsync(I.x.p, x, n * kIn * sizeof(float), cudaMemcpyHostToDevice, I.s));
    k_mlp_predict<<<I.blocks(n), kWarps * 32, 0, I.s>>>(I.params(), I.x.p, n, I.y.p);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaMemcpyAsync(y, I.y.p, n * sizeof(float), cudaMemcpyDeviceToHost, I.s));
    MLP_CK(cudaStreamSynchronize(I.s));
}

void CostModel::gradients(const float *x, const float *t, size_t n, float *g) const {
    const Impl &I = *impl_;
    if (n == 0) throw std::runtime_error("gradients of an empty batch");
    MLP_CK(cudaSetDevice(I.device));
    I.x.ensure(n * kIn);
    I.t.ensure(n);
    MLP_CK(cudaMemcpyAsync(I.x.p, x, n * kIn * sizeof(float), cudaMemcpyHostToDevice, I.s));
    MLP_CK(cudaMemcpyAsync(I.t.p, t, n * sizeof(float), cudaMemcpyHostToDevice, I.s));
    MLP_CK(cudaMemsetAsync(I.grad.p, 0, kParams * sizeof(float), I.s));
    MLP_CK(cudaMemsetAsync(I.loss.p, 0, sizeof(float), I.s));
    k_mlp_grad<<<I.blocks(n), kWarps * 32, 0, I.s>>>(I.params(), I.x.p, I.t.p, n, 1.f / (float)n, I.grad.p,
                                                     I.loss.p);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaMemcpyAsync(g, I.grad.p, kParams * sizeof(float), cudaMemcpyDeviceToHost, I.s));
    MLP_CK(cudaMemsetAsync(I.grad.p, 0, kParams * sizeof(float), I.s));
    MLP_CK(cudaStreamSynchronize(I.s));
}

double CostModel::train(const float *x, const float *t, size_t n, int epochs, int batch, float lr, uint64_t seed) {
    Impl &I = *impl_;
    if (n == 0 || epochs < 0 || batch < 16) throw std::runtime_error("train: empty data, epochs < 0 or batch < 16");
    MLP_CK(cudaSetDevice(I.device));
    // shuffled copies, one permutation per epoch, made on the host and uploaded once
    std::mt19937_64 rng(seed);
    std::vector<size_t> perm(n);
    std::vector<float> xs(n * kIn), ts(n);
    I.x.ensure(n * kIn);
    I.t.ensure(n);
    for (int e = 0; e < epochs; ++e) {
        for (size_t i = 0; i < n; ++i) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        for (size_t i = 0; i < n; ++i) {
            std::memcpy(&xs[i * kIn], &x[perm[i] * kIn], kIn * sizeof(float));
            ts[i] = t[perm[i]];
        }
        MLP_CK(cudaMemcpyAsync(I.x.p, xs.data(), n * kIn * sizeof(float), cudaMemcpyHostToDevice, I.s));
        MLP_CK(cudaMemcpyAsync(I.t.p, ts.data(), n * sizeof(float), cudaMemcpyHostToDevice, I.s));
        for (size_t b0 = 0; b0 < n; b0 += (size_t)batch) {
            const size_t nb = std::min<size_t>((size_t)batch, n - b0);
            k_mlp_grad<<<I.blocks(nb), kWarps * 32, 0, I.s>>>(I.params(), I.x.p + b0 * kIn, I.t.p + b0, nb,
                                                               1.f / (float)nb, I.grad.p, I.loss.p);
            MLP_CK(cudaGetLastError());
            ++I.adam_t;
            const float bc1 = 1.f - std::pow(0.9f, (float)I.adam_t), bc2 = 1.f - std::pow(0.999f, (float)I.adam_t);
            k_mlp_adam<<<(unsigned)((kParams + 255) / 256), 256, 0, I.s>>>(I.w.p, I.m.p, I.v.p, I.grad.p, I.w1b.p,
                                                                          I.w2b.p, I.w3b.p, lr, bc1, bc2);
            MLP_CK(cudaGetLastError());
        }
        // the copies of this epoch must be done before the host buffers are rewritten
        MLP_CK(cudaStreamSynchronize(I.s));
    }
    // final loss over all records at the trained weights
    MLP_CK(cudaMemcpyAsync(I.x.p, x, n * kIn * sizeof(float), cudaMemcpyHostToDevice, I.s));
    MLP_CK(cudaMemcpyAsync(I.t.p, t, n * sizeof(float), cudaMemcpyHostToDevice, I.s));
    MLP_CK(cudaMemsetAsync(I.loss.p, 0, sizeof(float), I.s));
    k_mlp_grad<<<I.blocks(n), kWarps * 32, 0, I.s>>>(I.params(), I.x.p, I.t.p, n, 1.f / (float)n, I.grad.p, I.loss.p);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaMemsetAsync(I.grad.p, 0, kParams * sizeof(float), I.s));
    float loss = 0;
    MLP_CK(cudaMemcpyAsync(&loss, I.loss.p, sizeof(float), cudaMemcpyDeviceToHost, I.s));
    MLP_CK(cudaStreamSynchronize(I.s));
    return (double)loss / (double)n;
}

}  // namespace tfsm
