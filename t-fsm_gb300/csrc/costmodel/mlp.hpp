// Learned cost model of a matching order: a 32-64-64-1 MLP (ReLU) with BF16 weights and FP32
// accumulation, trained and evaluated on the GPU by the hand-written kernels of mlp.cu.
//
// The model predicts log2(1 + chunk evaluations) of searching one pattern vertex's candidates
// with a given matching order (features: costmodel/features.hpp).  The engine uses it only to
// choose among valid matching orders, which never changes a result: every order finds the same
// embeddings.  Without a model the engine keeps the fixed GQL order.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace tfsm {

class CostModel {
  public:
    static constexpr int kIn = 32, kHidden = 64;
    // parameter vector layout (FP32 master copy): W1[in][hidden] row-major, b1[hidden],
    // W2[hidden][hidden], b2[hidden], W3[hidden], b3
    static constexpr size_t kParams = (size_t)kIn * kHidden + kHidden + (size_t)kHidden * kHidden + kHidden + kHidden + 1;

    explicit CostModel(uint64_t seed, int device = 0);  // He-uniform initial weights
    ~CostModel();
    CostModel(const CostModel &) = delete;
    CostModel &operator=(const CostModel &) = delete;

    // y[i] = model(x[i * kIn .. + kIn)), i < n.  Host arrays; computed on the GPU.
    void predict(const float *x, size_t n, float *y) const;
    // Mean-squared-error gradient of one batch of n records at the current weights, in the
    // parameter layout (for gradient checks).
    void gradients(const float *x, const float *t, size_t n, float *g) const;
    // Adam on minibatches of `batch` records for `epochs` passes over the data (shuffled with
    // `seed`); returns the final mean-squared error over all records.
    double train(const float *x, const float *t, size_t n, int epochs, int batch, float lr, uint64_t seed);

    std::vector<float> params() const;
    void set_params(const float *p);  // also resets the optimiser state

  private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
};

}  // namespace tfsm
