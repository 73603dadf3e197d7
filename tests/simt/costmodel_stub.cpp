// Test infrastructure: the SIMT emulation links the engine without the cost-model kernels (their
// tensor-core instructions have no CPU form); the emulated runs use the fixed GQL order only.
#include <stdexcept>

#include "costmodel/mlp.hpp"

namespace tfsm {

struct CostModel::Impl {};
CostModel::CostModel(uint64_t, int) { throw std::runtime_error("cost model not available in the SIMT emulation"); }
CostModel::~CostModel() = default;
void CostModel::predict(const float *, size_t, float *) const { throw std::runtime_error("no cost model"); }
void CostModel::gradients(const float *, const float *, size_t, float *) const { throw std::runtime_error("no cost model"); }
double CostModel::train(const float *, const float *, size_t, int, int, float, uint64_t) {
    throw std::runtime_error("no cost model");
}
std::vector<float> CostModel::params() const { throw std::runtime_error("no cost model"); }
void CostModel::set_params(const float *) { throw std::runtime_error("no cost model"); }

}  // namespace tfsm
