// Allocation-free support evaluation (definition and the rules of its scratch array: noalloc.cu).
#pragma once

#include <cstdint>

#include "../../include/tfsm.h"
#include "engine.hpp"

namespace tfsm {

// Evaluates one pattern with all per-call device buffers in a fixed file-scope device array.
// Returns a TFSM_* status; `msg` receives a static description on failure.
int noalloc_evaluate(const GpuEngine &eng, const tfsm_pattern *pattern, uint32_t tau, bool exact, tfsm_result *out,
                     const char *&msg);

}  // namespace tfsm
