// Launchers of the support-evaluation kernels (definitions in kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "dev_common.cuh"

namespace tfsm {
namespace dev {

constexpr int kSearchWarps = 8;  // warps per block of the search kernels
// Blocks of the search kernels that must fit on one SM at once (the register budget follows from
// it: 65536 / (256 x blocks)); the build may set it with -DTFSM_SEARCH_MIN_BLOCKS.
#ifndef TFSM_SEARCH_MIN_BLOCKS
#define TFSM_SEARCH_MIN_BLOCKS 4
#endif
constexpr int kSearchMinBlocks = TFSM_SEARCH_MIN_BLOCKS;

// LDF + NLF bitmaps of the items' (pattern, vertex) pairs, intersected with the final domains of
// the sources that PatDesc::parent_off / push_off reference in the table `srcs` (n_srcs pools of
// earlier calls; may be empty).
cudaError_t launch_domain_init(const Graph &g, const PatDesc *descs, PatStatus *st, const uint32_t *item_pu,
                               const uint64_t *prefix, uint32_t n_items, uint64_t total_words, uint32_t *dom,
                               uint32_t *found, uint32_t *failed, const SourceLevel *srcs, uint32_t n_srcs,
                               uint64_t chk_words, cudaStream_t s);

// Arc-consistency round `round` (0..31) over the items' words; see k_refine for which patterns
// take part.
cudaError_t launch_refine(const Graph &g, const PatDesc *descs, PatStatus *st, const uint32_t *item_pu,
                          const uint64_t *prefix, uint32_t n_items, uint64_t total_words, uint32_t *dom,
                          uint64_t chk_words, int round, uint32_t tau, bool exact, cudaStream_t s);

// One search pass: k_search over `prm.n_items` items.  `counters` (kNumCounters x u32) must be
// zero on entry; `splits` holds two buffers of prm.split_cap tasks each.
cudaError_t launch_search(const Graph &g, const PatDesc *descs, PatStatus *st, const ItemGroup *igroups,
                          const ItemEntry *ientries, const SearchParams &prm, uint32_t *counters, const uint32_t *dom,
                          uint32_t *found, uint32_t *failed, SplitTask *splits, SplitGroup *groups, cudaStream_t s);

// Split round `round` (0 <= round < kMaxRounds) of the pass whose counters are `counters`: the tasks
// written for it by the previous phase, each with a step budget of `budget` chunk evaluations (0:
// none).  Rounds run in order on one stream; round kMaxRounds - 1 has no step budget.
cudaError_t launch_split_round(const Graph &g, const PatDesc *descs, PatStatus *st, const SearchParams &prm,
                               uint32_t *counters, int round, uint32_t budget, const uint32_t *dom, uint32_t *found,
                               uint32_t *failed, SplitTask *splits, SplitGroup *groups, cudaStream_t s);

// Warps of k_search resident on the device at once (SMs x blocks per SM x warps per block).
uint32_t resident_search_warps();

// Checked builds (-DTFSM_BOUNDS_CHECK): the first out-of-bounds access the search kernels
// detected (count, site, index, bound); false when none or when checks are compiled out.
bool read_bounds_check(unsigned long long rec[4]);

}  // namespace dev
}  // namespace tfsm
