// GPU ingestion of the data graph: `.lg` text or edge arrays -> the engine's device graph.
//
// Builds on the device, in one stream, what host/lg_fast.hpp (`load_lg_fast`,
// `build_pruned_edges`: the reference's loader, parallel/graph.h:557-803) followed by the
// GpuEngine constructor's renumbering and upload builds on the host: label frequencies and
// pruning, the pruned vertex order, the label-grouped degree-ranked internal ids, the CSR sorted by
// (neighbour, edge label), the per-vertex label-offset table and the 1-edge pattern table
// (parallel/graph.h:685-803 "hashedEdges").  Only small tables (labels, counts, 1-edge patterns)
// travel back to the host.  Errors are the host loader's: same codes, same messages.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "host/lg_graph.hpp"

struct CUstream_st;

namespace tfsm {

// A device allocation held until the engine takes it over (release()).
struct DevOwned {
    void *p = nullptr;
    size_t bytes = 0;
    DevOwned() = default;
    DevOwned(const DevOwned &) = delete;
    DevOwned &operator=(const DevOwned &) = delete;
    ~DevOwned();
    void *release() {
        void *q = p;
        p = nullptr;
        return q;
    }
};

struct DeviceGraphBuild {
    LgGraph summary;                      // n, m, labels, 1-edge patterns, statistics (no adjacency)
    std::vector<uint32_t> lstart;         // first internal id of each dense label, NL + 1 entries
    std::vector<float> label_mean_deg;    // per dense label
    uint64_t m2 = 0;                      // directed adjacency entries
    DevOwned row_off;                     // u32 [n + 1]
    DevOwned col;                         // u32 [m2 + pad], pad entries 0xffffffff
    DevOwned elab;                        // u8  [m2], dense edge labels
    DevOwned label_start;                 // u32 [NL + 1]
    DevOwned lab_off;                     // u32 [n * (NL + 1)]
    std::string breakdown;                // phase times, milliseconds
    uint64_t h2d_bytes = 0;               // host -> device bytes copied (input and small tables)
};

// The graph of a `.lg` file, parsed on the GPU (the file is read by the host and copied as bytes).
void ingest_lg_file(const std::string &path, int tau, CUstream_st *s, DeviceGraphBuild &out);

// The graph of host arrays (tfsm_graph_from_edges): vertex labels [n], edges (src, dst, label) [m].
void ingest_edge_arrays(uint32_t n, const int32_t *vlabel, uint64_t m, const uint32_t *src, const uint32_t *dst,
                        const int32_t *elabel, int tau, CUstream_st *s, DeviceGraphBuild &out);

}  // namespace tfsm
