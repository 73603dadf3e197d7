// Features of a matching order for the cost model (32 values, each scaled to about [0, 1]).
//
// One record describes searching the candidates of pattern vertex `start` with the matching order
// `order` (order[0] == start); bn[i] is the mask of order[i]'s pattern neighbours that precede it:
//   0      pattern vertices / 8            1   pattern edges / 16
//   2      log2(tau + 1) / 20              3   log2(|D(start)| + 1) / 20
//   4..10  log2(|D(order[i])| + 1) / 20, i = 1..7          (0 past the pattern's size)
//   11..17 backward neighbours of order[i] / 4, i = 1..7   (how many lists are intersected)
//   18..24 log2(mean data degree of order[i]'s label + 1) / 16, i = 0..6
//   25..31 pattern degree of order[i] / 6, i = 0..6
// Domain sizes are the arc-consistent sizes the engine has when it chooses the order.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../cuda/dev_common.cuh"

namespace tfsm {
namespace costmodel {

constexpr int kFeatures = 32;
using Order = std::array<uint8_t, dev::kMaxN>;

inline uint32_t backward_mask(const dev::PatDesc &D, const Order &order, int i) {
    uint32_t before = 0;
    for (int k = 0; k < i; ++k) before |= 1u << order[(size_t)k];
    return D.adj[order[(size_t)i]] & before;
}

inline void order_features(const dev::PatDesc &D, const uint32_t *dsize, uint32_t tau, const float *label_mean_deg,
                           const Order &order, float *f) {
    const int n = D.n;
    int edges2 = 0;
    for (int u = 0; u < n; ++u) edges2 += __builtin_popcount(D.adj[u]);
    auto lg = [](double x) { return (float)std::log2(x + 1.0); };
    for (int i = 0; i < kFeatures; ++i) f[i] = 0.f;
    f[0] = (float)n / 8.f;
    f[1] = (float)(edges2 / 2) / 16.f;
    f[2] = lg((double)tau) / 20.f;
    f[3] = lg((double)dsize[order[0]]) / 20.f;
    for (int i = 1; i <= 7 && i < n; ++i) {
        f[3 + i] = lg((double)dsize[order[(size_t)i]]) / 20.f;
        f[10 + i] = (float)__builtin_popcount(backward_mask(D, order, i)) / 4.f;
    }
    for (int i = 0; i < 7 && i < n; ++i) {
        const int w = order[(size_t)i];
        f[18 + i] = lg((double)label_mean_deg[D.lab[w]]) / 16.f;
        f[25 + i] = (float)D.deg[w] / 6.f;
    }
}

// Connected matching orders from `start` (every vertex after the first has a pattern neighbour
// before it), depth-first in ascending vertex order, at most `cap` of them.
inline void enumerate_orders(const dev::PatDesc &D, int start, size_t cap, std::vector<Order> &out) {
    out.clear();
    Order cur{};
    cur[0] = (uint8_t)start;
    struct Rec {
        const dev::PatDesc &D;
        size_t cap;
        std::vector<Order> &out;
        Order &cur;
        void go(int depth, uint32_t visited) {
            if (out.size() >= cap) return;
            if (depth == D.n) {
                out.push_back(cur);
                return;
            }
            uint32_t reach = 0;
            for (int k = 0; k < depth; ++k) reach |= D.adj[cur[(size_t)k]];
            reach &= ~visited;
            for (int w = 0; w < D.n && out.size() < cap; ++w) {
                if (!((reach >> w) & 1u)) continue;
                cur[(size_t)depth] = (uint8_t)w;
                go(depth + 1, visited | (1u << w));
            }
        }
    } rec{D, cap, out, cur};
    rec.go(1, 1u << start);
}

}  // namespace costmodel
}  // namespace tfsm
