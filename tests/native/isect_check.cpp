// The oracle's hybrid sorted-set intersection (merge below a size ratio of 50, galloping above,
// oracle/port_mni.hpp after intersection/computesetintersection.cpp:9-44) equals
// std::set_intersection on random sorted lists: empty lists, equal sizes, ratios just below, at and
// above 50, and far above.  Test infrastructure only.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "../../oracle/port_mni.hpp"

int main() {
    std::mt19937 rng(20250101);
    const unsigned ratios[] = {0, 1, 2, 10, 49, 50, 51, 64, 100, 1000};
    int failures = 0, cases = 0;
    for (unsigned ratio : ratios)
        for (unsigned small : {0u, 1u, 3u, 17u, 64u})
            for (int rep = 0; rep < 20; ++rep) {
                const unsigned nb = ratio == 0 ? 0 : small * ratio + (unsigned)(rng() % (ratio + 1));
                const unsigned universe = 4 * (small + nb) + 8;
                auto draw = [&](unsigned n) {
                    std::vector<uint32_t> v;
                    while (v.size() < n) v.push_back(rng() % universe);
                    std::sort(v.begin(), v.end());
                    v.erase(std::unique(v.begin(), v.end()), v.end());
                    return v;
                };
                const std::vector<uint32_t> a = draw(small), b = draw(nb);
                std::vector<uint32_t> want;
                std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(want));
                for (int swap = 0; swap < 2; ++swap) {
                    const std::vector<uint32_t> &x = swap ? b : a, &y = swap ? a : b;
                    std::vector<uint32_t> out(std::max<size_t>(1, std::min(x.size(), y.size())));
                    uint32_t n = 0;
                    oracle::intersect(x.data(), (uint32_t)x.size(), y.data(), (uint32_t)y.size(), out.data(), n);
                    out.resize(n);
                    ++cases;
                    if (out != want) {
                        std::printf("FAIL ratio %u sizes %zu %zu: %zu vs %zu\n", ratio, x.size(), y.size(), out.size(),
                                    want.size());
                        ++failures;
                    }
                }
            }
    std::printf("%s %d cases\n", failures ? "FAILED" : "ok", cases);
    return failures ? 1 : 0;
}
