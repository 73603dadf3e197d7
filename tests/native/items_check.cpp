// Test driver: dev::item_at (cuda/dev_common.cuh), the search kernel's decoding of item k from the
// call's item groups, enumerates every group's runs round by round (round t: run t of every entry
// with more than t runs, entries in their sorted order), and so covers every (entry, run of
// `chunk_words` words) exactly once.  Random groups; prints "ok ..." and exits 0, or the first
// difference and exits 1.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "cuda/dev_common.cuh"

using namespace tfsm::dev;

int main(int argc, char **argv) {
    const uint64_t seed = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;
    std::mt19937_64 rng(seed);
    uint64_t checked = 0;
    for (int it = 0; it < 400; ++it) {
        const uint32_t cw = 1 + (uint32_t)(rng() % 4);
        const int n_groups = 1 + (int)(rng() % 6);
        std::vector<ItemGroup> groups;
        std::vector<ItemEntry> entries;
        std::vector<SearchItem> want;
        uint64_t n_items = 0;
        for (int gi = 0; gi < n_groups; ++gi) {
            const int m = 1 + (int)(rng() % 40);
            std::vector<ItemEntry> es((size_t)m);
            for (int j = 0; j < m; ++j) {
                std::memset(&es[(size_t)j], 0, sizeof(ItemEntry));
                es[(size_t)j].pat = (uint32_t)(gi * 100 + j);
                es[(size_t)j].u = (uint16_t)(j % 7);
                // ties and very uneven sizes
                const uint32_t words = rng() % 3 == 0 ? 1 + (uint32_t)(rng() % 4) : 1 + (uint32_t)(rng() % 300);
                es[(size_t)j].words = words;
                es[(size_t)j].runs = (words + cw - 1) / cw;
            }
            std::stable_sort(es.begin(), es.end(), [](const ItemEntry &x, const ItemEntry &y) { return x.runs > y.runs; });
            uint64_t acc = 0;
            for (size_t i = es.size(); i-- > 0;) {
                const uint32_t below = i + 1 < es.size() ? es[i + 1].runs : 0;
                acc += (uint64_t)(i + 1) * (es[i].runs - below);
                es[i].before = acc;
            }
            groups.push_back({n_items, (uint32_t)entries.size(), (uint32_t)m});
            entries.insert(entries.end(), es.begin(), es.end());
            // the order the decoding must produce
            for (uint32_t t = 0; t < es[0].runs; ++t)
                for (const ItemEntry &e : es)
                    if (e.runs > t) {
                        SearchItem s;
                        s.pat = e.pat;
                        s.u = e.u;
                        s.pad = 0;
                        s.word_lo = t * cw;
                        s.word_hi = std::min(e.words, t * cw + cw);
                        want.push_back(s);
                    }
            n_items += acc;
        }
        if (want.size() != n_items) {
            std::printf("differ: %zu items enumerated, %llu counted\n", want.size(), (unsigned long long)n_items);
            return 1;
        }
        for (uint64_t k = 0; k < n_items; ++k) {
            const SearchItem a = item_at(groups.data(), (uint32_t)groups.size(), entries.data(), cw, k);
            const SearchItem &b = want[k];
            if (a.pat != b.pat || a.u != b.u || a.word_lo != b.word_lo || a.word_hi != b.word_hi) {
                std::printf("differ at iteration %d item %llu: (%u %u %u-%u) vs (%u %u %u-%u)\n", it,
                            (unsigned long long)k, a.pat, a.u, a.word_lo, a.word_hi, b.pat, b.u, b.word_lo, b.word_hi);
                return 1;
            }
        }
        checked += n_items;
    }
    std::printf("ok: %llu items\n", (unsigned long long)checked);
    return 0;
}
