// C-ABI check of tfsm_evaluate_level under the SIMT emulation (test infrastructure only).
//
// usage: abi_emu GRAPH.lg TAU GOLDEN.mni.txt
// The environment variables ISECT_RATIO and SEARCH_LANES, when set, become the handle's
// isect_ratio and search_lanes options.
// Evaluates the golden patterns level by level (by DFS-code length) with TFSM_FLAG_EXACT. Each
// pattern whose DFS-code prefix (its code minus the last edge: the same vertex numbering, one edge
// less) was evaluated by the previous level's call starts from that prefix's kept domains. Every
// pattern's exact MNI counts must equal the golden ones. Then the parent checks: a parent that is
// not a sub-pattern (other labels, more vertices), an index out of range and domains of another
// graph give TFSM_ERR_ARG; a pattern may be its own parent.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tfsm.h"

namespace {

struct Golden {
    std::string key;
    std::vector<tfsm_dfs_code> codes;
    std::vector<uint32_t> mni;
};

std::string prefix_key(const std::string &key) {
    const size_t sp = key.rfind(' ');
    return sp == std::string::npos ? std::string() : key.substr(0, sp);
}

int failures = 0;

void expect(bool ok, const std::string &what) {
    if (!ok) {
        std::printf("FAIL %s\n", what.c_str());
        ++failures;
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s GRAPH.lg TAU GOLDEN.mni.txt\n", argv[0]);
        return 2;
    }
    const int tau = std::atoi(argv[2]);
    std::map<size_t, std::vector<Golden>> levels;  // by number of codes
    std::ifstream in(argv[3]);
    for (std::string line; std::getline(in, line);) {
        const size_t bar = line.find('|');
        if (bar == std::string::npos) continue;
        Golden gd;
        gd.key = line.substr(0, bar);
        while (!gd.key.empty() && gd.key.back() == ' ') gd.key.pop_back();
        std::istringstream codes(gd.key);
        for (std::string tok; codes >> tok;) {
            tfsm_dfs_code c;
            if (std::sscanf(tok.c_str(), "%d,%d,%d,%d,%d", &c.from, &c.to, &c.from_label, &c.edge_label,
                            &c.to_label) != 5)
                return 2;
            gd.codes.push_back(c);
        }
        std::istringstream counts(line.substr(bar + 1));
        for (uint32_t x; counts >> x;) gd.mni.push_back(x);
        levels[gd.codes.size()].push_back(gd);
    }
    tfsm_graph *g = nullptr, *other = nullptr;
    if (tfsm_graph_load(argv[1], tau, &g) != TFSM_OK || tfsm_graph_load(argv[1], tau, &other) != TFSM_OK) {
        std::printf("FAIL load: %s\n", tfsm_last_error());
        return 1;
    }
    {
        tfsm_options o;
        o.struct_size = sizeof(o);
        bool ok = tfsm_get_options(g, &o) == TFSM_OK;
        if (const char *r = std::getenv("ISECT_RATIO")) o.isect_ratio = (uint32_t)std::atoi(r);
        if (const char *l = std::getenv("SEARCH_LANES")) o.search_lanes = (uint32_t)std::atoi(l);
        ok = ok && tfsm_set_options(g, &o) == TFSM_OK;
        expect(ok, "options: " + std::string(tfsm_last_error()));
    }
    tfsm_domains *prev = nullptr, *first = nullptr;
    std::map<std::string, int> prev_index;
    size_t with_parent = 0, evaluated = 0;
    for (auto &kv : levels) {
        std::vector<Golden> &gs = kv.second;
        const size_t n = gs.size();
        std::vector<tfsm_pattern> pats(n);
        std::vector<tfsm_parent> parents(n, tfsm_parent{nullptr, 0});
        for (size_t i = 0; i < n; ++i) {
            pats[i].n_codes = (int32_t)gs[i].codes.size();
            pats[i].codes = gs[i].codes.data();
            auto it = prev_index.find(prefix_key(gs[i].key));
            if (prev && it != prev_index.end()) {
                parents[i] = tfsm_parent{prev, it->second};
                ++with_parent;
            }
        }
        std::vector<tfsm_result> res(n);
        tfsm_domains *cur = nullptr;
        const int rc = tfsm_evaluate_level(g, pats.data(), (int32_t)n, tau, TFSM_FLAG_EXACT, parents.data(), res.data(),
                                           &cur);
        expect(rc == TFSM_OK, "level call: " + std::string(tfsm_last_error()));
        for (size_t i = 0; i < n && rc == TFSM_OK; ++i) {
            bool same = res[i].status == TFSM_OK && (size_t)res[i].n_vertices == gs[i].mni.size();
            for (size_t u = 0; same && u < gs[i].mni.size(); ++u) same = res[i].mni[u] == gs[i].mni[u];
            expect(same, "mni of " + gs[i].key);
            ++evaluated;
        }
        if (!first) first = cur;
        else if (prev != first) tfsm_domains_free(prev);
        prev = cur;
        prev_index.clear();
        for (size_t i = 0; i < n; ++i) prev_index[gs[i].key] = (int)i;
    }
    // parent checks on the first level's patterns (single edges)
    const std::vector<Golden> &one = levels.begin()->second;
    std::vector<tfsm_pattern> p1(one.size());
    for (size_t i = 0; i < one.size(); ++i) p1[i] = tfsm_pattern{(int32_t)one[i].codes.size(), one[i].codes.data()};
    tfsm_result r;
    tfsm_parent bad{first, (int32_t)one.size()};
    expect(tfsm_evaluate_level(g, p1.data(), 1, tau, 0, &bad, &r, nullptr) == TFSM_OK && r.status == TFSM_ERR_ARG,
           "index out of range is TFSM_ERR_ARG");
    tfsm_parent self{first, 0};
    expect(tfsm_evaluate_level(other, p1.data(), 1, tau, 0, &self, &r, nullptr) == TFSM_OK &&
               r.status == TFSM_ERR_ARG,
           "domains of another graph are TFSM_ERR_ARG");
    for (size_t j = 1; j < one.size(); ++j) {  // a single edge with other labels is no sub-pattern
        tfsm_parent wrong{first, (int32_t)j};
        expect(tfsm_evaluate_level(g, p1.data(), 1, tau, 0, &wrong, &r, nullptr) == TFSM_OK &&
                   r.status == TFSM_ERR_ARG,
               "a parent with other labels is TFSM_ERR_ARG");
        break;
    }
    if (levels.size() > 1) {  // a larger pattern is no sub-pattern of a single edge
        const std::vector<Golden> &two = std::next(levels.begin())->second;
        std::vector<tfsm_pattern> p2(two.size());
        for (size_t i = 0; i < two.size(); ++i) p2[i] = tfsm_pattern{(int32_t)two[i].codes.size(), two[i].codes.data()};
        tfsm_domains *d2 = nullptr;
        tfsm_result r2;
        expect(tfsm_evaluate_level(g, p2.data(), 1, tau, 0, nullptr, &r2, &d2) == TFSM_OK && d2, "second-level call");
        tfsm_parent big{d2, 0};
        expect(tfsm_evaluate_level(g, p1.data(), 1, tau, 0, &big, &r, nullptr) == TFSM_OK && r.status == TFSM_ERR_ARG,
               "a larger parent is TFSM_ERR_ARG");
        tfsm_domains_free(d2);
    }
    expect(tfsm_evaluate_level(g, p1.data(), 1, tau, TFSM_FLAG_EXACT, &self, &r, nullptr) == TFSM_OK &&
               r.status == TFSM_OK && (size_t)r.n_vertices == one[0].mni.size() && r.mni[0] == one[0].mni[0],
           "a pattern is its own parent");
    if (prev != first) tfsm_domains_free(prev);
    tfsm_graph_free(g);       // domains may outlive their graph
    tfsm_domains_free(first);
    tfsm_graph_free(other);
    std::printf("%s evaluated=%zu with_parent=%zu levels=%zu\n", failures ? "FAILED" : "ok", evaluated, with_parent,
                levels.size());
    return failures ? 1 : 0;
}
