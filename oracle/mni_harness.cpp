// ORACLE — test infrastructure only.  Exact per-vertex MNI domains computed by the reference's
// own serial matching engine (serial/gmatch.h), compiled from the read-only reference tree by
// oracle/Makefile.  It pins oracle/port_mni.hpp and, through the golden fixtures it produces,
// the CUDA path.  The reference never reports supports (its lazy count stops at tau,
// serial/grami.h:312-320), so this driver runs the engine on every candidate with no early exit:
//   DPisoFilter (serial/gmatch.h:326-373)  ->  buildTable (687-823)
//   for each pattern vertex u: generateGQLQueryPlan(u) + generateBN (584-685)
//     for each candidate v of u: execute (174-188, LFTJ 906-987); on timeout resumeSearch (231-244)
//     every vertex of a found embedding joins the MNI domain of its pattern vertex.
//
// usage: mni_harness -file G.lg -freq TAU -patterns P.txt
//   P.txt: one pattern per line, DFS codes "from,to,from_label,edge_label,to_label" separated by
//   spaces.  Output: one line per pattern, "<codes> | c0 c1 ... c(n-1)" with the exact domain sizes.
#include "grami.h"

#include <sstream>

int Settings::maxNumNodes = -1;

int main(int argc, char *argv[]) {
    char *file = getCmdOption(argv, argv + argc, "-file");
    char *freq = getCmdOption(argv, argv + argc, "-freq");
    char *pats = getCmdOption(argv, argv + argc, "-patterns");
    if (!file || !freq || !pats) {
        std::cerr << "usage: mni_harness -file G.lg -freq TAU -patterns P.txt" << std::endl;
        return 2;
    }
    const int tau = atoi(freq);
    Graph graph(tau);
    Graph pruned(tau);
    graph.load_graph(pruned, file, " ");

    GMatchEngine eng;
    eng.initialize_space(pruned.maxLabelFreq, pruned.size());

    std::ifstream in(pats);
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::istringstream ss(line);
        std::string tok;
        Pattern p;
        bool first = true;
        while (ss >> tok) {
            int a, b, fl, el, tl;
            if (sscanf(tok.c_str(), "%d,%d,%d,%d,%d", &a, &b, &fl, &el, &tl) != 5) break;
            dfs_code_t c(a, b, fl, el, tl);
            if (first) {
                p.init(c, NULL);
                first = false;
            } else {
                p.extend(c);
            }
        }
        p.parent = NULL;
        const int n = p.size();
        p.non_candidates.resize(n);
        VectorOfSet found(n);
        eng.set(&pruned, &p);
        if (eng.DPisoFilter(false)) {
            eng.buildTable();
            for (int u = 0; u < n; ++u) {
                eng.generateGQLQueryPlan(u);
                eng.generateBN();
                ui idx = 0;
                for (auto it = p.candidates[u].candidate.begin(); it != p.candidates[u].candidate.end(); ++it, ++idx) {
                    vector<VertexID> emb(n);
                    emb[u] = *it;
                    MatchingStatus ms(n);
                    int val = eng.execute(u, idx, emb, ms);
                    if (val == -3) {
                        vector<VertexID> emb2(n);
                        emb2[u] = *it;
                        val = eng.resumeSearch(u, ms, emb2);
                        emb = emb2;
                    }
                    if (val == -1)
                        for (int j = 0; j < n; ++j) found[j].insert(emb[j]);
                }
                eng.clear_match();
            }
            eng.clear_table();
        }
        eng.reset();
        std::cout << line << " |";
        for (int j = 0; j < n; ++j) std::cout << ' ' << found[j].size();
        std::cout << std::endl;
    }
    return 0;
}
