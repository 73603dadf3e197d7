// Test driver for the rules the GPU ingestion shares with the host loader (cuda/ingest_rules.cuh):
//   ingest_rules_check parse SEED ITERS  random `.lg` texts (valid lines, malformed lines, white
//                                         space and sign variants, 64-bit overflow): parsing line by
//                                         line with lgparse::parse_line, then the vertex-order and
//                                         endpoint checks in the order the host applies them, gives
//                                         the host parser's result (same vertices and edges, or the
//                                         same error code and message) for the plain and the
//                                         multi-threaded host parsers
//   ingest_rules_check rank              rank_to_local equals the GpuEngine constructor's fill loop
//                                         for every class size up to 2000 and a few larger ones
// Prints "ok ..." and exits 0, or prints the first difference and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "cuda/ingest_rules.cuh"
#include "host/lg_fast.hpp"
#include "host/lg_graph.hpp"

using namespace tfsm;

struct Outcome {
    int code = 0;
    std::string msg;
    std::vector<int> vlabel;
    std::vector<std::tuple<uint32_t, uint32_t, int>> edges;
    bool operator==(const Outcome &o) const {
        return code == o.code && msg == o.msg && vlabel == o.vlabel && edges == o.edges;
    }
};

// The ingestion kernels' sequence, run serially: kinds and first malformed line, values in line
// order, vertex order, endpoints.
static Outcome by_rules(const std::vector<char> &buf) {
    Outcome o;
    const uint64_t size = buf.size();
    std::vector<std::pair<uint64_t, uint64_t>> lines;
    uint64_t ls = 0;
    for (uint64_t i = 0; i < size; ++i)
        if (buf[i] == '\n') {
            lines.push_back({ls, i});
            ls = i + 1;
        }
    std::vector<lgparse::Line> parsed;
    for (size_t k = 0; k < lines.size(); ++k) {
        parsed.push_back(lgparse::parse_line(buf.data(), size, lines[k].first, lines[k].second));
        const uint8_t kd = parsed.back().kind;
        if (kd >= lgparse::kBadVertex) {
            o.code = 3;
            o.msg = (kd == lgparse::kBadVertex ? "malformed vertex line "
                     : kd == lgparse::kBadEdge ? "malformed edge line "
                                               : "unknown line kind at line ") +
                    std::to_string(k + 1);
            return o;
        }
    }
    std::vector<int64_t> ids;
    for (auto &L : parsed) {
        if (L.kind == lgparse::kVertex) {
            ids.push_back(L.v[0]);
            o.vlabel.push_back((int32_t)(uint32_t)(uint64_t)L.v[1]);
        } else if (L.kind == lgparse::kEdge) {
            o.edges.emplace_back((uint32_t)(uint64_t)L.v[0], (uint32_t)(uint64_t)L.v[1],
                                 (int32_t)(uint32_t)(uint64_t)L.v[2]);
        }
    }
    for (size_t i = 0; i < ids.size(); ++i)
        if (ids[i] != (int64_t)i) {
            o = Outcome();
            o.code = 3;
            o.msg = "vertex ids must be 0..N-1 in order (line for id " + std::to_string(ids[i]) + ")";
            return o;
        }
    for (auto &e : o.edges)
        if (std::get<0>(e) >= o.vlabel.size() || std::get<1>(e) >= o.vlabel.size()) {
            o = Outcome();
            o.code = 3;
            o.msg = "edge endpoint out of range";
            return o;
        }
    return o;
}

template <class F>
static Outcome by_host(F parse) {
    Outcome o;
    try {
        RawLg raw = parse();
        o.vlabel = raw.vlabel;
        o.edges = raw.edges;
    } catch (const LgError &e) {
        o.code = e.code;
        o.msg = e.what();
    }
    return o;
}

static std::string random_text(std::mt19937_64 &rng) {
    auto pick = [&](int k) { return (int)(rng() % (uint64_t)k); };
    static const char *const junk[] = {" ", "  ", "\t", "\r", "\v", "\f", "-", "+", "x", "0x1", "#", "07",
                                       "99999999999999999999", "-9223372036854775808", "9223372036854775807",
                                       "4294967296", "4294967297", "-1", "+5", "- 3", "\t7", "1\t2"};
    std::string t;
    const int nv = pick(12), ne = pick(20);
    const bool messy = pick(5) == 0;
    if (pick(2)) t += "t # 0\n";
    int v = 0, e = 0;
    while (v < nv || e < ne) {
        const int what = pick(10);
        if (what < 4 && v < nv) {
            // a vertex line, usually well formed, ids mostly in order
            const long id = pick(150) ? v : v + pick(3) - 1;
            t += std::string(pick(4) ? "" : " ") + "v " + std::to_string(id) + " " + std::to_string(pick(7) - 2);
            ++v;
        } else if (what < 8 && e < ne) {
            const int span = nv + (pick(60) ? 0 : 1);  // now and then an endpoint past the last vertex
            const long a = pick(200) ? pick(std::max(span, 1)) : -1, b = pick(std::max(span, 1));
            t += "e " + std::to_string(a) + " " + std::to_string(b) + " " + std::to_string(pick(4));
            ++e;
        } else if (what == 8 || pick(20)) {
            t += pick(2) ? "# comment" : "";
        } else {
            t += pick(2) ? "v" : (pick(2) ? "e" : "q");
        }
        if (messy) {
            const int k = pick(5) ? 0 : pick(3) + 1;
            for (int i = 0; i < k; ++i) {
                t += junk[pick((int)(sizeof(junk) / sizeof(junk[0])))];
                if (pick(3) == 0) t += " ";
            }
        }
        if (pick(12) == 0) t += "\r";
        t += "\n";
        if (pick(25) == 0) t += "\n";
    }
    if (pick(5) == 0 && !t.empty()) t.pop_back();  // no final newline
    return t;
}

static int check_parse(uint64_t seed, int iters) {
    std::mt19937_64 rng(seed);
    int ok_graphs = 0, errors = 0;
    for (int it = 0; it < iters; ++it) {
        const std::string text = random_text(rng);
        // the host loader's buffer: the bytes and an appended newline (detail::read_file), here
        // followed by a terminator so that strtol never reads past it
        std::vector<char> buf(text.begin(), text.end());
        buf.push_back('\n');
        std::vector<char> term(buf);
        term.push_back('\0');
        const Outcome want = by_host([&] { return parse_lg_text(term.data(), buf.size()); });
        const Outcome fast = by_host([&] { return parse_lg_text_fast(term.data(), buf.size(), 3); });
        const Outcome got = by_rules(buf);
        if (!(got == want) || !(fast == want)) {
            std::printf("differ at iteration %d (rules: %d '%s', host: %d '%s', fast: %d '%s')\n---\n%s\n---\n", it,
                        got.code, got.msg.c_str(), want.code, want.msg.c_str(), fast.code, fast.msg.c_str(),
                        text.c_str());
            return 1;
        }
        (want.code ? errors : ok_graphs)++;
    }
    std::printf("ok parse: %d texts (%d graphs, %d errors)\n", iters, ok_graphs, errors);
    return 0;
}

static int check_rank() {
    std::vector<uint32_t> sizes;
    for (uint32_t c = 1; c <= 2000; ++c) sizes.push_back(c);
    for (uint32_t c : {4095u, 4096u, 4097u, 65535u, 100003u}) sizes.push_back(c);
    for (uint32_t c : sizes) {
        const uint32_t words = (c + 31) / 32;
        std::vector<uint32_t> want(c);
        uint32_t r = 0;
        for (uint32_t bit = 0; bit < 32 && r < c; ++bit)
            for (uint32_t w = 0; w < words && r < c; ++w) {
                const uint32_t local = w * 32 + bit;
                if (local < c) want[r++] = local;
            }
        for (uint32_t k = 0; k < c; ++k)
            if (rank_to_local(k, c) != want[k]) {
                std::printf("differ: c=%u rank=%u: %u vs %u\n", c, k, rank_to_local(k, c), want[k]);
                return 1;
            }
    }
    std::printf("ok rank: %zu class sizes\n", sizes.size());
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 4 && std::string(argv[1]) == "parse") return check_parse(std::strtoull(argv[2], nullptr, 10), std::atoi(argv[3]));
    if (argc >= 2 && std::string(argv[1]) == "rank") return check_rank();
    std::fprintf(stderr, "usage: ingest_rules_check parse SEED ITERS | rank\n");
    return 2;
}
