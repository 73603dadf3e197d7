// Seeded synthetic labelled-graph generator writing the T-FSM `.lg` text format.
//
// Format (the loader of the reference, parallel/graph.h:572-660, requires this layout):
//   t N M                       first line
//   v <id> <label> <degree>     one per vertex, ids 0..N-1 in order
//   e <a> <b> <elabel>          one per undirected edge, a < b, no self-loops or multi-edges
//
// Degrees follow a Chung-Lu model: vertex i gets weight w_i = c * (i+1)^(-1/(gamma-1)),
// capped at max_degree, with c chosen so the mean weight is mean_degree.  Edges are sampled by
// drawing both endpoints proportionally to w until round(N*mean/2) distinct non-loop edges exist.
// Vertex labels are i.i.d. Zipf(s) over `labels` values 0..labels-1; edge labels are uniform over
// 1..elabels.  Vertex order is shuffled once so that label and degree are independent of the id.
//
// The output is bit-identical on every host: the only floating-point operations are IEEE
// +,-,*,/ (the power function is computed here from series, with FMA contraction disabled by the
// build), and all randomness comes from a splitmix64/xoshiro256** stream seeded by --seed.
// A 64-bit FNV-1a checksum of the produced edge list is printed so that fixtures can assert that
// they were made from the same graph.
//
// usage: gen_lg --out G.lg --n N --mean D --gamma G --max-degree X --labels L --zipf S
//               --elabels E --seed K [--arrays PREFIX]
// --arrays also writes the same graph as raw little-endian arrays, in the .lg file's order:
// PREFIX.vlabel (int32 per vertex), PREFIX.src / PREFIX.dst (uint32 per edge), PREFIX.elabel
// (int32 per edge) — the host buffers of tfsm_graph_from_edges without parsing text.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto &w : s) w = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform double in [0,1) with 53 random bits
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t n) { return next() % n; }
};

// ln(x) for x > 0 from frexp range reduction and the atanh series; only +,-,*,/ are used.
double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752) {
        m *= 2.0;
        e -= 1;
    }
    const double t = (m - 1.0) / (m + 1.0);
    const double t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 1; k < 60; k += 2) {
        sum += term / (double)k;
        term *= t2;
    }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

// exp(x) by range reduction x = k*ln2 + r, |r| <= ln2/2, then a Taylor series.
double det_exp(double x) {
    const double ln2 = 0.69314718055994530942;
    double kf = x / ln2;
    long k = (long)(kf >= 0 ? kf + 0.5 : kf - 0.5);
    const double r = x - (double)k * ln2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; ++i) {
        term = term * r / (double)i;
        sum += term;
    }
    return std::ldexp(sum, (int)k);
}

double det_pow(double base, double expo) { return det_exp(expo * det_log(base)); }

struct Args {
    std::string out;
    std::string arrays;  // prefix of the raw array files, or empty
    long n = 5000;
    double mean = 8.0;
    double gamma = 2.5;
    double max_degree = 500.0;
    int labels = 10;
    double zipf = 1.0;
    int elabels = 1;
    uint64_t seed = 0;
};

bool parse(int argc, char **argv, Args &a) {
    for (int i = 1; i + 1 < argc; i += 2) {
        const char *k = argv[i];
        const char *v = argv[i + 1];
        if (!std::strcmp(k, "--out")) a.out = v;
        else if (!std::strcmp(k, "--arrays")) a.arrays = v;
        else if (!std::strcmp(k, "--n")) a.n = std::atol(v);
        else if (!std::strcmp(k, "--mean")) a.mean = std::atof(v);
        else if (!std::strcmp(k, "--gamma")) a.gamma = std::atof(v);
        else if (!std::strcmp(k, "--max-degree")) a.max_degree = std::atof(v);
        else if (!std::strcmp(k, "--labels")) a.labels = std::atoi(v);
        else if (!std::strcmp(k, "--zipf")) a.zipf = std::atof(v);
        else if (!std::strcmp(k, "--elabels")) a.elabels = std::atoi(v);
        else if (!std::strcmp(k, "--seed")) a.seed = std::strtoull(v, nullptr, 10);
        else {
            std::fprintf(stderr, "unknown option %s\n", k);
            return false;
        }
    }
    if (a.out.empty() || a.n < 2 || a.mean <= 0 || a.gamma <= 1.0 || a.labels < 1 || a.elabels < 1) {
        std::fprintf(stderr, "bad arguments\n");
        return false;
    }
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    Args a;
    if (!parse(argc, argv, a)) return 2;
    const long n = a.n;
    Rng rng(a.seed * 0x100000001B3ULL + 12345);

    // Chung-Lu weights, capped; rescale so that the capped mean equals the requested mean.
    const double alpha = 1.0 / (a.gamma - 1.0);
    std::vector<double> raw(n);
    double raw_sum = 0.0;
    for (long i = 0; i < n; ++i) {
        raw[i] = det_pow((double)(i + 1), -alpha);
        raw_sum += raw[i];
    }
    double c = a.mean * (double)n / raw_sum;
    std::vector<double> w(n);
    for (int it = 0; it < 60; ++it) {
        double s = 0.0;
        for (long i = 0; i < n; ++i) {
            double x = c * raw[i];
            w[i] = x < a.max_degree ? x : a.max_degree;
            s += w[i];
        }
        const double target = a.mean * (double)n;
        if (s >= target * 0.999999) break;
        c *= target / s;
    }

    // Vertex ids are a random permutation of weight ranks.
    std::vector<long> perm(n);
    for (long i = 0; i < n; ++i) perm[i] = i;
    for (long i = n - 1; i > 0; --i) {
        long j = (long)rng.below((uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
    }
    std::vector<double> cdf(n);
    double acc = 0.0;
    for (long i = 0; i < n; ++i) {
        acc += w[perm[i]];
        cdf[i] = acc;
    }
    const double total = acc;
    auto draw = [&]() -> uint32_t {
        const double x = rng.uniform() * total;
        const long i = (long)(std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin());
        return (uint32_t)(i < n ? i : n - 1);
    };

    const uint64_t m_target = (uint64_t)((double)n * a.mean / 2.0 + 0.5);
    std::vector<uint64_t> keys;
    keys.reserve(m_target + m_target / 8);
    for (int round = 0; round < 64 && keys.size() < m_target; ++round) {
        const uint64_t need = m_target - keys.size();
        for (uint64_t k = 0; k < need; ++k) {
            uint32_t x = draw(), y = draw();
            if (x == y) continue;
            if (x > y) std::swap(x, y);
            keys.push_back(((uint64_t)x << 32) | y);
        }
        std::sort(keys.begin(), keys.end());
        keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    }
    if (keys.size() > m_target) {
        // Drop a deterministic random subset so that exactly m_target edges remain.
        for (uint64_t i = keys.size() - 1; i > 0; --i) {
            uint64_t j = rng.below(i + 1);
            std::swap(keys[i], keys[j]);
        }
        keys.resize(m_target);
        std::sort(keys.begin(), keys.end());
    }

    // Labels.
    std::vector<double> zc(a.labels);
    double zs = 0.0;
    for (int k = 0; k < a.labels; ++k) {
        zs += det_pow((double)(k + 1), -a.zipf);
        zc[k] = zs;
    }
    std::vector<int> vlabel(n);
    for (long i = 0; i < n; ++i) {
        const double x = rng.uniform() * zs;
        int k = (int)(std::upper_bound(zc.begin(), zc.end(), x) - zc.begin());
        vlabel[i] = k < a.labels ? k : a.labels - 1;
    }
    std::vector<int> elabel(keys.size());
    for (size_t e = 0; e < keys.size(); ++e) elabel[e] = 1 + (int)rng.below((uint64_t)a.elabels);

    std::vector<uint32_t> deg(n, 0);
    for (uint64_t k : keys) {
        deg[k >> 32]++;
        deg[k & 0xffffffffu]++;
    }

    FILE *f = std::fopen(a.out.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", a.out.c_str());
        return 1;
    }
    std::vector<char> buf(1 << 22);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    std::fprintf(f, "t %ld %zu\n", n, keys.size());
    for (long i = 0; i < n; ++i) std::fprintf(f, "v %ld %d %u\n", i, vlabel[i], deg[i]);
    uint64_t h = 1469598103934665603ULL;
    auto mix = [&](uint64_t x) {
        for (int b = 0; b < 8; ++b) {
            h ^= (x >> (8 * b)) & 0xff;
            h *= 1099511628211ULL;
        }
    };
    for (size_t e = 0; e < keys.size(); ++e) {
        const uint32_t x = (uint32_t)(keys[e] >> 32), y = (uint32_t)(keys[e] & 0xffffffffu);
        std::fprintf(f, "e %u %u %d\n", x, y, elabel[e]);
        mix(keys[e]);
        mix((uint64_t)elabel[e]);
    }
    for (long i = 0; i < n; ++i) mix((uint64_t)vlabel[i]);
    std::fclose(f);
    if (!a.arrays.empty()) {
        auto dump = [&](const char *ext, const void *data, size_t bytes) {
            FILE *g = std::fopen((a.arrays + ext).c_str(), "wb");
            const bool ok = g && std::fwrite(data, 1, bytes, g) == bytes;
            if (g) std::fclose(g);
            return ok;
        };
        std::vector<uint32_t> src(keys.size()), dst(keys.size());
        for (size_t e = 0; e < keys.size(); ++e) {
            src[e] = (uint32_t)(keys[e] >> 32);
            dst[e] = (uint32_t)(keys[e] & 0xffffffffu);
        }
        if (!dump(".vlabel", vlabel.data(), vlabel.size() * sizeof(vlabel[0])) ||
            !dump(".src", src.data(), src.size() * 4) || !dump(".dst", dst.data(), dst.size() * 4) ||
            !dump(".elabel", elabel.data(), elabel.size() * sizeof(elabel[0]))) {
            std::fprintf(stderr, "cannot write the arrays %s.*\n", a.arrays.c_str());
            return 1;
        }
    }
    uint32_t maxdeg = 0;
    for (long i = 0; i < n; ++i) maxdeg = deg[i] > maxdeg ? deg[i] : maxdeg;
    std::printf("{\"n\": %ld, \"m\": %zu, \"max_degree\": %u, \"fnv64\": \"%016llx\"}\n", n, keys.size(), maxdeg,
                (unsigned long long)h);
    return 0;
}
