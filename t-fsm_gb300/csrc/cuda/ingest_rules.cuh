// Rules of the GPU ingestion that the host loader defines, shared by the ingestion kernels
// (cuda/ingest.cu) and CPU tests that compare them with the host code they restate.
//
// 1. One `.lg` line, parsed the way host/lg_graph.hpp `parse_lg_text` parses it (which follows
// parallel/graph.h:557-616).
// A line is the bytes [ls, le) before the newline at le.  Leading spaces are skipped; an empty
// line, one whose first other byte is '\r', a 't' line and a '#' line carry nothing.  'v' and 'e'
// lines carry two and three integer tokens; any other first byte is an error.  A token is a run
// of bytes other than ' ' and '\n', and its value is what C's strtol(token, nullptr, 10) returns
// when reading the whole buffer from the token's first byte: leading white space (which may run
// past the token and the line), an optional sign, decimal digits, saturation at the 64-bit range,
// 0 when no digit follows.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define TFSM_HD __host__ __device__ __forceinline__
#else
#define TFSM_HD inline
#endif

namespace tfsm {
namespace lgparse {

enum LineKind : uint8_t {
    kNone = 0,          // blank, 't' or '#'
    kVertex = 1,        // v id label
    kEdge = 2,          // e a b label
    kBadVertex = 3,     // malformed vertex line
    kBadEdge = 4,       // malformed edge line
    kUnknown = 5,       // unknown line kind
};

struct Line {
    uint8_t kind = kNone;
    int64_t v[3] = {0, 0, 0};  // vertex: id, label; edge: a, b, label
};

TFSM_HD bool c_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// strtol(buf + p, nullptr, 10) for a buffer of `size` bytes (reading stops at its end).
TFSM_HD int64_t c_strtol(const char *buf, uint64_t p, uint64_t size) {
    while (p < size && c_space(buf[p])) ++p;
    bool neg = false;
    if (p < size && (buf[p] == '+' || buf[p] == '-')) {
        neg = buf[p] == '-';
        ++p;
    }
    // magnitude limit: 2^63 - 1, or 2^63 for a negative value
    const uint64_t limit = neg ? (uint64_t)1 << 63 : ((uint64_t)1 << 63) - 1;
    uint64_t acc = 0;
    bool any = false, over = false;
    while (p < size && buf[p] >= '0' && buf[p] <= '9') {
        const uint64_t d = (uint64_t)(buf[p] - '0');
        any = true;
        if (!over) {
            if (acc > (limit - d) / 10) over = true;
            else acc = acc * 10 + d;
        }
        ++p;
    }
    if (!any) return 0;
    if (over) return neg ? (int64_t)((uint64_t)1 << 63) : (int64_t)(((uint64_t)1 << 63) - 1);
    return neg ? (int64_t)(0 - acc) : (int64_t)acc;
}

// The next token of the line from r (advanced past it); ok = false when the line has none left.
TFSM_HD int64_t next_int(const char *buf, uint64_t size, uint64_t &r, uint64_t le, bool &ok) {
    while (r < le && buf[r] == ' ') ++r;
    if (r >= le || buf[r] == '\n') {
        ok = false;
        return 0;
    }
    const uint64_t tok = r;
    while (r < le && buf[r] != ' ' && buf[r] != '\n') ++r;
    ok = true;
    return c_strtol(buf, tok, size);
}

TFSM_HD Line parse_line(const char *buf, uint64_t size, uint64_t ls, uint64_t le) {
    Line L;
    uint64_t q = ls;
    while (q < le && buf[q] == ' ') ++q;
    if (q >= le || buf[q] == '\r') return L;
    const char kind = buf[q];
    uint64_t r = q + 1;
    bool ok1 = false, ok2 = false, ok3 = false;
    if (kind == 't' || kind == '#') return L;
    if (kind == 'v') {
        L.v[0] = next_int(buf, size, r, le, ok1);
        L.v[1] = next_int(buf, size, r, le, ok2);
        L.kind = (!ok1 || !ok2 || L.v[0] < 0) ? kBadVertex : kVertex;
    } else if (kind == 'e') {
        L.v[0] = next_int(buf, size, r, le, ok1);
        L.v[1] = next_int(buf, size, r, le, ok2);
        L.v[2] = next_int(buf, size, r, le, ok3);
        L.kind = (!ok1 || !ok2 || !ok3 || L.v[0] < 0 || L.v[1] < 0) ? kBadEdge : kEdge;
    } else {
        L.kind = kUnknown;
    }
    return L;
}

}  // namespace lgparse

// 2. The internal id of a vertex of rank r (by descending degree) among the c vertices of its
// label, relative to the label's first id: the GpuEngine constructor's host loop fills the label's
// bitmap words column by column (bit 0 of every word, then bit 1, ...), and the last word holds
// only rem = c - 32 (words - 1) ids, so bits >= rem skip it.
TFSM_HD uint32_t rank_to_local(uint32_t r, uint32_t c) {
    const uint32_t words = (c + 31) / 32, rem = c - 32 * (words - 1);
    uint32_t bit, w;
    if (r < rem * words) {
        bit = r / words;
        w = r % words;
    } else {
        const uint32_t r2 = r - rem * words;
        bit = rem + r2 / (words - 1);
        w = r2 % (words - 1);
    }
    return w * 32 + bit;
}

}  // namespace tfsm
