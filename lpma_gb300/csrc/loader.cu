// Edgelist and query files of the reference's drivers (host code only).
//
// Edgelist (README.md:9-20): "N E", then E lines "src dst".  Timestamps: E
// integers, one per edge, in edge order (read_edgelist_and_timestamps,
// test.cu:191-221).  Queries: "Q", then Q lines "src lb ub" (read_queries,
// test.cu:223-241).  Whitespace of any kind separates numbers.  The whole
// file is read in one go and parsed without the C++ stream machinery (the
// reference's ifstream >> parses a few MB/s).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "lpma.h"

namespace {

constexpr uint64_t SRC_SHIFT = 42, DST_SHIFT = 20;
constexpr uint64_t MAX_ID = 0x3FFFFE;  // the sentinel's dst (NBR_END)
constexpr uint64_t MAX_T = 1ull << 20;

bool read_file(const char *path, std::vector<char> &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    buf.clear();
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    buf.push_back('\0');
    return ok;
}

// Unsigned decimal numbers separated by whitespace.
struct Scanner {
    const char *p;
    bool next(uint64_t &x) {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++;
        if (*p < '0' || *p > '9') return false;
        uint64_t v = 0;
        while (*p >= '0' && *p <= '9') {
            const uint64_t d = (uint64_t)(*p - '0');
            if (v > (UINT64_MAX - d) / 10) return false;
            v = v * 10 + d;
            p++;
        }
        if (*p != '\0' && *p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') return false;
        x = v;
        return true;
    }
};

}  // namespace

extern "C" {

lpma_status_t lpma_read_edgelist(const char *path, const char *timestamps_path, uint64_t *h_keys, size_t cap,
                                 uint32_t *num_vertices, size_t *num_edges) {
    if (!path || !num_vertices || !num_edges) return LPMA_ERR_INVALID_ARGUMENT;
    std::vector<char> buf;
    if (!read_file(path, buf)) return LPMA_ERR_IO;
    Scanner sc{buf.data()};
    uint64_t N = 0, E = 0;
    if (!sc.next(N) || !sc.next(E) || N > MAX_ID) return LPMA_ERR_IO;
    *num_vertices = (uint32_t)N;
    *num_edges = (size_t)E;
    if (E > cap) return LPMA_ERR_BUFFER_TOO_SMALL;
    if (E && !h_keys) return LPMA_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < E; i++) {
        uint64_t s, d;
        if (!sc.next(s) || !sc.next(d) || s >= N || d >= N) return LPMA_ERR_IO;
        h_keys[i] = s << SRC_SHIFT | d << DST_SHIFT;
    }
    if (timestamps_path) {
        std::vector<char> tb;
        if (!read_file(timestamps_path, tb)) return LPMA_ERR_IO;
        Scanner ts{tb.data()};
        for (uint64_t i = 0; i < E; i++) {
            uint64_t t;
            if (!ts.next(t) || t >= MAX_T) return LPMA_ERR_IO;
            h_keys[i] |= t;
        }
    }
    return LPMA_OK;
}

lpma_status_t lpma_read_queries(const char *path, uint32_t *h_srcs, uint64_t *h_windows, size_t cap,
                                size_t *num_queries) {
    if (!path || !num_queries) return LPMA_ERR_INVALID_ARGUMENT;
    std::vector<char> buf;
    if (!read_file(path, buf)) return LPMA_ERR_IO;
    Scanner sc{buf.data()};
    uint64_t Q = 0;
    if (!sc.next(Q)) return LPMA_ERR_IO;
    *num_queries = (size_t)Q;
    if (Q > cap) return LPMA_ERR_BUFFER_TOO_SMALL;
    if (Q && (!h_srcs || !h_windows)) return LPMA_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < Q; i++) {
        uint64_t s, lb, ub;
        if (!sc.next(s) || !sc.next(lb) || !sc.next(ub) || s >= MAX_ID || lb > 0xFFFFFFFFull || ub > 0xFFFFFFFFull)
            return LPMA_ERR_IO;
        h_srcs[i] = (uint32_t)s;
        h_windows[i] = lb << 32 | ub;
    }
    return LPMA_OK;
}

}  // extern "C"
