// Text data loader: loadtxtData (src/Utilities.cpp:57-95) without the
// transform (the fit applies it).  The file holds n_points lines of
// n_features whitespace-separated numbers; point n's values fill column n of
// the d x n column-major matrix, i.e. X_dxn[n * d + j] is the j-th number of
// line n.  Numbers are parsed with strtof (correctly rounded, the conversion
// fscanf("%f") performs).  The file is read once and parsed by several host
// threads: it is cut at whitespace into chunks, each chunk's numbers are
// counted, and each thread parses its chunk into its offset.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/sdbscan_gb300.h"

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Numbers in [b, e); each number starts after whitespace or at b.
size_t count_numbers(const char* b, const char* e) {
    size_t c = 0;
    bool in = false;
    for (const char* p = b; p < e; ++p) {
        const bool sp = is_space(*p);
        if (!sp && !in) ++c;
        in = !sp;
    }
    return c;
}

// Parses up to `want` numbers of [b, e) into out; returns how many parsed.
size_t parse_numbers(const char* b, const char* e, float* out, size_t want) {
    size_t c = 0;
    const char* p = b;
    while (c < want) {
        while (p < e && is_space(*p)) ++p;
        if (p >= e) break;
        char* end = nullptr;
        const float v = std::strtof(p, &end);
        if (end == p) break;  // not a number
        out[c++] = v;
        p = end;
    }
    return c;
}

}  // namespace

extern "C" sdb_status sdb_load_txt(const char* path, int32_t n_points, int32_t n_features, float* X_dxn) {
    if (!path || !X_dxn || n_points < 1 || n_features < 1) return SDB_ERR_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return SDB_ERR_ARG;
    std::vector<char> buf;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long sz = std::ftell(f);
        if (sz > 0) {
            buf.resize((size_t)sz + 1);
            std::fseek(f, 0, SEEK_SET);
            buf.resize(std::fread(buf.data(), 1, (size_t)sz, f) + 1);
        }
    }
    std::fclose(f);
    if (buf.empty()) return SDB_ERR_ARG;
    buf.back() = '\0';  // strtof stops at the terminator
    const char* b = buf.data();
    const char* e = b + buf.size() - 1;
    const size_t want = (size_t)n_points * (size_t)n_features;

    // chunk boundaries at whitespace
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt == 0 ? 1 : (nt > 64 ? 64 : nt);
    if ((size_t)(e - b) < ((size_t)1 << 20)) nt = 1;
    std::vector<const char*> cut(nt + 1);
    cut[0] = b;
    cut[nt] = e;
    for (unsigned t = 1; t < nt; ++t) {
        const char* p = b + (size_t)(e - b) * t / nt;
        if (p < cut[t - 1]) p = cut[t - 1];
        while (p < e && !is_space(*p)) ++p;
        cut[t] = p;
    }
    std::vector<size_t> cnt(nt), off(nt + 1, 0);
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t) th.emplace_back([&, t] { cnt[t] = count_numbers(cut[t], cut[t + 1]); });
        for (auto& x : th) x.join();
    }
    for (unsigned t = 0; t < nt; ++t) off[t + 1] = off[t] + cnt[t];
    if (off[nt] < want) return SDB_ERR_ARG;  // fewer numbers than n_points x n_features
    std::vector<size_t> got(nt, 0);
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t] {
                if (off[t] >= want) return;
                const size_t take = std::min(cnt[t], want - off[t]);
                got[t] = parse_numbers(cut[t], cut[t + 1], X_dxn + off[t], take);
            });
        for (auto& x : th) x.join();
    }
    for (unsigned t = 0; t < nt; ++t) {
        if (off[t] >= want) break;
        if (got[t] != std::min(cnt[t], want - off[t])) return SDB_ERR_ARG;  // a token that is not a number
    }
    return SDB_OK;
}
