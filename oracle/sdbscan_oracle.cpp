// ORACLE — test infrastructure, not product code.
//
// A from-scratch CPU restatement of the sDbscan / sOPTICS hot path of the
// reference (NinhPham/sDbscan), stage by stage, each function citing the
// reference lines it follows.  Only the tests, the smoke check and the CPU
// baseline leg of bench.py load it, and only as the checker / the timed CPU
// arm; the product never calls it.
//
// Parity pin: it is checked against the reference itself (its unmodified
// sources compiled against oracle/shim, see oracle/Makefile) through the
// golden fixtures in tests/golden, and directly against oracle/_ref where that
// library exists.  Numerical contract, identical to the shim's: dot products
// and squared norms are sequential fmaf over ascending index; sums are
// sequential adds; the Walsh-Hadamard transform is the radix-2 form with
// ascending strides (bit-identical to the reference's fht_float).
//
// Portable C++17 + OpenMP: builds and gives the same bits on x86-64 and
// aarch64 (-ffp-contract=off, explicit std::fma).
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <queue>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

namespace {

enum Dist { D_COSINE = 0, D_L1 = 1, D_L2 = 2, D_CHI2 = 3, D_JS = 4 };

const double kPI = 3.141592653589793238460;  // src/Header.h:19
const float kNegInf = -2147483648.0f;         // src/Header.h:20
const float kJsEps = 0.000001f;               // src/Header.h:22, converted to float by the array update

// Timing mode of the CPU baseline (orc_set_timing_mode).  The reference
// computes Cosine, L1 and L2 with Eigen expressions (src/Utilities.h:215,
// :217, :219) that real Eigen evaluates with SIMD partial sums; the
// sequential order of the numerical contract is what a checker needs but runs
// slower than that.  With the mode on, those three distances use 16 partial
// sums that the compiler vectorises on any target, so the timed CPU path runs
// at the speed of the reference's own build.  Its last bits differ from the
// contract's: the mode is for timing only and is off unless a timing leg
// turns it on.  Chi2 and JS are scalar loops in the reference too.
int g_timing_mode = 0;

template <int CODE>
float distance_lanes(const float* x, const float* y, int d) {
    float acc[16] = {0.0f};
    int i = 0;
    for (; i + 16 <= d; i += 16)
        for (int j = 0; j < 16; ++j) {
            const float a = x[i + j], b = y[i + j];
            if (CODE == D_COSINE) acc[j] += a * b;
            else if (CODE == D_L1) acc[j] += std::fabs(a - b);
            else acc[j] += (a - b) * (a - b);
        }
    float s = 0.0f;
    for (; i < d; ++i) {
        const float a = x[i], b = y[i];
        s += CODE == D_COSINE ? a * b : CODE == D_L1 ? std::fabs(a - b) : (a - b) * (a - b);
    }
    for (int j = 0; j < 16; ++j) s += acc[j];
    return CODE == D_COSINE ? 1 - s : CODE == D_L1 ? s : std::sqrt(s);
}

// computeDist (src/Utilities.h:212-287).
float distance(const float* x, const float* y, int d, int code) {
    if (g_timing_mode) {
        if (code == D_COSINE) return distance_lanes<D_COSINE>(x, y, d);
        if (code == D_L1) return distance_lanes<D_L1>(x, y, d);
        if (code == D_L2) return distance_lanes<D_L2>(x, y, d);
    }
    switch (code) {
        case D_COSINE: {  // 1 - x.y  (:214-215)
            float s = 0.0f;
            for (int i = 0; i < d; ++i) s = std::fma(x[i], y[i], s);
            return 1 - s;
        }
        case D_L1: {  // sum |x - y|  (:216-217)
            float s = 0.0f;
            for (int i = 0; i < d; ++i) s = s + std::fabs(x[i] - y[i]);
            return s;
        }
        case D_L2: {  // ||x - y||  (:218-219)
            float s = 0.0f;
            for (int i = 0; i < d; ++i) {
                const float t = x[i] - y[i];
                s = std::fma(t, t, s);
            }
            return std::sqrt(s);
        }
        case D_CHI2: {  // 1 - 2 sum_{x,y>0} xy/(x+y)  (:220-243)
            float t = 0.0f;
            for (int i = 0; i < d; ++i)
                if (x[i] > 0 && y[i] > 0) t = t + (x[i] * y[i]) / (x[i] + y[i]);
            return (float)(1.0 - 2.0 * (double)t);
        }
        case D_JS: {  // (:245-266), elementwise with EPSILON added to both
            const float l2 = (float)std::log(2.0);
            float s = 0.0f;
            for (int i = 0; i < d; ++i) {
                const float a = x[i] + kJsEps, b = y[i] + kJsEps;
                const float t1 = (std::log((a + b) / a) / l2) * a;
                const float t2 = (std::log((a + b) / b) / l2) * b;
                s = s + (t1 + t2);
            }
            return (float)(1.0 - (double)s / 2.0);
        }
    }
    return 0.0f;
}

// In-place radix-2 Walsh-Hadamard transform, strides 1, 2, 4, ... (the order
// the reference's fht_float reproduces bit for bit; src/fht.h:11).
void fwht(float* v, int N) {
    for (int h = 1; h < N; h <<= 1)
        for (int i = 0; i < N; i += 2 * h)
            for (int j = i; j < i + h; ++j) {
                const float a = v[j], b = v[j + h];
                v[j] = a + b;
                v[j + h] = a - b;
            }
}

// Kernel embedding of one point (src/sDbscan.cpp:53-68; embedChi2
// src/Utilities.h:132-164; embedJS :174-208).  `out` has ker zeros on entry.
void embed(const float* x, int d, int code, int ker, float L, const float* R, float* out) {
    if (code == D_COSINE) {
        std::memcpy(out, x, sizeof(float) * d);
    } else if (code == D_L1 || code == D_L2) {
        const int h = ker / 2;
        for (int r = 0; r < h; ++r) {  // R is h x d column-major
            float s = 0.0f;
            for (int c = 0; c < d; ++c) s = std::fma(R[(size_t)c * h + r], x[c], s);
            out[r] = std::cos(s);
            out[h + r] = std::sin(s);
        }
    } else if (code == D_CHI2 || code == D_JS) {
        int comps = (ker / d) - 1;
        comps /= 2;
        for (int i = 0; i < d; ++i)
            if (x[i] > 0) {
                if (code == D_CHI2) out[i] = std::sqrt(x[i] * L);
                else out[i] = (float)std::sqrt((double)(x[i] * L) * 2.0 / std::log(4.0));
            }
        for (int c = 1; c <= comps; ++c) {
            const int base = d + (c - 1) * 2 * d;
            for (int i = 0; i < d; ++i) {
                if (!(x[i] > 0)) continue;
                float f;
                if (code == D_CHI2) {
                    f = (float)std::sqrt(2.0 * (double)x[i] * (double)L / std::cosh(kPI * c * (double)L));
                } else {
                    const float cl = c * L;
                    const float q = 1 + 4 * cl * cl;
                    f = (float)(2.0 / (std::log(4.0) * (double)q * std::cosh(kPI * c * (double)L)));
                    f = (float)std::sqrt(2.0 * (double)x[i] * (double)L * (double)f);
                }
                const float ang = (c * L) * std::log(x[i]);
                out[base + i] = f * std::cos(ang);
                out[base + d + i] = f * std::sin(ang);
            }
        }
    }
}

// Fixed-size min-heap top-k with the reference's exact replacement rule:
// fill to k, then replace the minimum only on strict `>` (src/sDbscan.cpp:111-132).
// Comparisons look at the value only, as IFPair does (src/Header.h:56-69).
struct ValIdx {
    float v;
    int i;
};
struct GreaterVal {
    bool operator()(const ValIdx& a, const ValIdx& b) const { return a.v > b.v; }
};
typedef std::priority_queue<ValIdx, std::vector<ValIdx>, GreaterVal> MinHeap;

inline void heap_offer(MinHeap& h, int k, int idx, float v) {
    if ((int)h.size() < k) h.push({v, idx});
    else if (v > h.top().v) {
        h.pop();
        h.push({v, idx});
    }
}

struct Timer {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double lap() {
        auto t = std::chrono::steady_clock::now();
        double s = std::chrono::duration<double>(t - t0).count();
        t0 = t;
        return s;
    }
};

}  // namespace

extern "C" {

// ---- host RNG (src/Utilities.h:47-64, :76-93, :105-122) ----------------------

void orc_hd3_bits(int nbits, int seed, uint8_t* out) {
    std::default_random_engine gen((unsigned)seed);
    std::uniform_int_distribution<uint32_t> u(0, 1);
    for (int i = 0; i < nbits; ++i) out[i] = (uint8_t)(u(gen) & 1);
}

// rows x cols column-major, filled column first like the reference.
void orc_gauss(int rows, int cols, float mean, float stddev, int seed, float* out) {
    std::default_random_engine gen((unsigned)seed);
    std::normal_distribution<float> nd(mean, stddev);
    for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r) out[(size_t)c * rows + r] = nd(gen);
}

void orc_cauchy(int rows, int cols, float x0, float gamma, int seed, float* out) {
    std::default_random_engine gen((unsigned)seed);
    std::cauchy_distribution<float> cd(x0, gamma);
    for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r) out[(size_t)c * rows + r] = cd(gen);
}

// embedChi2 / embedJS fill the first d slots of a ker-long vector
// (src/Utilities.h:140-145), so the reference requires ker >= d
// (src/sDbscan.cpp:54) and overruns the vector otherwise.  Returns 3 for such
// parameters (the whole-fit entry points return -3), else 0.
static int embed_precondition(int code, int ker, int d) {
    return (code == D_CHI2 || code == D_JS) && ker < d ? 3 : 0;
}

// ---- transformData (src/Utilities.h:289-335) ---------------------------------
// X: d x n column-major, modified in place.  Returns 0, or 1 (negative value)
// / 2 (zero-sum column) where the reference prints an error and exits.
int orc_transform(float* X, int n, int d, int code) {
    if (code == D_COSINE) {
#pragma omp parallel for
        for (int p = 0; p < n; ++p) {
            float* x = X + (size_t)p * d;
            float s = 0.0f;
            for (int i = 0; i < d; ++i) s = std::fma(x[i], x[i], s);
            const float nrm = std::sqrt(s);
            for (int i = 0; i < d; ++i) x[i] = x[i] / nrm;
        }
    } else if (code == D_CHI2 || code == D_JS) {
        for (size_t i = 0; i < (size_t)n * d; ++i)
            if (X[i] < 0) return 1;
        int bad = 0;
#pragma omp parallel for reduction(| : bad)
        for (int p = 0; p < n; ++p) {
            float* x = X + (size_t)p * d;
            float s = 0.0f;
            for (int i = 0; i < d; ++i) s = s + x[i];
            if (s <= 0) {
                bad = 1;
                continue;
            }
            for (int i = 0; i < d; ++i) x[i] = x[i] / s;
        }
        if (bad) return 2;
    }
    return 0;
}

// ---- projection (src/sDbscan.cpp:46-91) --------------------------------------
// X: transformed data, d x n column-major.  bits: 3*fhtDim signs (0/1).
// R: (ker/2) x d column-major (L1/L2 only).  out: n x nproj, point-major
// (point p's projections contiguous) == the reference's MATRIX_FHT (nproj x n
// column-major).
void orc_project(const float* X, int n, int d, int code, int ker, float L, const float* R, const uint8_t* bits,
                 int fhtDim, int nproj, float* out) {
#pragma omp parallel
    {
        std::vector<float> v(fhtDim);
#pragma omp for
        for (int p = 0; p < n; ++p) {
            std::fill(v.begin(), v.end(), 0.0f);
            embed(X + (size_t)p * d, d, code, ker, L, R, v.data());
            for (int r = 0; r < 3; ++r) {
                for (int i = 0; i < fhtDim; ++i) v[i] *= (float)(2 * (int)bits[r * fhtDim + i] - 1);
                fwht(v.data(), fhtDim);
            }
            std::memcpy(out + (size_t)p * nproj, v.data(), sizeof(float) * nproj);
        }
    }
}

// ---- per-point top-k (src/sDbscan.cpp:97-143) --------------------------------
// P: n x nproj point-major.  topK: n x 2k point-major (== the reference's
// matrix_topK, 2k x n column-major); row 0 is the most extreme.
void orc_topk(const float* P, int n, int nproj, int k, int* topK) {
#pragma omp parallel for
    for (int p = 0; p < n; ++p) {
        MinHeap close, far;
        const float* v = P + (size_t)p * nproj;
        for (int r = 0; r < nproj; ++r) {
            heap_offer(close, k, r, v[r]);
            heap_offer(far, k, r, -v[r]);
        }
        int* o = topK + (size_t)p * 2 * k;
        for (int j = k - 1; j >= 0; --j) {
            o[j] = close.top().i;
            close.pop();
            o[j + k] = far.top().i;
            far.pop();
        }
    }
}

// ---- per-vector top-m (src/sDbscan.cpp:151-208) ------------------------------
// topM: nproj x 2m vector-major (== matrix_topM, 2m x nproj column-major).
void orc_topm(const float* P, int n, int nproj, int m, int* topM) {
#pragma omp parallel for
    for (int r = 0; r < nproj; ++r) {
        MinHeap close, far;
        for (int p = 0; p < n; ++p) {
            const float v = P[(size_t)p * nproj + r];
            heap_offer(close, m, p, v);
            heap_offer(far, m, p, -v);
        }
        int* o = topM + (size_t)r * 2 * m;
        for (int j = m - 1; j >= 0; --j) {
            o[j] = close.top().i;
            close.pop();
            o[j + m] = far.top().i;
            far.pop();
        }
    }
}

// ---- canonical tie rule for the selections ----------------------------------
// The reference's heaps (strict `>` replacement, src/sDbscan.cpp:115, :127,
// :178, :190) keep, among values equal to the k-th, the ones that the heap's
// internal order leaves in it.  The GPU engine keeps the smallest indices
// instead.  These two selections state that rule: the k largest by (value
// desc, index asc) (and the k smallest by (value asc, index asc) for the far
// side).  Where no boundary tie occurs they equal orc_topk / orc_topm as
// sets; where one does they are the engine's sets, so a whole fit can be
// checked bit for bit through the tie.  Rows are written in (value, index)
// order: row 0 is the most extreme.
extern "C++" {
namespace {
// "a ranks above b" for the close side: larger value, then smaller index.
inline bool ranks_above(float av, int ai, float bv, int bi) { return av > bv || (av == bv && ai < bi); }
struct WorstOnTop {  // heap top = the lowest-ranked kept entry
    bool operator()(const ValIdx& a, const ValIdx& b) const { return ranks_above(a.v, a.i, b.v, b.i); }
};
typedef std::priority_queue<ValIdx, std::vector<ValIdx>, WorstOnTop> CanonHeap;
inline void canon_offer(CanonHeap& h, int k, int idx, float v) {
    if ((int)h.size() < k) h.push({v, idx});
    else if (ranks_above(v, idx, h.top().v, h.top().i)) {
        h.pop();
        h.push({v, idx});
    }
}
inline void canon_drain(CanonHeap& h, int k, int* out) {
    for (int j = k - 1; j >= 0; --j) {
        out[j] = h.top().i;
        h.pop();
    }
}
}  // namespace
}  // extern "C++"

void orc_topk_canon(const float* P, int n, int nproj, int k, int* topK) {
#pragma omp parallel for
    for (int p = 0; p < n; ++p) {
        CanonHeap close, far;
        const float* v = P + (size_t)p * nproj;
        for (int r = 0; r < nproj; ++r) {
            canon_offer(close, k, r, v[r]);
            canon_offer(far, k, r, -v[r]);
        }
        canon_drain(close, k, topK + (size_t)p * 2 * k);
        canon_drain(far, k, topK + (size_t)p * 2 * k + k);
    }
}

void orc_topm_canon(const float* P, int n, int nproj, int m, int* topM) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < nproj; ++r) {
        CanonHeap close, far;
        for (int p = 0; p < n; ++p) {
            const float v = P[(size_t)p * nproj + r];
            canon_offer(close, m, p, v);
            canon_offer(far, m, p, -v);
        }
        canon_drain(close, m, topM + (size_t)r * 2 * m);
        canon_drain(far, m, topM + (size_t)r * 2 * m + m);
    }
}

// ---- core points (src/sDbscan.cpp:217-408) -----------------------------------
// Computes, for every point, its de-duplicated symmetric eps-neighbourhood
// (own candidates within eps, plus every point that found it as a candidate
// within eps), the core flag (|N| >= minPts - 1) and |N|.
// Outputs: core[n], degree[n]; neighbour lists are kept internally and can be
// read with orc_neighbors_* (sorted ascending, for every point).
struct Graph {
    std::vector<std::vector<int>> nb;
    std::vector<std::vector<float>> nd;  // distances (only when with_dist)
};
static Graph g_graph;

// ref_order=1 keeps each list in the order the reference leaves it: the push
// sequence de-duplicated through std::unordered_map<int, float> (:1428-1431)
// and read back in the map's iteration order.  With one thread the push
// sequence is the reference's own, so the lists match it element for element.
void orc_find_core(const float* X, int n, int d, int code, const int* topK, int k, const int* topM, int m, float eps,
                   int minPts, int with_dist, int ref_order, uint8_t* core, int32_t* degree) {
    std::vector<std::vector<std::pair<int, float>>> nb(n);
#pragma omp parallel
    {
        std::vector<uint64_t> seen(((size_t)n + 63) / 64);
#pragma omp for schedule(dynamic, 64)
        for (int p = 0; p < n; ++p) {
            std::fill(seen.begin(), seen.end(), 0ull);  // per-point n-bit set (:260)
            const float* xp = X + (size_t)p * d;
            for (int j = 0; j < k; ++j) {
                for (int side = 0; side < 2; ++side) {  // close list then far list (:262-356)
                    const int r = topK[(size_t)p * 2 * k + j + side * k];
                    for (int i = 0; i < m; ++i) {
                        const int q = topM[(size_t)r * 2 * m + i + side * m];
                        if (q == p) continue;  // (:272)
                        if (seen[q >> 6] >> (q & 63) & 1) continue;
                        seen[q >> 6] |= 1ull << (q & 63);
                        const float dist = distance(xp, X + (size_t)q * d, d, code);
                        if (dist <= eps) {  // (:286-296)
#pragma omp critical
                            {
                                nb[p].push_back({q, dist});
                                nb[q].push_back({p, dist});
                            }
                        }
                    }
                }
            }
        }
    }
    g_graph.nb.assign(n, {});
    g_graph.nd.assign(n, {});
#pragma omp parallel for schedule(dynamic, 256)
    for (int p = 0; p < n; ++p) {  // de-duplicate + core flag (:374-400)
        auto& l = nb[p];
        std::vector<int> ids;
        std::vector<float> ds;
        if (ref_order) {
            std::unordered_map<int, float> mp(l.begin(), l.end());
            for (const auto& e : mp) {
                ids.push_back(e.first);
                ds.push_back(e.second);
            }
        } else {
            std::sort(l.begin(), l.end(), [](const std::pair<int, float>& a, const std::pair<int, float>& b) {
                return a.first < b.first;
            });
            for (size_t t = 0; t < l.size(); ++t)
                if (t == 0 || l[t].first != l[t - 1].first) {
                    ids.push_back(l[t].first);
                    ds.push_back(l[t].second);
                }
        }
        degree[p] = (int32_t)ids.size();
        core[p] = (int)ids.size() >= minPts - 1 ? 1 : 0;
        g_graph.nb[p].swap(ids);
        if (with_dist) g_graph.nd[p].swap(ds);
        std::vector<std::pair<int, float>>().swap(l);
    }
}

int64_t orc_neighbors_total(int n) {
    int64_t t = 0;
    for (int p = 0; p < n; ++p) t += (int64_t)g_graph.nb[p].size();
    return t;
}
// CSR export: offsets[n+1], idx[total], dist[total] (dist may be null).
void orc_neighbors_export(int n, int64_t* offsets, int32_t* idx, float* dist) {
    int64_t o = 0;
    for (int p = 0; p < n; ++p) {
        offsets[p] = o;
        for (size_t t = 0; t < g_graph.nb[p].size(); ++t, ++o) {
            idx[o] = g_graph.nb[p][t];
            if (dist) dist[o] = g_graph.nd[p][t];
        }
    }
    offsets[n] = o;
}
void orc_graph_free() {
    std::vector<std::vector<int>>().swap(g_graph.nb);
    std::vector<std::vector<float>>().swap(g_graph.nd);
}

// ---- formCluster (src/sDbscan.cpp:509-637) -----------------------------------
// Over a CSR neighbour graph (lists of core points are what matters; lists
// of non-core points are ignored, as the reference clears them at :379).
// Returns n_clusters_ (number of clusters + 1, or 2 when there are none: :633).
int orc_form_cluster(int n, const uint8_t* core, const int64_t* off, const int32_t* idx, int32_t* labels) {
    std::fill(labels, labels + n, -1);
    int id = -1, ncl = 0;
    std::vector<uint8_t> conn(n, 0);
    std::vector<int> touched;
    for (int p = 0; p < n; ++p) {
        if (!core[p] || labels[p] != -1) continue;
        ++id;
        std::vector<int> seeds(1, p);
        touched.assign(1, p);
        conn[p] = 1;
        while (!seeds.empty()) {
            const int x = seeds.back();
            seeds.pop_back();
            for (int64_t t = off[x]; t < off[x + 1]; ++t) {
                const int y = idx[t];
                if (conn[y]) continue;
                conn[y] = 1;
                touched.push_back(y);
                if (core[y] && labels[y] == -1) seeds.push_back(y);
            }
        }
        for (int y : touched) {
            if (labels[y] == -1) labels[y] = id;
            conn[y] = 0;
        }
        ncl = id;
    }
    return ncl + 2;
}

// ---- core points + clusters for large n (src/sDbscan.cpp:217-408, 509-637) ---
// The neighbourhood sizes, core flags, labels and n_clusters_ of orc_find_core
// followed by orc_form_cluster, computed without the global lock and the
// per-pair pushes of the reference's loop, so a million-point fit checks in a
// minute or two of host time and a few GB of memory:
//  - every candidate distance of point p through list (r, side) -- top-m
//    member q of a random vector in p's top-k (:262-283) -- is evaluated list
//    by list: the list's m rows are held transposed in cache and each of its
//    member points is compared with all of them, leaving one pass bit per
//    (p, slot, candidate) (dist <= eps, :286);
//  - A(p): the distinct candidates of p whose bit is set, self skipped
//    (:272-277), sorted.  A candidate met through two lists has the same
//    distance both times, so evaluating it twice changes nothing;
//  - B(q): every p with q in A(p), i.e. the reverse insertions of :293-294
//    (a counted CSR: only top-m members ever receive one), sorted;
//  - N(p) = A(p) u B(p): |N(p)| is the degree, core iff >= minPts - 1 (:382);
//  - formCluster (:509-637): for p ascending, an unlabelled core point opens
//    the next id and a flood through core points labels every point it
//    reaches that is still -1.
// Distances follow the numerical contract: each one is a sequential chain
// over ascending dimension (fmaf for Cosine / L2, adds for L1 and Chi2); the
// chains of a block of 16 candidates run side by side in SIMD lanes, which
// changes no bits.  JS uses the scalar distance().  Returns n_clusters_.
extern "C++" {
namespace {
constexpr int kLeanBlk = 16;
// Eight lanes of float, GCC's generic vectors (SIMD on x86-64 and aarch64;
// every lane op is the IEEE scalar op).
typedef float f8 __attribute__((vector_size(32)));
typedef int i8 __attribute__((vector_size(32)));
template <int CODE>
void block_dist(const float* x, const float* Ct, int d, float* out) {
    if (CODE == D_COSINE || CODE == D_L2) {
        float s[kLeanBlk];
        for (int j = 0; j < kLeanBlk; ++j) s[j] = 0.0f;
        for (int i = 0; i < d; ++i) {
            const float a = x[i];
            const float* c = Ct + (size_t)i * kLeanBlk;
            for (int j = 0; j < kLeanBlk; ++j) {
                if (CODE == D_COSINE) {
                    s[j] = std::fma(a, c[j], s[j]);
                } else {
                    const float t = a - c[j];
                    s[j] = std::fma(t, t, s[j]);
                }
            }
        }
        for (int j = 0; j < kLeanBlk; ++j) out[j] = CODE == D_COSINE ? 1 - s[j] : std::sqrt(s[j]);
        return;
    }
    static_assert(kLeanBlk == 16, "two f8 lanes per block");
    f8 s0 = {}, s1 = {};
    const f8 zero = {};
    for (int i = 0; i < d; ++i) {
        const f8 a = zero + x[i];
        f8 b0, b1;
        std::memcpy(&b0, Ct + (size_t)i * kLeanBlk, sizeof(f8));
        std::memcpy(&b1, Ct + (size_t)i * kLeanBlk + 8, sizeof(f8));
        if (CODE == D_L1) {
            const f8 t0 = a - b0, t1 = a - b1;
            s0 = s0 + (t0 < zero ? -t0 : t0);  // |a - b|
            s1 = s1 + (t1 < zero ? -t1 : t1);
        } else {  // Chi2: only entries where both are > 0 contribute (Utilities.h:235-241)
            const f8 q0 = (a * b0) / (a + b0), q1 = (a * b1) / (a + b1);
            const i8 ok0 = (a > zero) & (b0 > zero), ok1 = (a > zero) & (b1 > zero);
            s0 = ok0 ? s0 + q0 : s0;
            s1 = ok1 ? s1 + q1 : s1;
        }
    }
    for (int j = 0; j < 8; ++j) {
        out[j] = CODE == D_L1 ? s0[j] : (float)(1.0 - 2.0 * (double)s0[j]);
        out[j + 8] = CODE == D_L1 ? s1[j] : (float)(1.0 - 2.0 * (double)s1[j]);
    }
}
}  // namespace
}  // extern "C++"

namespace {
// A(p) (ids ascending, with distances when asked) and B as a CSR, as stated
// above.
struct LeanGraph {
    std::vector<std::vector<int>> A;
    std::vector<std::vector<float>> Ad;
    std::vector<int64_t> roff;
    std::vector<int32_t> B;
    std::vector<float> Bd;
};

void lean_build(const float* X, int n, int d, int code, const int* topK, int k, const int* topM, int m, float eps,
                bool withDist, LeanGraph& g) {
    const int S = 2 * k, W = (m + 63) / 64;
    int D = 0;  // number of random vectors: one past the largest list id in topK
    for (size_t t = 0; t < (size_t)n * S; ++t) D = std::max(D, topK[t] + 1);
    // members of each list (r, side): (point, slot) pairs, points ascending
    std::vector<int64_t> loff((size_t)2 * D + 1, 0);
    for (int p = 0; p < n; ++p)
        for (int sl = 0; sl < S; ++sl) loff[(size_t)(sl >= k) * D + topK[(size_t)p * S + sl] + 1] += 1;
    for (size_t l = 0; l < (size_t)2 * D; ++l) loff[l + 1] += loff[l];
    std::vector<int64_t> lcur(loff.begin(), loff.end() - 1);
    std::vector<int32_t> lmem((size_t)n * S);
    for (int p = 0; p < n; ++p)
        for (int sl = 0; sl < S; ++sl) lmem[lcur[(size_t)(sl >= k) * D + topK[(size_t)p * S + sl]]++] = p * S + sl;
    std::vector<uint64_t> pass((size_t)n * S * W, 0ull);
    std::vector<float> pdist(withDist ? (size_t)n * S * m : 0);
    const int nb = (m + kLeanBlk - 1) / kLeanBlk;
#pragma omp parallel
    {
        std::vector<float> Ct((size_t)nb * d * kLeanBlk);
        std::vector<float> dd((size_t)nb * kLeanBlk);
#pragma omp for schedule(dynamic, 1)
        for (int l = 0; l < 2 * D; ++l) {
            if (loff[l + 1] == loff[l]) continue;
            const int side = l >= D, r = l - side * D;
            const int* cand = topM + (size_t)r * 2 * m + side * m;
            for (int b = 0; b < nb; ++b)  // candidates transposed, padded with copies of the first
                for (int j = 0; j < kLeanBlk; ++j) {
                    const int c = b * kLeanBlk + j < m ? cand[b * kLeanBlk + j] : cand[0];
                    const float* y = X + (size_t)c * d;
                    for (int i = 0; i < d; ++i) Ct[((size_t)b * d + i) * kLeanBlk + j] = y[i];
                }
            for (int64_t t = loff[l]; t < loff[l + 1]; ++t) {
                const int ps = lmem[t], p = ps / S;
                const float* xp = X + (size_t)p * d;
                for (int b = 0; b < nb; ++b) {
                    const float* cb = Ct.data() + (size_t)b * d * kLeanBlk;
                    float* o = dd.data() + (size_t)b * kLeanBlk;
                    if (code == D_COSINE) block_dist<D_COSINE>(xp, cb, d, o);
                    else if (code == D_L2) block_dist<D_L2>(xp, cb, d, o);
                    else if (code == D_L1) block_dist<D_L1>(xp, cb, d, o);
                    else if (code == D_CHI2) block_dist<D_CHI2>(xp, cb, d, o);
                    else
                        for (int j = 0; j < kLeanBlk && b * kLeanBlk + j < m; ++j)
                            o[j] = distance(xp, X + (size_t)cand[b * kLeanBlk + j] * d, d, code);
                }
                uint64_t* w = pass.data() + (size_t)ps * W;
                for (int i = 0; i < m; ++i)
                    if (dd[i] <= eps) w[i >> 6] |= 1ull << (i & 63);
                if (withDist) std::memcpy(pdist.data() + (size_t)ps * m, dd.data(), sizeof(float) * m);
            }
        }
    }
    std::vector<int32_t>().swap(lmem);
    g.A.assign(n, {});
    g.Ad.assign(withDist ? n : 0, {});
#pragma omp parallel
    {
        std::vector<uint64_t> seen(((size_t)n + 63) / 64, 0ull);
        std::vector<std::pair<int, float>> tmp;
#pragma omp for schedule(dynamic, 256)
        for (int p = 0; p < n; ++p) {
            tmp.clear();
            for (int sl = 0; sl < S; ++sl) {
                const int side = sl >= k, r = topK[(size_t)p * S + sl];
                const int* cand = topM + (size_t)r * 2 * m + side * m;
                const uint64_t* w = pass.data() + ((size_t)p * S + sl) * W;
                for (int i = 0; i < m; ++i) {
                    if (!(w[i >> 6] >> (i & 63) & 1)) continue;
                    const int q = cand[i];
                    if (q == p || (seen[q >> 6] >> (q & 63) & 1)) continue;
                    seen[q >> 6] |= 1ull << (q & 63);
                    tmp.push_back({q, withDist ? pdist[((size_t)p * S + sl) * m + i] : 0.0f});
                }
            }
            for (const auto& e : tmp) seen[e.first >> 6] = 0ull;
            std::sort(tmp.begin(), tmp.end(),
                      [](const std::pair<int, float>& a, const std::pair<int, float>& b) { return a.first < b.first; });
            g.A[p].resize(tmp.size());
            for (size_t t = 0; t < tmp.size(); ++t) g.A[p][t] = tmp[t].first;
            if (withDist) {
                g.Ad[p].resize(tmp.size());
                for (size_t t = 0; t < tmp.size(); ++t) g.Ad[p][t] = tmp[t].second;
            }
        }
    }
    std::vector<uint64_t>().swap(pass);
    std::vector<float>().swap(pdist);
    // B as a CSR, filled without atomics: thread t scatters the A lists of a
    // fixed range of p into slots counted for it, so every B(q) comes out
    // in ascending p
    const int T = omp_get_max_threads();
    std::vector<std::vector<int32_t>> cnt(T);
    g.roff.assign((size_t)n + 1, 0);
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const int p0 = (int)((int64_t)n * t / nt), p1 = (int)((int64_t)n * (t + 1) / nt);
        std::vector<int32_t>& c = cnt[t];
        c.assign(n, 0);
        for (int p = p0; p < p1; ++p)
            for (int q : g.A[p]) c[q] += 1;
#pragma omp barrier
#pragma omp single
        {
            for (int q = 0; q < n; ++q) {
                int64_t o = g.roff[q];
                for (int u = 0; u < nt; ++u) {
                    const int32_t v = cnt[u][q];
                    cnt[u][q] = (int32_t)(o - g.roff[q]);  // start of thread u's run inside B(q)
                    o += v;
                }
                g.roff[q + 1] = o;
            }
            g.B.resize((size_t)g.roff[n]);
            if (withDist) g.Bd.resize((size_t)g.roff[n]);
        }
        for (int p = p0; p < p1; ++p)
            for (size_t t2 = 0; t2 < g.A[p].size(); ++t2) {
                const int q = g.A[p][t2];
                const int64_t slot = g.roff[q] + c[q]++;
                g.B[slot] = p;
                // dist(p, q) == dist(q, p) bit for bit: every formula is symmetric
                if (withDist) g.Bd[slot] = g.Ad[p][t2];
            }
    }
}

// |A(q) u B(q)| for sorted A(q), B(q).
int32_t lean_degree(const LeanGraph& g, int q) {
    const std::vector<int>& a = g.A[q];
    size_t i = 0, both = 0;
    for (int64_t t = g.roff[q]; t < g.roff[q + 1]; ++t) {
        while (i < a.size() && a[i] < g.B[t]) ++i;
        if (i < a.size() && a[i] == g.B[t]) ++both;
    }
    return (int32_t)(a.size() + (size_t)(g.roff[q + 1] - g.roff[q]) - both);
}
}  // namespace

int orc_core_cluster_lean(const float* X, int n, int d, int code, const int* topK, int k, const int* topM, int m,
                          float eps, int minPts, uint8_t* core, int32_t* degree, int32_t* labels) {
    LeanGraph g;
    lean_build(X, n, d, code, topK, k, topM, m, eps, false, g);
#pragma omp parallel for schedule(dynamic, 256)
    for (int q = 0; q < n; ++q) {
        degree[q] = lean_degree(g, q);
        core[q] = degree[q] >= minPts - 1 ? 1 : 0;
    }
    std::fill(labels, labels + n, -1);
    std::vector<uint8_t> conn(n, 0);
    std::vector<int> touched, seeds;
    int id = -1;
    auto visit = [&](int y) {
        if (conn[y]) return;
        conn[y] = 1;
        touched.push_back(y);
        if (core[y] && labels[y] == -1) seeds.push_back(y);
    };
    for (int p = 0; p < n; ++p) {
        if (!core[p] || labels[p] != -1) continue;
        ++id;
        seeds.assign(1, p);
        touched.assign(1, p);
        conn[p] = 1;
        while (!seeds.empty()) {
            const int x = seeds.back();
            seeds.pop_back();
            for (int y : g.A[x]) visit(y);
            for (int64_t t = g.roff[x]; t < g.roff[x + 1]; ++t) visit(g.B[t]);
        }
        for (int y : touched) {
            if (labels[y] == -1) labels[y] = id;
            conn[y] = 0;
        }
    }
    return id >= 0 ? id + 2 : 2;  // n_clusters_ = last id + 2, and 2 with no cluster (:633)
}

// orc_find_core (ref_order = 0) through the large-n construction: the same
// core flags and sizes, and the same neighbour graph (ids ascending, with
// distances when with_dist) for orc_core_dist / orc_neighbors_export.
void orc_find_core_lean(const float* X, int n, int d, int code, const int* topK, int k, const int* topM, int m,
                        float eps, int minPts, int with_dist, uint8_t* core, int32_t* degree) {
    LeanGraph g;
    lean_build(X, n, d, code, topK, k, topM, m, eps, with_dist != 0, g);
    g_graph.nb.assign(n, {});
    g_graph.nd.assign(n, {});
#pragma omp parallel for schedule(dynamic, 256)
    for (int q = 0; q < n; ++q) {
        const std::vector<int>& a = g.A[q];
        std::vector<int>& o = g_graph.nb[q];
        std::vector<float>& od = g_graph.nd[q];
        size_t i = 0;
        int64_t t = g.roff[q];
        const int64_t te = g.roff[q + 1];
        while (i < a.size() || t < te) {  // merge of two ascending lists, equal ids once
            const bool takeA = t == te || (i < a.size() && a[i] <= g.B[t]);
            if (takeA) {
                const bool dup = t < te && a[i] == g.B[t];
                o.push_back(a[i]);
                if (with_dist) od.push_back(g.Ad[q][i]);
                ++i;
                if (dup) ++t;
            } else {
                o.push_back(g.B[t]);
                if (with_dist) od.push_back(g.Bd[t]);
                ++t;
            }
        }
        degree[q] = (int32_t)o.size();
        core[q] = (int)o.size() >= minPts - 1 ? 1 : 0;
    }
}

// ---- core distance (src/sDbscan.cpp:1424-1460) -------------------------------
// coreDist[p] = (minPts-1)-th smallest neighbour distance for core points, 0
// otherwise (FVector(n, 0.0) at :1420).  Uses the graph of orc_find_core.
void orc_core_dist(int n, int minPts, const uint8_t* core, float* coreDist) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int p = 0; p < n; ++p) {
        coreDist[p] = 0.0f;
        if (!core[p]) continue;
        std::vector<float> v = g_graph.nd[p];
        std::nth_element(v.begin(), v.begin() + (minPts - 2), v.end());
        coreDist[p] = v[minPts - 2];
    }
}

// ---- formOptics_scikit (src/sDbscan.cpp:1588-1703) ---------------------------
// CSR graph with distances.  tie_mode 0: the reference's heap, which compares
// reachability values only (Min_PQ_Pair, src/Header.h:100), so equal values
// pop in an order set by the heap and the neighbour-list order.  tie_mode 1:
// the canonical order used by the GPU engine — pops by (reachability, point
// id), which makes the ordering independent of neighbour-list order.
int64_t orc_form_optics(int n, const uint8_t* core, const float* coreDist, const int64_t* off, const int32_t* idx,
                        const float* dist, int tie_mode, int32_t* ordering, float* reach) {
    std::fill(reach, reach + n, kNegInf);
    std::vector<uint8_t> done(n, 0);
    int64_t no = 0;
    struct E {
        float v;
        int i;
    };
    auto cmp0 = [](const E& a, const E& b) { return a.v > b.v; };
    auto cmp1 = [](const E& a, const E& b) { return a.v > b.v || (a.v == b.v && a.i > b.i); };
    std::priority_queue<E, std::vector<E>, decltype(cmp0)> h0(cmp0);
    std::priority_queue<E, std::vector<E>, decltype(cmp1)> h1(cmp1);
    auto push = [&](int y, float v) {
        if (tie_mode) h1.push({v, y});
        else h0.push({v, y});
    };
    auto relax = [&](int x) {
        const float cd = coreDist[x];
        for (int64_t t = off[x]; t < off[x + 1]; ++t) {
            const int y = idx[t];
            if (done[y]) continue;
            const float r = std::max(cd, dist[t]);
            if (reach[y] == kNegInf) {
                reach[y] = r;
                push(y, r);
            } else if (reach[y] > r) {
                reach[y] = r;
                push(y, r);
            }
        }
    };
    for (int p = 0; p < n; ++p) {
        if (done[p]) continue;
        done[p] = 1;
        ordering[no++] = p;
        if (!core[p]) continue;
        relax(p);
        while (tie_mode ? !h1.empty() : !h0.empty()) {
            int y;
            if (tie_mode) {
                y = h1.top().i;
                h1.pop();
            } else {
                y = h0.top().i;
                h0.pop();
            }
            if (done[y]) continue;
            done[y] = 1;
            ordering[no++] = y;
            if (core[y]) relax(y);
        }
    }
    return no;
}

// ---- sDbscan-1NN noise labelling (labelNoise, src/sDbscan.cpp:648-807) ------
// clusterNoise == 1: every point left as noise takes the label of the sampled
// core point whose projections best match its top-k vectors: the estimate
// sum_k P[c][close_k] - P[c][far_k] (accumulated in that order, :786-793), the
// first maximum over the sampled cores in ascending index order (:798-806).
// The cores are sampled with probability fProb = samplingProb n / #cores when
// #cores >= samplingProb n (:683-699).  The reference draws with the unseeded
// rand(); here point p is sampled iff fmix32(seed + 0x9E3779B9 (p + 1)) 2^-32
// <= fProb (MurmurHash3's 32-bit finaliser), the engine's rule.
static inline uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

void orc_label_noise(const float* P, int n, int nproj, const int* topK, int k, const uint8_t* core,
                     float samplingProb, uint32_t seed, int32_t* labels) {
    int numCore = 0;
    for (int p = 0; p < n; ++p) numCore += core[p] ? 1 : 0;
    float fProb = 1.0f;
    if ((float)numCore >= samplingProb * (float)n) fProb = samplingProb * (float)n / (float)numCore;
    std::vector<int> cores;
    for (int p = 0; p < n; ++p) {
        if (!core[p]) continue;
        const double u = (double)fmix32(seed + 0x9E3779B9u * (uint32_t)(p + 1)) * (1.0 / 4294967296.0);
        if (fProb == 1.0f || u <= (double)fProb) cores.push_back(p);
    }
    if (cores.empty()) return;  // no cluster to join (the reference indexes labels_[-1] here)
    std::vector<int32_t> base(labels, labels + n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int x = 0; x < n; ++x) {
        if (base[x] != -1) continue;
        const int* tk = topK + (size_t)x * 2 * k;
        float best = -2147483648.0f;  // NEG_INF (Header.h:20)
        int bestCore = -1;
        for (int c : cores) {
            const float* pc = P + (size_t)c * nproj;
            float v = 0.0f;
            for (int j = 0; j < k; ++j) {
                v += pc[tk[j]];
                v -= pc[tk[j + k]];
            }
            if (v > best) {
                best = v;
                bestCore = c;
            }
        }
        if (bestCore >= 0) labels[x] = base[bestCore];
    }
}

// ---- whole fits, for the CPU baseline (src/sDbscan.cpp:830-890, 1711-1769) ---
// X: d x n column-major, not modified.  bits: 3*fhtDim; R may be null unless
// L1/L2.  times[5]: transform, index, core, cluster/optics, total (seconds).
// Returns n_clusters_ (fit_sdbscan) or 0, or a negative transform error.
int orc_fit_sdbscan(const float* X, int n, int d, int code, int nproj, int k, int m, int ker, float L,
                    const float* R, const uint8_t* bits, int fhtDim, float eps, int minPts, int threads,
                    int clusterNoise, float samplingProb, uint32_t seed, int32_t* labels, uint8_t* core,
                    double* times) {
    if (threads > 0) omp_set_num_threads(threads);
    if (int e = embed_precondition(code, ker, d)) return -e;
    Timer tm, all;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    times[0] = tm.lap();
    std::vector<float> P((size_t)n * nproj);
    std::vector<int> topK((size_t)n * 2 * k), topM((size_t)nproj * 2 * m);
    orc_project(Xc.data(), n, d, code, ker, L, R, bits, fhtDim, nproj, P.data());
    orc_topk(P.data(), n, nproj, k, topK.data());
    orc_topm(P.data(), n, nproj, m, topM.data());
    if (clusterNoise != 1) std::vector<float>().swap(P);
    times[1] = tm.lap();
    std::vector<int32_t> deg(n);
    orc_find_core(Xc.data(), n, d, code, topK.data(), k, topM.data(), m, eps, minPts, 0, 0, core, deg.data());
    times[2] = tm.lap();
    std::vector<int64_t> off(n + 1);
    std::vector<int32_t> idx(orc_neighbors_total(n));
    orc_neighbors_export(n, off.data(), idx.data(), nullptr);
    const int ncl = orc_form_cluster(n, core, off.data(), idx.data(), labels);
    if (clusterNoise == 1) orc_label_noise(P.data(), n, nproj, topK.data(), k, core, samplingProb, seed, labels);
    times[3] = tm.lap();
    times[4] = all.lap();
    orc_graph_free();
    return ncl;
}

// The reference's index-once eps sweep (test_sDbscan, src/sDbscan.cpp:980-1039):
// transform and index once, then for each eps find the core points and form
// the clusters.  labels: nEps x n; ncl: nEps.  times as orc_fit_sdbscan, with
// core and cluster summed over the eps values.
int orc_fit_sdbscan_sweep(const float* X, int n, int d, int code, int nproj, int k, int m, int ker, float L,
                          const float* R, const uint8_t* bits, int fhtDim, const float* eps, int nEps, int minPts,
                          int threads, int32_t* labels, int32_t* ncl, double* times) {
    if (threads > 0) omp_set_num_threads(threads);
    if (int e = embed_precondition(code, ker, d)) return -e;
    Timer tm, all;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    times[0] = tm.lap();
    std::vector<float> P((size_t)n * nproj);
    std::vector<int> topK((size_t)n * 2 * k), topM((size_t)nproj * 2 * m);
    orc_project(Xc.data(), n, d, code, ker, L, R, bits, fhtDim, nproj, P.data());
    orc_topk(P.data(), n, nproj, k, topK.data());
    orc_topm(P.data(), n, nproj, m, topM.data());
    std::vector<float>().swap(P);
    times[1] = tm.lap();
    times[2] = times[3] = 0.0;
    std::vector<int32_t> deg(n);
    std::vector<uint8_t> core(n);
    for (int e = 0; e < nEps; ++e) {
        orc_find_core(Xc.data(), n, d, code, topK.data(), k, topM.data(), m, eps[e], minPts, 0, 0, core.data(),
                      deg.data());
        times[2] += tm.lap();
        std::vector<int64_t> off(n + 1);
        std::vector<int32_t> idx(orc_neighbors_total(n));
        orc_neighbors_export(n, off.data(), idx.data(), nullptr);
        ncl[e] = orc_form_cluster(n, core.data(), off.data(), idx.data(), labels + (size_t)e * n);
        orc_graph_free();
        times[3] += tm.lap();
    }
    times[4] = all.lap();
    return 0;
}

int orc_fit_soptics(const float* X, int n, int d, int code, int nproj, int k, int m, int ker, float L,
                    const float* R, const uint8_t* bits, int fhtDim, float eps, int minPts, int threads,
                    int tie_mode, int32_t* ordering, float* reach, uint8_t* core, float* coreDist, double* times) {
    if (threads > 0) omp_set_num_threads(threads);
    if (int e = embed_precondition(code, ker, d)) return -e;
    Timer tm, all;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    times[0] = tm.lap();
    std::vector<float> P((size_t)n * nproj);
    std::vector<int> topK((size_t)n * 2 * k), topM((size_t)nproj * 2 * m);
    orc_project(Xc.data(), n, d, code, ker, L, R, bits, fhtDim, nproj, P.data());
    orc_topk(P.data(), n, nproj, k, topK.data());
    orc_topm(P.data(), n, nproj, m, topM.data());
    std::vector<float>().swap(P);
    times[1] = tm.lap();
    std::vector<int32_t> deg(n);
    orc_find_core(Xc.data(), n, d, code, topK.data(), k, topM.data(), m, eps, minPts, 1, tie_mode == 0, core, deg.data());
    orc_core_dist(n, minPts, core, coreDist);
    times[2] = tm.lap();
    const int64_t tot = orc_neighbors_total(n);
    std::vector<int64_t> off(n + 1);
    std::vector<int32_t> idx(tot);
    std::vector<float> dist(tot);
    orc_neighbors_export(n, off.data(), idx.data(), dist.data());
    orc_form_optics(n, core, coreDist, off.data(), idx.data(), dist.data(), tie_mode, ordering, reach);
    times[3] = tm.lap();
    times[4] = all.lap();
    orc_graph_free();
    return 0;
}

// ---- sngDbscan (fit_sngDbscan, src/sDbscan.cpp:1131-1179) --------------------
// sng_findCorePoints (:416-504) as the reference states it, point by point:
// point p seeds default_random_engine with `seed` (>= 0 here: a clock seed
// cannot be reproduced) and draws uniform_int_distribution(0, n - 1) until it
// has S = ceil(1.0 n samplingProb) draws that are not p; each draw q within
// eps is pushed into both lists (:459-464).  samplingProb >= 1: every other
// point, forward only (:466-479).  Core points: list size, repeats counted,
// >= minPts - 1; other lists cleared (:488-496); then formCluster.
// labels / core / degree: n.  Returns n_clusters_, a negative transform
// error, or -3 for one point with samplingProb < 1 (it can only draw itself).
// times[5] as orc_fit_sdbscan (index = 0).
int orc_fit_sngdbscan(const float* X, int n, int d, int code, float samplingProb, int seed, float eps, int minPts,
                      int threads, int32_t* labels, uint8_t* core, int32_t* degree, double* times) {
    if (threads > 0) omp_set_num_threads(threads);
    if (n < 2 && samplingProb < 1.0 && std::ceil(1.0 * n * samplingProb) >= 1.0)
        return -3;  // a single point draws only itself: the reference's loop never ends
    Timer tm, all;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    times[0] = tm.lap();
    times[1] = 0.0;
    const float* Y = Xc.data();
    std::vector<std::vector<int>> nb(n);
    if (samplingProb < 1.0) {
        const long long S = (long long)std::ceil(1.0 * n * samplingProb);
        std::vector<std::vector<std::pair<int, int>>> found(n);
#pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < n; ++p) {
            std::default_random_engine gen((unsigned)seed);
            std::uniform_int_distribution<> distrib(0, n - 1);
            for (long long s = 0; s < S;) {
                const int q = distrib(gen);
                if (q == p) continue;
                ++s;
                if (distance(Y + (size_t)p * d, Y + (size_t)q * d, d, code) <= eps) found[p].push_back({p, q});
            }
        }
        for (int p = 0; p < n; ++p)
            for (const auto& e : found[p]) {
                nb[e.first].push_back(e.second);
                nb[e.second].push_back(e.first);
            }
    } else {
#pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < n; ++p)
            for (int q = 0; q < n; ++q)
                if (q != p && distance(Y + (size_t)p * d, Y + (size_t)q * d, d, code) <= eps) nb[p].push_back(q);
    }
    for (int p = 0; p < n; ++p) {
        degree[p] = (int32_t)nb[p].size();
        core[p] = degree[p] >= minPts - 1 ? 1 : 0;
        if (!core[p]) nb[p].clear();
    }
    times[2] = tm.lap();
    std::vector<int64_t> off(n + 1, 0);
    for (int p = 0; p < n; ++p) off[p + 1] = off[p] + (int64_t)nb[p].size();
    std::vector<int32_t> idx(off[n]);
    for (int p = 0; p < n; ++p) std::copy(nb[p].begin(), nb[p].end(), idx.begin() + off[p]);
    const int ncl = orc_form_cluster(n, core, off.data(), idx.data(), labels);
    times[3] = tm.lap();
    times[4] = all.lap();
    return ncl;
}

// ---- sngOptics (fit_sngOptics, src/sDbscan.cpp:1846-1880) --------------------
// sng_findCoreDist (:1484-1583) with the engine's reproducible sample: every
// point draws the same seeded sequence (the reference seeds each point from
// std::random_device, :1500-1501) of S = ceil(samplingProb n) (float product,
// :1490) draws, skipping its own index without replacing it (:1507-1508);
// each draw within eps is pushed into both lists with its distance; lists are
// de-duplicated (:1537-1541); core points have >= minPts - 1 distinct
// neighbours and core distance the (minPts-1)-th smallest (:1543-1555), 0
// otherwise; then formOptics_scikit with (reachability, id) ties (tie_mode 1).
int orc_fit_sngoptics(const float* X, int n, int d, int code, float samplingProb, int seed, float eps, int minPts,
                      int threads, int32_t* ordering, float* reach, uint8_t* core, float* coreDist, int32_t* degree,
                      double* times) {
    if (threads > 0) omp_set_num_threads(threads);
    Timer tm, all;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    times[0] = tm.lap();
    times[1] = 0.0;
    const float* Y = Xc.data();
    const long long S = (long long)std::ceil(samplingProb * (float)n);
    std::vector<int> draws;
    {
        std::default_random_engine gen((unsigned)seed);
        std::uniform_int_distribution<> distrib(0, n - 1);
        for (long long s = 0; s < S; ++s) draws.push_back(distrib(gen));
    }
    std::vector<std::vector<std::pair<int, float>>> found(n);
#pragma omp parallel for schedule(dynamic, 64)
    for (int p = 0; p < n; ++p)
        for (int q : draws) {
            if (q == p) continue;
            const float dd = distance(Y + (size_t)p * d, Y + (size_t)q * d, d, code);
            if (dd <= eps) found[p].push_back({q, dd});
        }
    std::vector<std::map<int, float>> lists(n);
    for (int p = 0; p < n; ++p)
        for (const auto& e : found[p]) {
            lists[p].emplace(e.first, e.second);
            lists[e.first].emplace(p, e.second);
        }
    std::vector<int64_t> off(n + 1, 0);
    for (int p = 0; p < n; ++p) off[p + 1] = off[p] + (int64_t)lists[p].size();
    std::vector<int32_t> idx(off[n]);
    std::vector<float> dist(off[n]);
    for (int p = 0; p < n; ++p) {
        int64_t o = off[p];
        for (const auto& e : lists[p]) {
            idx[o] = e.first;
            dist[o++] = e.second;
        }
        degree[p] = (int32_t)lists[p].size();
        core[p] = degree[p] >= minPts - 1 ? 1 : 0;
        coreDist[p] = 0.0f;
        if (core[p]) {
            std::vector<float> v(dist.begin() + off[p], dist.begin() + off[p + 1]);
            std::nth_element(v.begin(), v.begin() + (minPts - 2), v.end());
            coreDist[p] = v[minPts - 2];
        }
    }
    times[2] = tm.lap();
    orc_form_optics(n, core, coreDist, off.data(), idx.data(), dist.data(), 1, ordering, reach);
    times[3] = tm.lap();
    times[4] = all.lap();
    return 0;
}

// ---- block-sampled sngDbscan / sngOptics --------------------------------------
// The reference's unreproducible samples (sngOptics: std::random_device per
// point, src/sDbscan.cpp:1500-1502; sngDbscan with random_seed < 0: a clock
// seed per point, :437-440) are independent per point.  This rule keeps their
// statistics in a form a GPU can tile: the points are cut into blocks of
// blockRows consecutive indices, and block b draws its own S columns,
// draw j being q = floor(hi32(splitmix64(key + b S + j)) n / 2^32) with
// key = splitmix64(seed) (splitmix64: Steele, Lea and Flood, OOPSLA 2014).
// Every point of block b pairs with each of the block's draws that is not
// itself (no replacement draw), and each pair within eps is pushed into both
// lists, as the reference's loops do.  S = ceil(1.0 n samplingProb) for
// sngDbscan (:449) and ceil(samplingProb n) in float for sngOptics (:1490).
// blockRows = 1 is the reference's independent sampling exactly in law.
static inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline int block_draw(uint64_t key, int64_t S, int64_t b, int64_t j, int n) {
    const uint64_t z = splitmix64(key + (uint64_t)(b * S + j));
    return (int)(((z >> 32) * (uint64_t)n) >> 32);
}

// The pairs within eps of every block: found[p] holds (q, dist) for p's own
// draws.  Returns S.
static int64_t block_pairs(const float* Y, int n, int d, int code, int64_t S, uint32_t seed, int blockRows, float eps,
                           std::vector<std::vector<std::pair<int, float>>>& found) {
    const uint64_t key = splitmix64(seed);
    const int64_t nb = (n + blockRows - 1) / blockRows;
    found.assign(n, {});
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t b = 0; b < nb; ++b) {
        std::vector<int> cols(S);
        for (int64_t j = 0; j < S; ++j) cols[j] = block_draw(key, S, b, j, n);
        const int p1 = (int)std::min<int64_t>(n, (b + 1) * blockRows);
        for (int p = (int)(b * blockRows); p < p1; ++p)
            for (int q : cols) {
                if (q == p) continue;
                const float dd = distance(Y + (size_t)p * d, Y + (size_t)q * d, d, code);
                if (dd <= eps) found[p].push_back({q, dd});
            }
    }
    return S;
}

// sngDbscan under the block rule: neighbourhood sizes with repeats counted,
// core >= minPts - 1, formCluster over the symmetric lists of the cores.
// samplingProb >= 1 is the exact mode (:466-479), identical to
// orc_fit_sngdbscan's.  Returns n_clusters_ or a negative transform error.
int orc_fit_sngdbscan_blocks(const float* X, int n, int d, int code, float samplingProb, uint32_t seed, int blockRows,
                             float eps, int minPts, int threads, int32_t* labels, uint8_t* core, int32_t* degree) {
    if (threads > 0) omp_set_num_threads(threads);
    if (blockRows < 1) return -100;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    const float* Y = Xc.data();
    std::vector<std::vector<int>> nb(n);
    if (samplingProb < 1.0) {
        std::vector<std::vector<std::pair<int, float>>> found;
        block_pairs(Y, n, d, code, (int64_t)std::ceil(1.0 * n * samplingProb), seed, blockRows, eps, found);
        for (int p = 0; p < n; ++p)
            for (const auto& e : found[p]) {
                nb[p].push_back(e.first);
                nb[e.first].push_back(p);
            }
    } else {
#pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < n; ++p)
            for (int q = 0; q < n; ++q)
                if (q != p && distance(Y + (size_t)p * d, Y + (size_t)q * d, d, code) <= eps) nb[p].push_back(q);
    }
    for (int p = 0; p < n; ++p) {
        degree[p] = (int32_t)nb[p].size();
        core[p] = degree[p] >= minPts - 1 ? 1 : 0;
        if (!core[p]) nb[p].clear();
    }
    std::vector<int64_t> off(n + 1, 0);
    for (int p = 0; p < n; ++p) off[p + 1] = off[p] + (int64_t)nb[p].size();
    std::vector<int32_t> idx(off[n]);
    for (int p = 0; p < n; ++p) std::copy(nb[p].begin(), nb[p].end(), idx.begin() + off[p]);
    return orc_form_cluster(n, core, off.data(), idx.data(), labels);
}

// sngOptics under the block rule: de-duplicated lists with distances
// (:1537-1541), core distance the (minPts-1)-th smallest (:1543-1555), then
// formOptics_scikit with (reachability, id) ties.  Returns 0 or a negative
// transform error.
int orc_fit_sngoptics_blocks(const float* X, int n, int d, int code, float samplingProb, uint32_t seed, int blockRows,
                             float eps, int minPts, int threads, int32_t* ordering, float* reach, uint8_t* core,
                             float* coreDist, int32_t* degree) {
    if (threads > 0) omp_set_num_threads(threads);
    if (blockRows < 1 || minPts < 2) return -100;
    std::vector<float> Xc(X, X + (size_t)n * d);
    int err = orc_transform(Xc.data(), n, d, code);
    if (err) return -err;
    std::vector<std::vector<std::pair<int, float>>> found;
    block_pairs(Xc.data(), n, d, code, (int64_t)std::ceil(samplingProb * (float)n), seed, blockRows, eps, found);
    std::vector<std::map<int, float>> lists(n);
    for (int p = 0; p < n; ++p)
        for (const auto& e : found[p]) {
            lists[p].emplace(e.first, e.second);
            lists[e.first].emplace(p, e.second);
        }
    std::vector<int64_t> off(n + 1, 0);
    for (int p = 0; p < n; ++p) off[p + 1] = off[p] + (int64_t)lists[p].size();
    std::vector<int32_t> idx(off[n]);
    std::vector<float> dist(off[n]);
    for (int p = 0; p < n; ++p) {
        int64_t o = off[p];
        for (const auto& e : lists[p]) {
            idx[o] = e.first;
            dist[o++] = e.second;
        }
        degree[p] = (int32_t)lists[p].size();
        core[p] = degree[p] >= minPts - 1 ? 1 : 0;
        coreDist[p] = 0.0f;
        if (core[p]) {
            std::vector<float> v(dist.begin() + off[p], dist.begin() + off[p + 1]);
            std::nth_element(v.begin(), v.begin() + (minPts - 2), v.end());
            coreDist[p] = v[minPts - 2];
        }
    }
    orc_form_optics(n, core, coreDist, off.data(), idx.data(), dist.data(), 1, ordering, reach);
    return 0;
}

// Distance of one pair, exposed for tests of the numerical contract.
float orc_distance(const float* x, const float* y, int d, int code) { return distance(x, y, d, code); }

// 1: the timing mode above (CPU baseline legs only); 0: the numerical contract.
void orc_set_timing_mode(int on) { g_timing_mode = on ? 1 : 0; }

void orc_set_threads(int t) {
    if (t > 0) omp_set_num_threads(t);
}

}  // extern "C"
