// Stage 5: neighbourhood sizes and core flags (src/sDbscan.cpp:374-400), and
// for sOPTICS the core distance (src/sDbscan.cpp:1424-1460).
//
// The reference de-duplicates each point's neighbour list, which holds both
// its own candidates within eps (A) and every point that found it within eps
// (B).  Here |A u B| = |A| + |B| - |A n B| is assembled without materialising
// the lists:
//  - |A(p)|: distinct passing candidates of p, from p's mask words; a
//    candidate met through several of p's lists is counted at its first list;
//  - |B(i)|: the distance kernel added, per tile, how many members pass
//    against candidate i (with multiplicity when a member meets i through
//    several of its lists); here each point p removes its surplus (mult - 1)
//    for every distinct candidate i;
//  - |A n B|: i in A(p) and p in A(i).  Only possible when p is itself a
//    candidate of someone ("hub"); then p in A(i) iff one of the top-m lists
//    holding p is among i's 2k lists (equal distance both ways).  Such pairs
//    are removed from B(i)'s count as well.
#include "common.cuh"

#include <algorithm>

namespace sdb {
namespace {

// true iff hub point p is in one of point i's 2k candidate lists, i.e. one
// of the top-m lists holding p is among the lists i meets through its top-k.
// Two equivalent tests; the cheaper one for p is used:
//  - p's lists (|L(p)| of them, passed in pl/np) against i's list mask
//    (kMask, one bit per list, L2-resident: only hubs have one);
//  - i's 2k top-k entries against p's list mask in shared memory.
__device__ __forceinline__ bool in_candidates_of(const CoreArgs& a, const uint32_t* listMask, const int32_t* pl,
                                                 int np, int i) {
    const int words = (2 * a.nproj + 31) / 32;
    if (np <= 2 * a.k) {
        const uint32_t* km = a.kMask + (size_t)__ldg(a.hubIdx + i) * words;
        for (int t = 0; t < np; ++t) {
            const int lst = __ldg(pl + t);
            if ((__ldg(km + (lst >> 5)) >> (lst & 31)) & 1u) return true;
        }
        return false;
    }
    const int32_t* ki = a.topK + (size_t)i * 2 * a.k;
    for (int j = 0; j < 2 * a.k; ++j) {
        const int lst = __ldg(ki + j) + (j >= a.k ? a.nproj : 0);
        if ((listMask[lst >> 5] >> (lst & 31)) & 1u) return true;
    }
    return false;
}

__global__ void k_hub_flags(const int64_t* __restrict__ hubOff, int n, int64_t* __restrict__ flag) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p <= n) flag[p] = (p < n && hubOff[p + 1] > hubOff[p]) ? 1 : 0;
}

__global__ void k_hub_index(CoreArgs a, const int64_t* __restrict__ scanned, int32_t* __restrict__ hubIdx,
                            uint32_t* __restrict__ kMask, int64_t* __restrict__ nHubs) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *nHubs = scanned[a.n];
    if (p >= a.n) return;
    const bool hub = a.hubOff[p + 1] > a.hubOff[p];
    const int h = hub ? (int)scanned[p] : -1;
    hubIdx[p] = h;
    if (!hub) return;
    const int words = (2 * a.nproj + 31) / 32;
    uint32_t* km = kMask + (size_t)h * words;
    for (int j = 0; j < 2 * a.k; ++j) {
        const int lst = a.topK[(size_t)p * 2 * a.k + j] + (j >= a.k ? a.nproj : 0);
        atomicOr(km + (lst >> 5), 1u << (lst & 31));
    }
}

// Duplicates without hashing.  Point p meets candidate i once per list of p
// that holds i, so with K(p) = p's 2k lists and L(i) = the top-m lists
// holding i, i's multiplicity among p's candidates is |K(p) n L(i)|, and the
// occurrence through list l is the first one iff no smaller list of
// K(p) n L(i) exists.  sig[l][s] lists, for the point in slot s of list l, the
// other lists holding it (up to three; cnt > 3 sends the test to the hub-list
// CSR), and K(p) sits as a bit mask in shared memory while p is processed.

__global__ void k_slot_sigs(const int32_t* __restrict__ topM, int D, int m, const int64_t* __restrict__ hubOff,
                            const int32_t* __restrict__ hubLists, int4* __restrict__ sig) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * D * m) return;
    const int l = q / m, s = q % m, r = l % D, side = l / D;
    const int i = topM[(size_t)r * 2 * m + side * m + s];
    int o[3] = {-1, -1, -1}, c = 0;
    for (int64_t h = hubOff[i]; h < hubOff[i + 1]; ++h) {
        const int lst = hubLists[h];
        if (lst == l) continue;
        if (c < 3) o[c] = lst;
        ++c;
    }
    sig[q] = make_int4(o[0], o[1], o[2], c);
}

// multi[l][w] bit j: the point in slot 64 w + j of list l is held by another
// list too.  Most slots hold a point of one list only (about 84 % of the
// passing pairs at 1M x 784); such an occurrence is the first and only one.
__global__ void k_multi_bits(const int4* __restrict__ sig, int D, int m, int W, uint64_t* __restrict__ multi) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * D * W) return;
    const int l = q / W, wd = q % W;
    uint64_t bits = 0;
    for (int j = 0; j < 64 && wd * 64 + j < m; ++j)
        bits |= (uint64_t)(sig[(size_t)l * m + wd * 64 + j].w > 0) << j;
    multi[q] = bits;
}

__device__ __forceinline__ bool has_list(const uint32_t* km, int lst) { return (km[lst >> 5] >> (lst & 31)) & 1u; }

// Multiplicity and first-occurrence test of candidate i, met through list l.
__device__ __forceinline__ void occurrence(const CoreArgs& a, const uint32_t* km, const int4* sig, int l, int s, int i,
                                          int& mult, bool& first) {
    const int4 g = __ldg(sig + (size_t)l * a.m + s);
    mult = 1;
    first = true;
    if (g.w <= 3) {
        if (g.w > 0 && has_list(km, g.x)) { ++mult; first &= g.x > l; }
        if (g.w > 1 && has_list(km, g.y)) { ++mult; first &= g.y > l; }
        if (g.w > 2 && has_list(km, g.z)) { ++mult; first &= g.z > l; }
    } else {
        for (int64_t h = a.hubOff[i]; h < a.hubOff[i + 1]; ++h) {
            const int o = a.hubLists[h];
            if (o != l && has_list(km, o)) {
                ++mult;
                first &= o > l;
            }
        }
    }
}

// Per-warp shared memory: K(p) mask and p's hub-list mask (2D bits each).
__device__ __forceinline__ void set_k_mask(uint32_t* km, int l, bool on) {
    if (on) atomicOr(km + (l >> 5), 1u << (l & 31));
}

// Visits the passing slots of point p, slot by slot; f(jj, l, s, i, first,
// mult) on lanes (the sOPTICS list emission).
template <typename F>
__device__ __forceinline__ void visit_point(const CoreArgs& a, uint32_t* km, const int4* sig, int p, F&& f) {
    const unsigned lane = lane_id();
    const int slots = 2 * a.k;
    const unsigned long long* mk64 = reinterpret_cast<const unsigned long long*>(a.masks);
    int rA = 0, rB = 0;
    uint64_t mA0 = 0, mB0 = 0;
    if ((int)lane < slots) {
        rA = __ldg(a.topK + (size_t)p * slots + lane);
        mA0 = __ldg(mk64 + ((size_t)p * slots + lane) * a.W);
    }
    if ((int)lane + 32 < slots) {
        rB = __ldg(a.topK + (size_t)p * slots + lane + 32);
        mB0 = __ldg(mk64 + ((size_t)p * slots + lane + 32) * a.W);
    }
    const int lA = rA + ((int)lane >= a.k ? a.nproj : 0), lB = rB + ((int)lane + 32 >= a.k ? a.nproj : 0);
    set_k_mask(km, lA, (int)lane < slots);
    set_k_mask(km, lB, (int)lane + 32 < slots);
    __syncwarp();
    for (int jj = 0; jj < slots; ++jj) {
        const int src = jj & 31;
        const int l = __shfl_sync(0xffffffffu, jj < 32 ? lA : lB, src);
        const int r = l % a.nproj, side = l / a.nproj;
        const int32_t* lst = a.topM + (size_t)r * 2 * a.m + side * a.m;
        for (int wd = 0; wd < a.W; ++wd) {
            uint64_t mk;
            if (wd == 0) {
                const uint64_t mine = jj < 32 ? mA0 : mB0;
                const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)mine, src);
                const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(mine >> 32), src);
                mk = ((uint64_t)hi << 32) | lo;
            } else {
                mk = __ldg(mk64 + ((size_t)p * slots + jj) * a.W + wd);
            }
            if (mk) {
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const int bit = half * 32 + (int)lane;
                    if ((mk >> bit) & 1ull) {
                        const int s = wd * 64 + bit;
                        const int i = __ldg(lst + s);
                        int mult;
                        bool isFirst;
                        occurrence(a, km, sig, l, s, i, mult, isFirst);
                        f(jj, l, s, i, isFirst, mult);
                    }
                }
            }
        }
    }
    __syncwarp();
    if ((int)lane < slots) km[lA >> 5] = 0u;
    if ((int)lane + 32 < slots) km[lB >> 5] = 0u;
    __syncwarp();
}

__device__ __forceinline__ void mark_lists(const CoreArgs& a, uint32_t* listMask, int64_t h0, int64_t h1,
                                           int maskWords) {
    const unsigned l = lane_id();
    for (int t = (int)l; t < maskWords; t += 32) listMask[t] = 0u;
    __syncwarp();
    for (int64_t h = h0 + l; h < h1; h += 32) {
        const int lst = a.hubLists[h];
        atomicOr(&listMask[lst >> 5], 1u << (lst & 31));
    }
    __syncwarp();
}

// Per-warp shared memory of k_core_dedupe (after the two list masks).
constexpr int kDdWords = 32;   // mask words per round, one per lane
constexpr int kDdSlots = 62;   // 2k for k <= 31
struct DedupeWarp {
    uint32_t fresh[2 * kDdWords];       // first-occurrence bits found by the per-pair test (32-bit halves)
    int32_t list[kDdSlots];             // per slot: its list
    int32_t rowOff[kDdSlots];           // per slot: its list's row in topM
    uint16_t item[kDdWords * 64];       // the round's pairs that need the per-pair test: (word, bit)
};
__host__ __device__ constexpr size_t dedupe_warp_bytes(int maskWords) {
    return sizeof(uint32_t) * 2 * (size_t)maskWords + sizeof(DedupeWarp);
}

// Persistent warps, each over points p = warp, warp + total, ...
// A point that is no hub (no top-m list holds it) takes the pairs whose
// candidate no other list holds straight from the mask words (first
// occurrence, multiplicity 1, nothing to correct) and runs the per-pair test
// only on the others; a hub runs it on all its pairs, since each of its first
// occurrences needs the in-candidates test too.  The pairs to test are first
// gathered into a dense per-warp list, so the warp's instructions follow those
// pairs rather than every slot and lane.
__global__ void __launch_bounds__(256, 4) k_core_dedupe(CoreArgs a, const int4* __restrict__ sig) {
    extern __shared__ __align__(16) uint32_t shm[];
    const int w = threadIdx.x >> 5;
    const unsigned lane = lane_id();
    const int maskWords = (2 * a.nproj + 31) / 32;
    uint32_t* km = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(shm) + (size_t)w * dedupe_warp_bytes(maskWords));
    uint32_t* listMask = km + maskWords;
    DedupeWarp& sw = *reinterpret_cast<DedupeWarp*>(listMask + maskWords);
    for (int t = (int)lane; t < maskWords; t += 32) km[t] = 0u;
    __syncwarp();
    const int gw = blockIdx.x * (blockDim.x >> 5) + w;
    const int nw = gridDim.x * (blockDim.x >> 5);
    const int slots = 2 * a.k;
    const int nWords = slots * a.W;
    const unsigned long long* mk64 = reinterpret_cast<const unsigned long long*>(a.masks);
    for (int p = gw; p < a.n; p += nw) {
        const unsigned long long* pm = mk64 + (size_t)p * nWords;
        // a point without a passing pair (common in a sweep round) only clears
        // its first-occurrence words (this round's words when accumulating)
        bool any = false;
        for (int t = (int)lane; t < nWords; t += 32) any |= __ldg(pm + t) != 0ull;
        if (!__any_sync(0xffffffffu, any)) {
            uint64_t* out = a.accumulate ? a.newMasks : a.firstMasks;
            for (int t = (int)lane; t < nWords; t += 32) out[(size_t)p * nWords + t] = 0ull;
            if (lane == 0) a.aCount[p] = 0;
            continue;
        }
        const int64_t h0 = a.hubOff[p], h1 = a.hubOff[p + 1];
        const bool hub = h1 > h0;
        if (hub) mark_lists(a, listMask, h0, h1, maskWords);
        for (int j = (int)lane; j < slots; j += 32) {
            const int l = __ldg(a.topK + (size_t)p * slots + j) + (j >= a.k ? a.nproj : 0);
            sw.list[j] = l;
            sw.rowOff[j] = (l % a.nproj) * 2 * a.m + (l / a.nproj) * a.m;
            atomicOr(km + (l >> 5), 1u << (l & 31));
        }
        __syncwarp();
        int distinct = 0;
        for (int wb = 0; wb < nWords; wb += kDdWords) {
            const int g = wb + (int)lane;  // this lane's mask word: slot g / W, word g % W
            uint64_t mk = 0, mu = 0;
            if (g < nWords) {
                mk = __ldg(pm + g);
                // a hub's every first occurrence needs the in-candidates test
                mu = hub ? ~0ull : __ldg(a.multi + (size_t)sw.list[g / a.W] * a.W + g % a.W);
            }
            const uint64_t sole = mk & ~mu, todo = mk & mu;
            distinct += __popcll(sole);
            sw.fresh[2 * lane] = 0u;
            sw.fresh[2 * lane + 1] = 0u;
            // gather the pairs that need the test: lane-serial over its word's bits
            const int cnt = __popcll(todo);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            int at = incl - cnt;
            for (uint64_t t = todo; t; t &= t - 1) sw.item[at++] = (uint16_t)((lane << 6) | (__ffsll((long long)t) - 1));
            __syncwarp();
            for (int t = (int)lane; t < total; t += 32) {
                const int it = sw.item[t];
                const int wl = it >> 6, bit = it & 63;
                const int gg = wb + wl;
                const int jj = gg / a.W, s = (gg % a.W) * 64 + bit;
                const int l = sw.list[jj];
                const int i = __ldg(a.topM + sw.rowOff[jj] + s);
                int mult;
                bool first;
                occurrence(a, km, sig, l, s, i, mult, first);
                if (!first) continue;
                ++distinct;
                atomicOr(&sw.fresh[2 * wl + (bit >> 5)], 1u << (bit & 31));
                int corr = mult - 1;
                if (hub && in_candidates_of(a, listMask, a.hubLists + h0, (int)(h1 - h0), i)) corr += 1;
                if (corr) atomicSub(a.inRaw + i, corr);
            }
            __syncwarp();
            if (g < nWords) {
                const size_t o = (size_t)p * nWords + g;
                const uint64_t f64 = sole | ((uint64_t)sw.fresh[2 * lane + 1] << 32) | sw.fresh[2 * lane];
                if (a.accumulate) {
                    a.firstMasks[o] |= f64;
                    a.newMasks[o] = f64;
                } else {
                    a.firstMasks[o] = f64;
                }
            }
            __syncwarp();
        }
        for (int j = (int)lane; j < slots; j += 32) km[sw.list[j] >> 5] = 0u;
        __syncwarp();
        distinct = warp_sum(distinct);
        if (lane == 0) a.aCount[p] = distinct;
    }
}

// sOPTICS neighbour lists (src/sDbscan.cpp:1371-1372, :1404-1405, de-duplicated
// at :1428-1431): for every point p, its distinct candidates within eps (own
// entries, first |A(p)| slots of its row) and every point that found p within
// eps without p finding it back (in entries, after them).  Row p starts at
// nbOff[p] and holds degree[p] = |A(p)| + |B(p) \ A(p)| entries.
__global__ void k_core_emit(CoreArgs a, const int4* __restrict__ sig, const int64_t* __restrict__ nbOff,
                            int32_t* __restrict__ nbIdx, float* __restrict__ nbDist, int32_t* __restrict__ nbFill) {
    extern __shared__ uint32_t shm[];
    const int w = threadIdx.x >> 5;
    const unsigned lane = lane_id();
    const int maskWords = (2 * a.nproj + 31) / 32;
    uint32_t* km = shm + (size_t)w * (2 * maskWords + 1);
    uint32_t* listMask = km + maskWords;
    int* cursor = reinterpret_cast<int*>(listMask + maskWords);  // next own-entry slot of the row
    for (int t = (int)lane; t < maskWords; t += 32) km[t] = 0u;
    __syncwarp();
    const int gw = blockIdx.x * (blockDim.x >> 5) + w;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int p = gw; p < a.n; p += nw) {
        const int64_t h0 = a.hubOff[p], h1 = a.hubOff[p + 1];
        const bool hub = h1 > h0;
        if (hub) mark_lists(a, listMask, h0, h1, maskWords);
        if (lane == 0) *cursor = 0;
        __syncwarp();
        const int64_t row = nbOff[p];
        visit_point(a, km, sig, p, [&](int jj, int, int s, int i, bool first, int) {
            if (!first) return;
            const float dd = a.dists[((size_t)p * 2 * a.k + jj) * a.m + s];
            const int pos = atomicAdd(cursor, 1);
            nbIdx[row + pos] = i;
            nbDist[row + pos] = dd;
            if (!(hub && in_candidates_of(a, listMask, a.hubLists + h0, (int)(h1 - h0), i))) {
                const int q = atomicAdd(nbFill + i, 1);
                const int64_t at = nbOff[i] + a.aCount[i] + q;
                nbIdx[at] = p;
                nbDist[at] = dd;
            }
        });
    }
}

__global__ void k_core_finish(CoreArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    if (a.accumulate) {  // this round's pairs are new neighbours: the degree grows
        const int deg = a.degree[p] + a.aCount[p] + a.inRaw[p];
        a.degree[p] = deg;
        if (!a.core[p] && deg >= a.minPts - 1) {
            a.core[p] = 1;
            a.coreEps[p] = a.round;
        }
        return;
    }
    const int deg = a.aCount[p] + a.inRaw[p];
    a.degree[p] = deg;
    a.core[p] = deg >= a.minPts - 1 ? 1 : 0;
}

// Core distance: the (minPts-1)-th smallest distance of a core point's row
// (nth_element at minPts-2, src/sDbscan.cpp:1443-1446); 0 for other points
// (src/sDbscan.cpp:1420).  One warp per point, 4-pass radix select over the
// order-preserving keys of the distances.
__global__ void k_core_dist(CoreArgs a, const int64_t* __restrict__ nbOff, const float* __restrict__ nbDist) {
    __shared__ unsigned hist[8][256];
    const int w = threadIdx.x >> 5;
    const unsigned l = lane_id();
    const int p = blockIdx.x * (blockDim.x >> 5) + w;
    if (p >= a.n) return;
    if (!a.core[p]) {
        if (l == 0) a.coreDist[p] = 0.0f;
        return;
    }
    const int64_t r0 = nbOff[p], r1 = nbOff[p + 1];
    int need = a.minPts - 1;  // 1-based rank of the wanted value
    uint32_t prefix = 0, pmask = 0;
    unsigned* hs = hist[w];
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = (int)l; b < 256; b += 32) hs[b] = 0;
        __syncwarp();
        for (int64_t t = r0 + l; t < r1; t += 32) {
            const uint32_t k = key_of(nbDist[t]);
            if ((k & pmask) == prefix) atomicAdd(&hs[(k >> shift) & 255u], 1u);
        }
        __syncwarp();
        // find the bucket holding the need-th smallest
        int acc = 0, pick = 255;
        for (int b = 0; b < 256; ++b) {
            const int c = (int)hs[b];
            if (acc + c >= need) {
                pick = b;
                break;
            }
            acc += c;
        }
        need -= acc;
        prefix |= (uint32_t)pick << shift;
        pmask |= 255u << shift;
        __syncwarp();
    }
    if (l == 0) a.coreDist[p] = float_of_key(prefix);
}

}  // namespace

static int core_grid(int n, int warps) {
    const int blocks = (n + warps - 1) / warps;
    return std::min(blocks, sm_count() * 8);
}

int launch_slot_sigs(const int32_t* topM, int D, int m, const int64_t* hubOff, const int32_t* hubLists, void* sig,
                     uint64_t* multi, int W, cudaStream_t st) {
    const int total = 2 * D * m;
    k_slot_sigs<<<(total + 255) / 256, 256, 0, st>>>(topM, D, m, hubOff, hubLists, static_cast<int4*>(sig));
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    k_multi_bits<<<(2 * D * W + 255) / 256, 256, 0, st>>>(static_cast<const int4*>(sig), D, m, W, multi);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

int launch_core_dedupe(const CoreArgs& a, const void* sig, cudaStream_t st) {
    const int warps = 8;
    if (2 * a.k > kDdSlots || a.multi == nullptr) return -1;
    const size_t sm = dedupe_warp_bytes((2 * a.nproj + 31) / 32) * warps;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_core_dedupe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_core_dedupe<<<core_grid(a.n, warps), warps * 32, sm, st>>>(a, static_cast<const int4*>(sig));
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_hub_masks(const CoreArgs& a, int32_t* hubIdx, int64_t* idxTmp, uint32_t* kMask, int64_t* scanTmp,
                     int64_t* nHubsDev, cudaStream_t st) {
    k_hub_flags<<<(a.n + 1 + 255) / 256, 256, 0, st>>>(a.hubOff, a.n, idxTmp);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    int r = launch_scan_i64(idxTmp, idxTmp, (size_t)a.n + 1, scanTmp, st);
    if (r < 0) return -1;
    k_hub_index<<<(a.n + 255) / 256, 256, 0, st>>>(a, idxTmp, hubIdx, kMask, nHubsDev);
    return cudaPeekAtLastError() == cudaSuccess ? r + 2 : -1;
}

int launch_core_finish(const CoreArgs& a, cudaStream_t st) {
    k_core_finish<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_core_emit(const CoreArgs& a, const void* sig, const int64_t* nbOff, int32_t* nbIdx, float* nbDist,
                     int32_t* nbFill, cudaStream_t st) {
    const int warps = 8;
    const size_t sm = sizeof(uint32_t) * (2 * ((2 * a.nproj + 31) / 32) + 1) * warps;
    k_core_emit<<<core_grid(a.n, warps), warps * 32, sm, st>>>(a, static_cast<const int4*>(sig), nbOff, nbIdx,
                                                               nbDist, nbFill);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_core_dist(const CoreArgs& a, const int64_t* nbOff, const float* nbDist, cudaStream_t st) {
    k_core_dist<<<(a.n + 7) / 8, 256, 0, st>>>(a, nbOff, nbDist);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
