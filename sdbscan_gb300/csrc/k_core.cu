// Stage 5: neighbourhood sizes and core flags (src/sDbscan.cpp:374-400), and
// for sOPTICS the core distance (src/sDbscan.cpp:1424-1460).
//
// The reference de-duplicates each point's neighbour list, which holds both
// its own candidates within eps (A) and every point that found it within eps
// (B).  Here |A u B| = |A| + |B| - |A n B| is assembled without materialising
// the lists:
//  - |A(p)|: distinct passing candidates of p, from p's mask words, through a
//    per-warp hash set in shared memory;
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

constexpr int kEmpty = -1;

__device__ __forceinline__ unsigned hash_pt(int p, unsigned mask) { return ((unsigned)p * 2654435761u) & mask; }

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

// Per-warp working set in shared memory (see core_smem_words):
//   keys[T], cnts[T]          open-addressing set of candidate ids (T = pow2 >= 2 * inserts)
//   dsts[T]                   distance of each id (sOPTICS only)
//   used[T]                   slots taken by the current point, in insertion order
//   listMask[2D/32]           the lists holding the current point (hubs)
struct WarpSet {
    int* keys;
    int* cnts;
    float* dsts;
    uint16_t* used;
    uint32_t* listMask;
    int* nUsed;
};

__host__ __device__ inline int warp_set_words(int T, int maskWords, bool withDist) {
    return 2 * T + T / 2 + maskWords + 1 + (withDist ? T : 0);
}

__device__ __forceinline__ WarpSet warp_set(int* sh, int w, int T, int maskWords, bool withDist) {
    int* b = sh + (size_t)w * warp_set_words(T, maskWords, withDist);
    WarpSet ws;
    ws.keys = b;
    ws.cnts = b + T;
    ws.used = reinterpret_cast<uint16_t*>(b + 2 * T);
    ws.listMask = reinterpret_cast<uint32_t*>(b + 2 * T + T / 2);
    ws.nUsed = b + 2 * T + T / 2 + maskWords;
    ws.dsts = withDist ? reinterpret_cast<float*>(b + 2 * T + T / 2 + maskWords + 1) : nullptr;
    return ws;
}

// Inserts point p's candidates within eps (from its mask words) into the
// warp's set; returns the number of distinct ids.  The 2k top-k ids and mask
// words of p are fetched up front (two slots per lane), so the only
// dependent loads left are the candidate ids themselves.
__device__ int build_set(const CoreArgs& a, const WarpSet& ws, int p, unsigned tmask, uint64_t* firstOut) {
    const unsigned l = lane_id();
    const int slots = 2 * a.k;
    int rA = 0, rB = 0;
    uint64_t mA0 = 0, mA1 = 0, mB0 = 0, mB1 = 0;
    const unsigned long long* mk64 = reinterpret_cast<const unsigned long long*>(a.masks);
    if ((int)l < slots) {
        rA = __ldg(a.topK + (size_t)p * slots + l);
        mA0 = __ldg(mk64 + ((size_t)p * slots + l) * a.W);
        if (a.W > 1) mA1 = __ldg(mk64 + ((size_t)p * slots + l) * a.W + 1);
    }
    if ((int)l + 32 < slots) {
        rB = __ldg(a.topK + (size_t)p * slots + l + 32);
        mB0 = __ldg(mk64 + ((size_t)p * slots + l + 32) * a.W);
        if (a.W > 1) mB1 = __ldg(mk64 + ((size_t)p * slots + l + 32) * a.W + 1);
    }
    if (l == 0) *ws.nUsed = 0;
    __syncwarp();
    for (int jj = 0; jj < slots; ++jj) {
        const int src = jj & 31;
        const int r = __shfl_sync(0xffffffffu, jj < 32 ? rA : rB, src);
        const int side = jj >= a.k;
        const int32_t* lst = a.topM + (size_t)r * 2 * a.m + side * a.m;
        for (int wd = 0; wd < a.W; ++wd) {
            uint64_t mk;
            if (wd < 2) {
                const uint64_t mine = jj < 32 ? (wd == 0 ? mA0 : mA1) : (wd == 0 ? mB0 : mB1);
                const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)mine, src);
                const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(mine >> 32), src);
                mk = ((uint64_t)hi << 32) | lo;
            } else {
                mk = __ldg(mk64 + ((size_t)p * slots + jj) * a.W + wd);
            }
            uint32_t fresh[2] = {0u, 0u};
            if (mk) {
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const int bit = half * 32 + (int)l;
                    bool isNew = false;
                    if ((mk >> bit) & 1ull) {
                        const int s = wd * 64 + bit;
                        const int i = __ldg(lst + s);
                        unsigned h = hash_pt(i, tmask);
                        while (true) {
                            const int old = atomicCAS(&ws.keys[h], kEmpty, i);
                            if (old == kEmpty) {
                                ws.used[atomicAdd(ws.nUsed, 1)] = (uint16_t)h;
                                atomicAdd(&ws.cnts[h], 1);
                                if (ws.dsts) ws.dsts[h] = a.dists[((size_t)p * slots + jj) * a.m + s];
                                isNew = true;
                                break;
                            }
                            if (old == i) {
                                atomicAdd(&ws.cnts[h], 1);
                                break;
                            }
                            h = (h + 1) & tmask;
                        }
                    }
                    fresh[half] = __ballot_sync(0xffffffffu, isNew);
                }
            }
            if (firstOut && l == 0)
                firstOut[((size_t)p * slots + jj) * a.W + wd] = ((uint64_t)fresh[1] << 32) | fresh[0];
        }
    }
    __syncwarp();
    return *ws.nUsed;
}

// Marks, in the warp's list mask, the top-m lists holding hub point p.
__device__ __forceinline__ void mark_lists(const CoreArgs& a, const WarpSet& ws, int64_t h0, int64_t h1,
                                           int maskWords) {
    const unsigned l = lane_id();
    for (int t = (int)l; t < maskWords; t += 32) ws.listMask[t] = 0u;
    __syncwarp();
    for (int64_t h = h0 + l; h < h1; h += 32) {
        const int lst = a.hubLists[h];
        atomicOr(&ws.listMask[lst >> 5], 1u << (lst & 31));
    }
    __syncwarp();
}

__device__ __forceinline__ void clear_set(const WarpSet& ws, int nd) {
    for (int u = (int)lane_id(); u < nd; u += 32) {
        const int h = ws.used[u];
        ws.keys[h] = kEmpty;
        ws.cnts[h] = 0;
    }
    __syncwarp();
}

// Persistent warps, each over points p = warp, warp + total, ...
__global__ void k_core_dedupe(CoreArgs a, int T) {
    extern __shared__ int sh[];
    const int w = threadIdx.x >> 5;
    const unsigned l = lane_id();
    const int maskWords = (2 * a.nproj + 31) / 32;
    const WarpSet ws = warp_set(sh, w, T, maskWords, a.dists != nullptr);
    const unsigned tmask = (unsigned)T - 1u;
    for (int s = (int)l; s < T; s += 32) {
        ws.keys[s] = kEmpty;
        ws.cnts[s] = 0;
    }
    __syncwarp();
    const int gw = blockIdx.x * (blockDim.x >> 5) + w;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int p = gw; p < a.n; p += nw) {
        const int nd = build_set(a, ws, p, tmask, a.firstMasks);
        const int64_t h0 = a.hubOff[p], h1 = a.hubOff[p + 1];
        const bool hub = h1 > h0;
        if (hub) mark_lists(a, ws, h0, h1, maskWords);
        for (int u = (int)l; u < nd; u += 32) {
            const int h = ws.used[u];
            const int i = ws.keys[h];
            int corr = ws.cnts[h] - 1;
            if (hub && in_candidates_of(a, ws.listMask, a.hubLists + h0, (int)(h1 - h0), i)) corr += 1;
            if (corr) atomicSub(a.inRaw + i, corr);
        }
        if (l == 0) a.aCount[p] = nd;
        __syncwarp();
        clear_set(ws, nd);
    }
}

__global__ void k_core_finish(CoreArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int deg = a.aCount[p] + a.inRaw[p];
    a.degree[p] = deg;
    a.core[p] = deg >= a.minPts - 1 ? 1 : 0;
}

// sOPTICS neighbour lists (src/sDbscan.cpp:1371-1372, :1404-1405, de-duplicated
// at :1428-1431): for every point p, its distinct candidates within eps (own
// entries, first |A(p)| slots of its row) and every point that found p within
// eps without p finding it back (in entries, after them).  Row p starts at
// nbOff[p] and holds degree[p] = |A(p)| + |B(p) \ A(p)| entries.
__global__ void k_core_emit(CoreArgs a, int T, const int64_t* __restrict__ nbOff, int32_t* __restrict__ nbIdx,
                            float* __restrict__ nbDist, int32_t* __restrict__ nbFill) {
    extern __shared__ int sh[];
    const int w = threadIdx.x >> 5;
    const unsigned l = lane_id();
    const int maskWords = (2 * a.nproj + 31) / 32;
    const WarpSet ws = warp_set(sh, w, T, maskWords, true);
    const unsigned tmask = (unsigned)T - 1u;
    for (int s = (int)l; s < T; s += 32) {
        ws.keys[s] = kEmpty;
        ws.cnts[s] = 0;
    }
    __syncwarp();
    const int gw = blockIdx.x * (blockDim.x >> 5) + w;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int p = gw; p < a.n; p += nw) {
        const int nd = build_set(a, ws, p, tmask, nullptr);
        const int64_t h0 = a.hubOff[p], h1 = a.hubOff[p + 1];
        const bool hub = h1 > h0;
        if (hub) mark_lists(a, ws, h0, h1, maskWords);
        const int64_t row = nbOff[p];
        for (int u = (int)l; u < nd; u += 32) {
            const int h = ws.used[u];
            const int i = ws.keys[h];
            const float dd = ws.dsts[h];
            nbIdx[row + u] = i;
            nbDist[row + u] = dd;
            if (!(hub && in_candidates_of(a, ws.listMask, a.hubLists + h0, (int)(h1 - h0), i))) {
                const int q = atomicAdd(nbFill + i, 1);
                const int64_t at = nbOff[i] + a.aCount[i] + q;
                nbIdx[at] = p;
                nbDist[at] = dd;
            }
        }
        __syncwarp();
        clear_set(ws, nd);
    }
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

// Table slots: a power of two above the most candidates a point can insert
// (2km), so probing always ends; typical fill is well under half.
int core_table_size(int k, int m) {
    int t = 64;
    while (t < 2 * k * m + 1) t <<= 1;
    return t;
}

static size_t core_warp_bytes(const CoreArgs& a, int T, bool withDist) {
    return sizeof(int) * (size_t)warp_set_words(T, (2 * a.nproj + 31) / 32, withDist);
}

static int core_grid(int n, int warps) {
    const int blocks = (n + warps - 1) / warps;
    return std::min(blocks, 152 * 16);
}

int launch_core_dedupe(const CoreArgs& a, cudaStream_t st) {
    const int T = core_table_size(a.k, a.m);
    const size_t perWarp = core_warp_bytes(a, T, a.dists != nullptr);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / perWarp));
    const size_t sm = perWarp * warps;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_core_dedupe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_core_dedupe<<<core_grid(a.n, warps), warps * 32, sm, st>>>(a, T);
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

int launch_core_emit(const CoreArgs& a, const int64_t* nbOff, int32_t* nbIdx, float* nbDist, int32_t* nbFill,
                     cudaStream_t st) {
    const int T = core_table_size(a.k, a.m);
    const size_t perWarp = core_warp_bytes(a, T, true);
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / perWarp));
    const size_t sm = perWarp * warps;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_core_emit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_core_emit<<<core_grid(a.n, warps), warps * 32, sm, st>>>(a, T, nbOff, nbIdx, nbDist, nbFill);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_core_dist(const CoreArgs& a, const int64_t* nbOff, const float* nbDist, cudaStream_t st) {
    k_core_dist<<<(a.n + 7) / 8, 256, 0, st>>>(a, nbOff, nbDist);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
