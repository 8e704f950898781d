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

// true iff point p (a hub) is in one of point i's 2k candidate lists.
__device__ bool in_candidates_of(const CoreArgs& a, int p, int i) {
    const int64_t h0 = a.hubOff[p], h1 = a.hubOff[p + 1];
    const int32_t* ki = a.topK + (size_t)i * 2 * a.k;
    for (int64_t h = h0; h < h1; ++h) {
        const int lst = a.hubLists[h];
        const int r = lst % a.nproj, side = lst / a.nproj;
        for (int j = 0; j < a.k; ++j)
            if (__ldg(ki + side * a.k + j) == r) return true;
    }
    return false;
}

// One warp per point.
__global__ void k_core_dedupe(CoreArgs a, int tableSize) {
    extern __shared__ int sh[];
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const unsigned l = lane_id();
    int* keys = sh + (size_t)w * tableSize * 2;
    int* cnts = keys + tableSize;
    float* dsts = nullptr;
    if (a.dists) dsts = reinterpret_cast<float*>(sh + (size_t)warps * tableSize * 2) + (size_t)w * tableSize;
    const unsigned tmask = (unsigned)tableSize - 1u;
    const int p = blockIdx.x * warps + w;
    if (p >= a.n) return;

    for (int s = (int)l; s < tableSize; s += 32) {
        keys[s] = kEmpty;
        cnts[s] = 0;
    }
    __syncwarp();
    const int slots = 2 * a.k;
    for (int jj = 0; jj < slots; ++jj) {
        const int r = __ldg(a.topK + (size_t)p * slots + jj);
        const int side = jj >= a.k;
        const int32_t* lst = a.topM + (size_t)r * 2 * a.m + side * a.m;
        for (int wd = 0; wd < a.W; ++wd) {
            const uint64_t mk = __ldg(reinterpret_cast<const unsigned long long*>(a.masks) +
                                      ((size_t)p * slots + jj) * a.W + wd);
            if (!mk) continue;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int bit = half * 32 + (int)l;
                if ((mk >> bit) & 1ull) {
                    const int s = wd * 64 + bit;
                    const int i = __ldg(lst + s);
                    unsigned h = hash_pt(i, tmask);
                    while (true) {
                        const int old = atomicCAS(&keys[h], kEmpty, i);
                        if (old == kEmpty || old == i) {
                            atomicAdd(&cnts[h], 1);
                            if (dsts && old == kEmpty)
                                dsts[h] = a.dists[((size_t)p * slots + jj) * a.m + s];
                            break;
                        }
                        h = (h + 1) & tmask;
                    }
                }
            }
        }
    }
    __syncwarp();
    const bool hub = a.hubOff[p + 1] > a.hubOff[p];
    int distinct = 0;
    for (int s = (int)l; s < tableSize; s += 32) {
        const int i = keys[s];
        if (i == kEmpty) continue;
        ++distinct;
        int corr = cnts[s] - 1;
        if (hub && in_candidates_of(a, p, i)) corr += 1;
        if (corr) atomicSub(a.inRaw + i, corr);
    }
    distinct = warp_sum(distinct);
    if (l == 0) a.aCount[p] = distinct;
}

__global__ void k_core_finish(CoreArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int deg = a.aCount[p] + a.inRaw[p];
    a.degree[p] = deg;
    a.core[p] = deg >= a.minPts - 1 ? 1 : 0;
}

}  // namespace

int core_table_size(int k, int m) {
    int t = 64;
    while (t < 2 * 2 * k * m) t <<= 1;
    return t;
}

int launch_core_dedupe(const CoreArgs& a, cudaStream_t st) {
    const int T = core_table_size(a.k, a.m);
    const size_t perWarp = sizeof(int) * 2 * T + (a.dists ? sizeof(float) * T : 0);
    int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024) / perWarp));
    const size_t sm = perWarp * warps;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_core_dedupe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_core_dedupe<<<(a.n + warps - 1) / warps, warps * 32, sm, st>>>(a, T);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_core_finish(const CoreArgs& a, cudaStream_t st) {
    k_core_finish<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
