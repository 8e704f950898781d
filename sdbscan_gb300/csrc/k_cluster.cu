// Stage 6: cluster labels — formCluster (src/sDbscan.cpp:509-637) as a
// parallel union-find over the core graph.
//
// What the reference's BFS computes, stated without an order:
//  - cores connected through core-core edges share a cluster;
//  - clusters are numbered 0, 1, ... in increasing order of their smallest
//    core index (the outer loop visits points in ascending order, :518);
//  - a non-core point within eps of a core takes the smallest cluster id
//    among its adjacent cores (first cluster whose BFS reaches it, :603);
//  - every other point is noise (-1); n_clusters_ = clusters + 1, or 2 when
//    there is no cluster (:619, :633).
// Union-find hooks the larger root under the smaller one, so each root is
// its component's minimum index and ids follow from a prefix sum over roots.
#include "uf.cuh"

#include <climits>

namespace sdb {
namespace {

__global__ void k_init(int32_t* parent, int32_t* border, int n, int keepParent) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (!keepParent) parent[p] = p;
    border[p] = INT_MAX;
}

// A tile of the distance stage: list l's member rows [mbeg, mend) against its
// candidate columns [64 ct, 64 ct + 64) (mask word ct).
struct Tile {
    int64_t mbeg, mend;
    int ct;
    const int32_t* cand;
};

__device__ __forceinline__ bool tile_of(const ClusterArgs& a, int64_t b, Tile& tl) {
    if (b >= *a.tileTotal) return false;
    const int64_t t = tile_at(a.tilePerm, b);
    const int l = a.tileList[t];
    const int64_t ti = t - a.tileOff[l];
    const int mt = (int)(ti / a.nct);
    tl.ct = (int)(ti % a.nct);
    tl.mbeg = a.listOff[l] + (int64_t)mt * a.TM;
    tl.mend = min(tl.mbeg + a.TM, a.listOff[l + 1]);
    const int r = l % a.nproj, side = l / a.nproj;
    tl.cand = a.topM + (size_t)r * 2 * a.m + side * a.m;
    return true;
}

// Union over the core-core edges of one tile.  The roots of the tile's core
// candidates are found once and cached in shared memory; a member row then
// compares its own root with the cached roots of its passing candidates and
// unites only where they differ.  A cached value is always an ancestor of its
// candidate (parents only move up), so equality proves the same set; a stale
// value only costs a redundant unite.
__global__ void __launch_bounds__(128) k_union_tiles(ClusterArgs a) {
    __shared__ int croot[64];
    __shared__ unsigned long long newCoreCand;  // carry: candidates that became core this round
    Tile tl;
    if (!tile_of(a, blockIdx.x, tl)) return;
    volatile int* vroot = croot;
    if (threadIdx.x == 0) newCoreCand = 0ull;
    __syncthreads();
    int q = -1;  // this thread's candidate (threads < 64)
    if (threadIdx.x < 64) {
        const int c = tl.ct * 64 + threadIdx.x;
        if (c < a.m) {
            q = __ldg(tl.cand + c);
            if (a.carry && a.core[q] && a.coreEps[q] == a.round) atomicOr(&newCoreCand, 1ull << threadIdx.x);
        }
    }
    __syncthreads();
    const int64_t row = tl.mbeg + threadIdx.x;
    int p = -1;
    uint64_t bits = 0;
    if (row < tl.mend) {
        const int2 mb = __ldg(a.members + row);
        if (a.core[mb.x]) {
            p = mb.x;
            const size_t at = ((size_t)p * 2 * a.k + mb.y) * a.W + tl.ct;
            bits = __ldg(reinterpret_cast<const unsigned long long*>(a.masks) + at);
            // carrying over a smaller eps's union-find, only edges that are new (a
            // new pair, or an endpoint that just became core) can join components
            if (a.carry && a.coreEps[p] != a.round)
                bits &= __ldg(reinterpret_cast<const unsigned long long*>(a.newMasks) + at) | newCoreCand;
        }
    }
    if (!__syncthreads_or(bits != 0)) return;  // nothing to unite in this tile
    if (threadIdx.x < 64) croot[threadIdx.x] = (q >= 0 && a.core[q]) ? find_root(a.parent, q) : -1;
    __syncthreads();
    if (!bits) return;
    int rp = find_root(a.parent, p);
    while (bits) {
        const int j = __ffsll((long long)bits) - 1;
        bits &= bits - 1;
        const int cr = vroot[j];
        if (cr < 0 || cr == rp) continue;
        unite(a.parent, rp, cr);
        rp = find_root(a.parent, rp);
        vroot[j] = rp;
    }
}

__global__ void k_compress(ClusterArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    if (a.core[p]) a.parent[p] = find_root(a.parent, p);
}

// Border labels of one tile (parents are roots after k_compress).  A non-core
// member takes the smallest root among its passing core candidates; a non-core
// candidate takes the smallest root among the core members passing with it,
// reduced in shared memory first so each candidate sees one global atomic.
__global__ void __launch_bounds__(128) k_border_tiles(ClusterArgs a) {
    __shared__ int croot[64], cbest[64], cpt[64];
    Tile tl;
    if (!tile_of(a, blockIdx.x, tl)) return;
    if (threadIdx.x < 64) {
        const int c = tl.ct * 64 + threadIdx.x;
        const int q = c < a.m ? __ldg(tl.cand + c) : -1;
        cpt[threadIdx.x] = q;
        croot[threadIdx.x] = (q >= 0 && a.core[q]) ? __ldcg(a.parent + q) : INT_MAX;
        cbest[threadIdx.x] = INT_MAX;
    }
    __syncthreads();
    const int64_t row = tl.mbeg + threadIdx.x;
    if (row < tl.mend) {
        const int2 mb = __ldg(a.members + row);
        const int p = mb.x;
        uint64_t bits = __ldg(reinterpret_cast<const unsigned long long*>(a.masks) +
                              ((size_t)p * 2 * a.k + mb.y) * a.W + tl.ct);
        if (bits) {
            if (a.core[p]) {
                const int rp = __ldcg(a.parent + p);
                while (bits) {
                    const int j = __ffsll((long long)bits) - 1;
                    bits &= bits - 1;
                    if (croot[j] == INT_MAX) atomicMin(&cbest[j], rp);
                }
            } else {
                int best = INT_MAX;
                while (bits) {
                    const int j = __ffsll((long long)bits) - 1;
                    bits &= bits - 1;
                    best = min(best, croot[j]);
                }
                if (best != INT_MAX) atomicMin(a.border + p, best);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < 64 && cbest[threadIdx.x] != INT_MAX) atomicMin(a.border + cpt[threadIdx.x], cbest[threadIdx.x]);
}

__global__ void k_root_flags(ClusterArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > a.n) return;
    a.rootFlag[p] = (p < a.n && a.core[p] && a.parent[p] == p) ? 1 : 0;
}

__global__ void k_labels(ClusterArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        const int c = (int)a.rootFlag[a.n];
        *a.nClusters = c >= 1 ? c + 1 : 2;
    }
    if (p >= a.n) return;
    int lab = -1;
    if (a.core[p]) lab = (int)a.rootFlag[a.parent[p]];
    else if (a.border[p] != INT_MAX) lab = (int)a.rootFlag[a.border[p]];
    a.labels[p] = lab;
}

}  // namespace

int launch_cluster(const ClusterArgs& a, cudaStream_t st) {
    int launches = 0;
    const int g = (a.n + 255) / 256;
    k_init<<<g, 256, 0, st>>>(a.parent, a.border, a.n, a.carry && a.round > 0);
    ++launches;
    k_union_tiles<<<(unsigned)a.nTiles, 128, 0, st>>>(a);
    ++launches;
    k_compress<<<g, 256, 0, st>>>(a);
    ++launches;
    k_border_tiles<<<(unsigned)a.nTiles, 128, 0, st>>>(a);
    ++launches;
    k_root_flags<<<(a.n + 1 + 255) / 256, 256, 0, st>>>(a);
    ++launches;
    int r = launch_scan_i64(a.rootFlag, a.rootFlag, (size_t)a.n + 1, a.scanTmp, st);
    if (r < 0) return -1;
    launches += r;
    k_labels<<<g, 256, 0, st>>>(a);
    ++launches;
    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

// The union-find steps for callers with their own edge kernels (sngDbscan).
int launch_uf_init(int32_t* parent, int32_t* border, int n, cudaStream_t st) {
    k_init<<<(n + 255) / 256, 256, 0, st>>>(parent, border, n, 0);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_uf_compress(const ClusterArgs& a, cudaStream_t st) {
    k_compress<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_cluster_labels(const ClusterArgs& a, cudaStream_t st) {
    k_root_flags<<<(a.n + 1 + 255) / 256, 256, 0, st>>>(a);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    const int r = launch_scan_i64(a.rootFlag, a.rootFlag, (size_t)a.n + 1, a.scanTmp, st);
    if (r < 0) return -1;
    k_labels<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? r + 2 : -1;
}

}  // namespace sdb
