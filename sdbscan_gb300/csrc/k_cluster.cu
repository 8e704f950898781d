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
#include "common.cuh"

#include <climits>

namespace sdb {
namespace {

__device__ __forceinline__ int load_parent(const int32_t* parent, int x) { return __ldcg(parent + x); }

__device__ int find_root(int32_t* parent, int x) {
    while (true) {
        const int px = load_parent(parent, x);
        if (px == x) return x;
        const int gx = load_parent(parent, px);
        if (gx != px) parent[x] = gx;  // path halving: gx is an ancestor of x forever
        x = px;
    }
}

__device__ void unite(int32_t* parent, int a, int b) {
    while (true) {
        a = find_root(parent, a);
        b = find_root(parent, b);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(parent + b, b, a);
        if (old == b) return;
        b = old;
    }
}

__global__ void k_init(int32_t* parent, int32_t* border, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    parent[p] = p;
    border[p] = INT_MAX;
}

template <typename F>
__device__ __forceinline__ void for_passing(const ClusterArgs& a, int p, F&& f) {
    for_each_passing(a.topK, a.topM, a.masks, a.k, a.m, a.W, p, f);
}

__global__ void k_union(ClusterArgs a) {
    const int warps = blockDim.x >> 5;
    const int p = blockIdx.x * warps + (threadIdx.x >> 5);
    if (p >= a.n || !a.core[p]) return;
    int rp = find_root(a.parent, p);
    for_passing(a, p, [&](int i) {
        if (!a.core[i]) return;
        const int pi = load_parent(a.parent, i);
        if (pi == rp || load_parent(a.parent, pi) == rp) return;  // already joined (common case)
        unite(a.parent, rp, i);
        rp = find_root(a.parent, rp);
    });
}

__global__ void k_compress(ClusterArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    if (a.core[p]) a.parent[p] = find_root(a.parent, p);
}

__global__ void k_border(ClusterArgs a) {
    const int warps = blockDim.x >> 5;
    const int p = blockIdx.x * warps + (threadIdx.x >> 5);
    if (p >= a.n) return;
    if (a.core[p]) {
        const int rp = a.parent[p];
        for_passing(a, p, [&](int i) {
            if (!a.core[i]) atomicMin(a.border + i, rp);
        });
    } else {
        int best = INT_MAX;
        for_passing(a, p, [&](int i) {
            if (a.core[i]) best = min(best, __ldcg(a.parent + i));
        });
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, m));
        if (lane_id() == 0 && best != INT_MAX) atomicMin(a.border + p, best);
    }
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
    k_init<<<g, 256, 0, st>>>(a.parent, a.border, a.n);
    ++launches;
    const int wg = (a.n + 7) / 8;
    k_union<<<wg, 256, 0, st>>>(a);
    ++launches;
    k_compress<<<g, 256, 0, st>>>(a);
    ++launches;
    k_border<<<wg, 256, 0, st>>>(a);
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

}  // namespace sdb
