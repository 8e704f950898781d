// Union-find over point ids shared by the cluster stages (formCluster,
// src/sDbscan.cpp:509-637): a root is its set's smallest point id, so set
// ids follow from a prefix sum over roots.
#pragma once

#include "common.cuh"

namespace sdb {

__device__ __forceinline__ int load_parent(const int32_t* parent, int x) { return __ldcg(parent + x); }

static __device__ int find_root(int32_t* parent, int x) {
    while (true) {
        const int px = load_parent(parent, x);
        if (px == x) return x;
        const int gx = load_parent(parent, px);
        if (gx != px) parent[x] = gx;  // path halving: gx is an ancestor of x forever
        x = px;
    }
}

static __device__ void unite(int32_t* parent, int a, int b) {
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

}  // namespace sdb
