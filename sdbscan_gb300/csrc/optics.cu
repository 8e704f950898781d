// sOPTICS stage: neighbour lists with distances and core distances on the
// GPU (rp_findCoreDist, src/sDbscan.cpp:1314-1474), then the ordering and
// reachability (formOptics_scikit, src/sDbscan.cpp:1588-1703).
//
// The ordering is a priority flood: each step pops the unprocessed point of
// least reachability, so it is inherently sequential.  It runs here in host
// C++ over the CSR the GPU produced.  Ties between equal reachability values,
// which the reference's value-only heap resolves by heap order, are resolved
// by the smaller point id, so the ordering does not depend on the order of
// the neighbour lists.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "engine_internal.h"

namespace sdb {
int launch_core_emit(const CoreArgs& a, const void* sig, const int64_t* nbOff, int32_t* nbIdx, float* nbDist,
                     int32_t* nbFill, cudaStream_t st);
int launch_core_dist(const CoreArgs& a, const int64_t* nbOff, const float* nbDist, cudaStream_t st);
int launch_i32_to_i64(const int32_t* in, int64_t* out, int n, cudaStream_t st);
}  // namespace sdb

using namespace sdb;

namespace {

// formOptics_scikit with (reachability, point id) order.  reach[] holds
// NEG_INF (-2^31) for points never reached (src/sDbscan.cpp:1590).  The
// reference keeps a lazy-deletion heap (Min_PQ_Pair seedSet, :1609); here the
// seed queue is an indexed 4-ary min-heap on (reach, id) with decrease-key,
// each unprocessed point in it at most once: the same pop sequence as a lazy
// heap with that order, with fewer heap operations.
void form_optics(int n, const uint8_t* core, const float* coreDist, const int64_t* off, const int32_t* idx,
                 const float* dist, int32_t* ordering, float* reach) {
    std::fill(reach, reach + n, kNegInfReach);
    std::vector<uint8_t> done(n, 0);
    std::vector<int32_t> pos(n, -1), heap;
    heap.reserve(4096);
    auto less = [&](int a, int b) { return reach[a] < reach[b] || (reach[a] == reach[b] && a < b); };
    auto sift_up = [&](int i) {
        const int y = heap[i];
        while (i > 0) {
            const int par = (i - 1) >> 2;
            if (!less(y, heap[par])) break;
            heap[i] = heap[par];
            pos[heap[i]] = i;
            i = par;
        }
        heap[i] = y;
        pos[y] = i;
    };
    auto sift_down = [&](int i) {
        const int y = heap[i], sz = (int)heap.size();
        while (true) {
            const int c0 = 4 * i + 1;
            if (c0 >= sz) break;
            int b = c0;
            for (int c = c0 + 1; c < std::min(c0 + 4, sz); ++c)
                if (less(heap[c], heap[b])) b = c;
            if (!less(heap[b], y)) break;
            heap[i] = heap[b];
            pos[heap[i]] = i;
            i = b;
        }
        heap[i] = y;
        pos[y] = i;
    };
    int64_t no = 0;
    auto relax = [&](int x) {
        const float cd = coreDist[x];
        for (int64_t t = off[x]; t < off[x + 1]; ++t) {
            const int y = idx[t];
            if (done[y]) continue;
            const float r = std::max(cd, dist[t]);
            if (reach[y] == kNegInfReach) {
                reach[y] = r;
                heap.push_back(y);
                sift_up((int)heap.size() - 1);
            } else if (reach[y] > r) {
                reach[y] = r;
                sift_up(pos[y]);
            }
        }
    };
    for (int p = 0; p < n; ++p) {
        if (done[p]) continue;
        done[p] = 1;
        ordering[no++] = p;
        if (!core[p]) continue;
        relax(p);
        while (!heap.empty()) {
            const int y = heap[0];
            const int last = heap.back();
            heap.pop_back();
            if (!heap.empty()) {
                heap[0] = last;
                sift_down(0);
            }
            pos[y] = -1;
            done[y] = 1;
            ordering[no++] = y;
            if (core[y]) relax(y);
        }
    }
}

}  // namespace

sdb_status sdb_engine::optics_stage(const CoreArgs& ca, int& launches) {
    cudaStream_t st = stream;
    if (!ensure(nbOff, sizeof(int64_t) * (n + 1)) || !ensure(nbFill, sizeof(int32_t) * n)) return SDB_ERR_NOMEM;
    cudaError_t e = cudaMemsetAsync(nbOff.ptr, 0, sizeof(int64_t) * (n + 1), st);
    if (e != cudaSuccess) return cuda_fail(e, "memset");
    int r = launch_i32_to_i64(ca.degree, i64(nbOff), n, st);
    if (r < 0) return fail(SDB_ERR_CUDA, "degree conversion launch failed");
    launches += r;
    r = launch_scan_i64(i64(nbOff), i64(nbOff), (size_t)n + 1, i64(scanTmp), st);
    if (r < 0) return fail(SDB_ERR_CUDA, "scan launch failed");
    launches += r;
    int64_t total = 0;
    e = cudaMemcpyAsync(&total, i64(nbOff) + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "neighbour count");
    if (!ensure(nbIdx, sizeof(int32_t) * std::max<int64_t>(total, 1)) ||
        !ensure(nbDist, sizeof(float) * std::max<int64_t>(total, 1)))
        return SDB_ERR_NOMEM;
    e = cudaMemsetAsync(nbFill.ptr, 0, sizeof(int32_t) * n, st);
    if (e != cudaSuccess) return cuda_fail(e, "memset");
    r = launch_core_emit(ca, sig.ptr, i64(nbOff), i32(nbIdx), f32(nbDist), i32(nbFill), st);
    if (r < 0) return fail(SDB_ERR_CUDA, "neighbour list launch failed");
    launches += r;
    r = launch_core_dist(ca, i64(nbOff), f32(nbDist), st);
    if (r < 0) return fail(SDB_ERR_CUDA, "core distance launch failed");
    launches += r;

    return optics_order(total);
}

// Downloads the CSR neighbour lists (nbOff / nbIdx / nbDist), core flags and
// core distances of the last fit and runs the ordering on the host.
// The staging buffers are kept across fits and not zero-filled: a fresh,
// zeroed buffer per fit costs a memset and first-touch page faults over the
// whole list (hundreds of MB at 500K points) before the copy overwrites it.
sdb_status sdb_engine::optics_order(int64_t total) {
    cudaStream_t st = stream;
    cudaError_t e;
    int64_t* hOff = nullptr;
    int32_t* hIdx = nullptr;
    float *hDist = nullptr, *hCd = nullptr;
    uint8_t* hCore = nullptr;
    try {
        hOff = stageOff.get((size_t)n + 1);
        hIdx = stageIdx.get((size_t)std::max<int64_t>(total, 1));
        hDist = stageDist.get((size_t)std::max<int64_t>(total, 1));
        hCd = stageCd.get((size_t)n);
        hCore = stageCore.get((size_t)n);
        hostOrdering.assign(n, 0);
        hostReach.assign(n, 0.0f);
    } catch (const std::bad_alloc&) {
        return fail(SDB_ERR_NOMEM, "host memory for the sOPTICS neighbour lists");
    }
    e = cudaMemcpyAsync(hOff, nbOff.ptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && total)
        e = cudaMemcpyAsync(hIdx, nbIdx.ptr, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && total)
        e = cudaMemcpyAsync(hDist, nbDist.ptr, sizeof(float) * total, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hCd, coreDist.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hCore, core.ptr, n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "neighbour list download");
    form_optics(n, hCore, hCd, hOff, hIdx, hDist, hostOrdering.data(), hostReach.data());
    return SDB_OK;
}
