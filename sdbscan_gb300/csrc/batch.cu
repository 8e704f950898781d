// Many datasets, each with an eps sweep, as one CUDA graph.
//
// sdb_batch_create plans every dataset once (a normal sweep fit that sizes
// the buffers and uploads the random signs), then records the whole batch —
// every dataset's index, distances and per-eps core/cluster stages — into one
// CUDA graph.  Datasets run on their engines' own streams; at most `lanes` of
// them run at a time (set i waits for set i - lanes).  The batch's autotuner
// picks, per set, the distance stage's form (the plain kernel's tile shapes
// and, in BF16 mode, the tensor-core screening, timing the set's sweep with
// each) and then the lane count (timing each candidate graph).
// sdb_batch_run replays the graph: one launch for all the clusterings.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/sdbscan_gb300.h"
#include "engine_internal.h"

struct sdb_batch {
    int device = 0;
    std::vector<sdb_engine*> eng;
    std::vector<const float*> X;
    std::vector<float> eps;
    int minPts = 0;
    cudaStream_t origin = nullptr;
    cudaGraphExec_t exec = nullptr;
    int lanes = 0;
    std::vector<float> tuneMs;  // per candidate lane count
    std::vector<int> tuneLanes;
    std::string err;
    std::vector<cudaEvent_t> done;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<DevBuf> labels, ncl;
};

namespace {

sdb_status batch_fail(sdb_batch* b, sdb_status s, const std::string& m) {
    b->err = m;
    return s;
}

// Records the whole batch with the given concurrency into a graph.
sdb_status record(sdb_batch* b, int lanes, cudaGraphExec_t* exec) {
    const int ns = (int)b->eng.size();
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return batch_fail(b, SDB_ERR_CUDA, "begin capture failed");
    cudaEventRecord(b->fork, b->origin);
    sdb_status s = SDB_OK;
    for (int i = 0; i < ns && s == SDB_OK; ++i) {
        sdb_engine* e = b->eng[i];
        cudaStreamWaitEvent(e->stream, b->fork, 0);
        if (i >= lanes) cudaStreamWaitEvent(e->stream, b->done[i - lanes], 0);
        SweepSpec sw;
        sw.eps = b->eps.data();
        sw.nEps = (int)b->eps.size();
        sw.labelsDev = static_cast<int32_t*>(b->labels[i].ptr);
        sw.nclDev = static_cast<int32_t*>(b->ncl[i].ptr);
        sw.capture = true;
        s = e->fit(b->X[i], true, b->eps[0], b->minPts, false, &sw);
        if (s != SDB_OK) b->err = "set " + std::to_string(i) + ": " + e->err;
        cudaEventRecord(b->done[i], e->stream);
    }
    for (int i = 0; i < ns; ++i) cudaStreamWaitEvent(b->origin, b->done[i], 0);
    cudaError_t c = cudaStreamEndCapture(b->origin, &g);
    if (s != SDB_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (c != cudaSuccess) return batch_fail(b, SDB_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(c));
    c = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (c != cudaSuccess) return batch_fail(b, SDB_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(c));
    return SDB_OK;
}

sdb_status launch_timed(sdb_batch* b, cudaGraphExec_t exec, float* ms) {
    cudaEventRecord(b->t0, b->origin);
    cudaError_t c = cudaGraphLaunch(exec, b->origin);
    cudaEventRecord(b->t1, b->origin);
    if (c == cudaSuccess) c = cudaStreamSynchronize(b->origin);
    if (c != cudaSuccess) return batch_fail(b, SDB_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(c));
    if (ms) cudaEventElapsedTime(ms, b->t0, b->t1);
    for (size_t i = 0; i < b->eng.size(); ++i) {
        sdb_status s = b->eng[i]->check_flags();
        if (s != SDB_OK) return batch_fail(b, s, "set " + std::to_string(i) + ": " + b->eng[i]->err);
    }
    return SDB_OK;
}

}  // namespace

extern "C" {

sdb_status sdb_batch_create(int32_t n_sets, const int32_t* n_points, const int32_t* n_features,
                            const float* const* X_device, const sdb_params* p, const float* eps, int32_t n_eps,
                            int32_t minPts, int32_t device, sdb_batch** out) {
    if (!out || n_sets < 1 || !n_points || !n_features || !X_device || !p || !eps || n_eps < 1) return SDB_ERR_ARG;
    *out = nullptr;
    sdb_batch* b = new sdb_batch();
    b->device = device;
    b->eps.assign(eps, eps + n_eps);
    b->minPts = minPts;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
        delete b;
        return SDB_ERR_CUDA;
    }
    sdb_params q = *p;  // BF16 precision screens each set's distances (exact re-decision near every eps)
    if (q.random_seed < 0) q.random_seed = 42;
    b->labels.resize(n_sets);
    b->ncl.resize(n_sets);
    b->done.resize(n_sets);
    for (int i = 0; i < n_sets; ++i) {
        sdb_engine* e = nullptr;
        sdb_status s = sdb_engine_create(n_points[i], n_features[i], device, &e);
        if (s != SDB_OK) {
            *out = b;
            return batch_fail(b, s, "engine " + std::to_string(i));
        }
        b->eng.push_back(e);
        b->X.push_back(X_device[i]);
        cudaEventCreateWithFlags(&b->done[i], cudaEventDisableTiming);
        s = sdb_set_params(e, &q);
        if (s != SDB_OK) {
            *out = b;
            return batch_fail(b, s, "set " + std::to_string(i) + ": " + e->err);
        }
        if (!e->ensure(b->labels[i], sizeof(int32_t) * (size_t)n_eps * n_points[i]) ||
            !e->ensure(b->ncl[i], sizeof(int32_t) * n_eps)) {
            *out = b;
            return batch_fail(b, SDB_ERR_NOMEM, "outputs of set " + std::to_string(i));
        }
        // sizing run: allocates every buffer and uploads the signs
        SweepSpec sw;
        sw.eps = b->eps.data();
        sw.nEps = n_eps;
        sw.labelsDev = static_cast<int32_t*>(b->labels[i].ptr);
        sw.nclDev = static_cast<int32_t*>(b->ncl[i].ptr);
        s = e->fit(X_device[i], true, eps[0], minPts, false, &sw);
        if (s != SDB_OK) {
            *out = b;
            return batch_fail(b, s, "set " + std::to_string(i) + ": " + e->err);
        }
        // tile autotuner: when the tile shapes all apply (m <= 50), time the
        // set's distance stage with each plain shape and, in BF16 mode, with
        // the tensor-core screening too; the set keeps the fastest (a sweep's
        // screening re-decides the pairs near every eps, which on small sets
        // of low dimension can cost more than it saves)
        if (q.topM <= 50) {
            float best = 1e30f;
            int bestV = 0;
            if (q.precision == SDB_PREC_BF16) {
                s = e->fit(X_device[i], true, eps[0], minPts, false, &sw);
                if (s != SDB_OK) {
                    *out = b;
                    return batch_fail(b, s, "set " + std::to_string(i) + ": " + e->err);
                }
                best = e->stageMs[4];
                e->prm.precision = SDB_PREC_FP32;
            }
            for (int v : {1, 2, 3}) {
                e->distVariant = v;
                s = e->fit(X_device[i], true, eps[0], minPts, false, &sw);
                if (s != SDB_OK) {
                    *out = b;
                    return batch_fail(b, s, "set " + std::to_string(i) + ": " + e->err);
                }
                if (e->stageMs[4] < best) {
                    best = e->stageMs[4];
                    bestV = v;
                }
            }
            e->distVariant = bestV;
            if (bestV == 0) e->prm.precision = SDB_PREC_BF16;  // the screening won
        }
    }
    // autotune the number of datasets in flight
    float best = 1e30f;
    for (int lanes : {4, 8, 16, 32, 64}) {
        if (lanes > 2 * n_sets && !b->tuneLanes.empty()) break;
        cudaGraphExec_t ex = nullptr;
        sdb_status s = record(b, std::min(lanes, n_sets), &ex);
        if (s != SDB_OK) {
            *out = b;
            return s;
        }
        float ms = 0.0f;
        s = launch_timed(b, ex, nullptr);  // warm
        if (s == SDB_OK) s = launch_timed(b, ex, &ms);
        if (s != SDB_OK) {
            cudaGraphExecDestroy(ex);
            *out = b;
            return s;
        }
        b->tuneLanes.push_back(std::min(lanes, n_sets));
        b->tuneMs.push_back(ms);
        if (ms < best) {
            best = ms;
            if (b->exec) cudaGraphExecDestroy(b->exec);
            b->exec = ex;
            b->lanes = std::min(lanes, n_sets);
        } else {
            cudaGraphExecDestroy(ex);
        }
    }
    *out = b;
    return SDB_OK;
}

sdb_status sdb_batch_run(sdb_batch* b, float* elapsed_ms) {
    if (!b || !b->exec) return SDB_ERR_STATE;
    cudaSetDevice(b->device);
    return launch_timed(b, b->exec, elapsed_ms);
}

sdb_status sdb_batch_labels(sdb_batch* b, int32_t set, int32_t eps_index, int32_t* labels, int32_t* n_clusters) {
    if (!b || set < 0 || set >= (int)b->eng.size() || eps_index < 0 || eps_index >= (int)b->eps.size())
        return SDB_ERR_ARG;
    sdb_engine* e = b->eng[set];
    cudaSetDevice(b->device);
    cudaError_t c = cudaSuccess;
    if (labels)
        c = cudaMemcpy(labels, static_cast<int32_t*>(b->labels[set].ptr) + (size_t)eps_index * e->n,
                       sizeof(int32_t) * e->n, cudaMemcpyDeviceToHost);
    if (c == cudaSuccess && n_clusters)
        c = cudaMemcpy(n_clusters, static_cast<int32_t*>(b->ncl[set].ptr) + eps_index, sizeof(int32_t),
                       cudaMemcpyDeviceToHost);
    return c == cudaSuccess ? SDB_OK : batch_fail(b, SDB_ERR_CUDA, cudaGetErrorString(c));
}

int32_t sdb_batch_lanes(sdb_batch* b) { return b ? b->lanes : 0; }

int32_t sdb_batch_tile_variant(sdb_batch* b, int32_t set) {
    if (!b || set < 0 || set >= (int)b->eng.size()) return -1;
    return b->eng[set]->distVariant;
}

void sdb_batch_destroy(sdb_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->origin) cudaStreamSynchronize(b->origin);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (size_t i = 0; i < b->eng.size(); ++i) {
        for (DevBuf* d : {&b->labels[i], &b->ncl[i]})
            if (d->ptr) cudaFree(d->ptr);
        sdb_engine_destroy(b->eng[i]);
    }
    for (cudaEvent_t ev : b->done)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : {b->fork, b->t0, b->t1})
        if (ev) cudaEventDestroy(ev);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

const char* sdb_batch_last_error(sdb_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
