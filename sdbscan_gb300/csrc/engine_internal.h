// The engine object behind the opaque sdb_engine handle of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/sdbscan_gb300.h"
#include "common.cuh"

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Host staging kept across fits: grow-only, and its contents are not
// initialised (each use overwrites what it reads).  get() may throw
// std::bad_alloc.
template <typename T>
struct HostBuf {
    std::unique_ptr<T[]> p;
    size_t cap = 0;
    T* get(size_t count) {
        if (count > cap) {
            p.reset(new T[count]);
            cap = count;
        }
        return p.get();
    }
};

// Eps sweep of one fit (the reference's test_sDbscan pattern): the index and
// the candidate distances are computed once, then core points and clusters
// per eps value.  capture = enqueue only (no events, host syncs or pageable
// uploads), for recording into a CUDA graph after a normal run has sized the
// buffers and uploaded the random signs.
struct SweepSpec {
    const float* eps = nullptr;  // host, nEps values
    int nEps = 0;
    int32_t* labelsDev = nullptr;  // nEps x n device output
    int32_t* nclDev = nullptr;     // nEps device output
    bool capture = false;
};

// Device error / status flags of a fit (int32 each):
//   [0] negative Chi2/JS input   [1] zero point   [2] non-finite value
//   [3] top-m internal error     [4] BF16 distance screening failed (plain path redoes it)
//   [5] tensor-core embedding failed (FP32 redoes it)   [6] sngOptics list overflow
//   [7] sng BF16 block failed (FP32 redoes it)   [8] a bounded wait of the plain distance kernel ran out
constexpr int kErrSlots = 16;

struct sdb_engine {
    int n = 0, d = 0, device = 0;
    sdb_params prm{};
    bool paramsSet = false;
    bool sngParamsSet = false;  // set_sngParams (enough for the sng fits)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[9] = {};
    // host input is uploaded in segments, spread round-robin over the copy
    // streams, each segment's projection starting as soon as its rows have
    // landed.  One stream: a single copy already runs at the host link's rate,
    // and concurrent copies only delay each segment's arrival (1M x 784 from
    // pinned memory: projection stage 15.7 ms with one stream, 21.0 with two,
    // 23.9 with four, against 14.8 ms for the bare copy)
    static constexpr int kUploadSegs = 16, kCopyStreams = 1;
    cudaStream_t copyStream[kCopyStreams] = {};
    cudaEvent_t segEv[kUploadSegs + 1] = {};
    std::string err;

    // derived from the parameters
    int ker = 0, fhtDim = 0, ld = 0, seedUsed = 0;
    double ln4 = 0.0;
    std::vector<uint32_t> hostSigns;
    std::vector<float> hostRt;
    std::vector<double> hostCosh;

    // device buffers (grow-only; kept across fits)
    DevBuf Xin, Xt, scale, P, topK, chunkMax, chunkMin, thr, cand, candCount, topM, listCount, listOff,
        members, tileOff, tileList, hubCount, hubOff, hubLists, masks, inRaw, aCount, degree, core, parent, border,
        rootFlag, labels, nClusters, scanTmp, errFlags, counters, E, Rt, signs, compCosh, dists, coreDist, nbOff,
        nbIdx, nbDist, nbFill, hubIdx, kMask, firstMasks, Xb, queue, sweepLabels, sweepNcl, sig, Rb, newMasks,
        coreEps, sampleFlag, noiseFlag, noiseCores, noisePts, PcT, numCore, pairRound, sngCols, sngMult, sngColOf,
        sngExtras, sngExtraPass, sngMask, rowDeg, colCnt, sngUb, sngHeavy, chunkOff, tileKey, keyOff, tilePerm, Cb,
        tileKeyTc, keyOffTc, tilePermTc, sngWords, hashOffB, hashIdB, hashDistB, sqNorm, multiMask;

    // results
    bool haveLabels = false, haveOptics = false, haveFit = false, lastOptics = false;
    bool lastSng = false;  // the last fit was sngDbscan / sngOptics (no index state)
    std::vector<int32_t> hostOrdering;
    std::vector<float> hostReach;
    // the sOPTICS neighbour lists, core distances and core flags downloaded
    // for the host ordering
    HostBuf<int64_t> stageOff;
    HostBuf<int32_t> stageIdx;
    HostBuf<float> stageDist, stageCd;
    HostBuf<uint8_t> stageCore;
    int32_t* hostErr = nullptr;
    unsigned long long* hostCounters = nullptr;
    int launchCount = 0;
    int64_t fallbacks = 0;  // BF16 screening fits redone on the plain path
    int sngColsLast = 0, sngExtraLast = 0;  // sampled columns and extra draws of the last sng fit
    int distVariant = 0;    // plain distance tile shape (DistArgs::variant), set by the batch's autotuner
    int sngSampling = 0;    // sngDbscan sample: 0 = by seed (shared when >= 0, blocks when < 0), 1 = shared, 2 = blocks
    // test and diagnostic limits (sdb_set_debug_limits), 0 = off
    long long dbgStallSpins = 0;  // each tensor-core / persistent distance kernel takes its failure path once
    int64_t dbgQueueCap = 0;      // cap of the BF16 re-decision queues
    size_t dbgDeviceCap = 0;      // cap of the engine's device memory
    size_t devBytes = 0;          // device memory the engine holds now
    float stageMs[9] = {};

    bool ensure(DevBuf& b, size_t bytes);
    sdb_status fail(sdb_status s, const std::string& msg);
    sdb_status cuda_fail(cudaError_t e, const char* where);
    void free_all();
    std::vector<DevBuf*> all_bufs();
    sdb_status derive();
    void host_random(int seed);
    sdb_status fit(const float* X, bool xOnDevice, float eps, int minPts, bool optics,
                   const SweepSpec* sw = nullptr);
    sdb_status check_flags();
    sdb_status optics_stage(const sdb::CoreArgs& ca, int& launches);
    sdb_status optics_order(int64_t total);
    // sngDbscan (optics = false; every eps of epsList, labels of eps i to
    // labelsOut + i n when given) or sngOptics (one eps)
    sdb_status fit_sng(const float* X, bool xOnDevice, const float* epsList, int nEps, int minPts, bool optics,
                       int32_t* labelsOut = nullptr, int32_t* nclOut = nullptr);
    // sngDbscan with independent samples per block of points (k_sng_blocks.cu)
    sdb_status fit_sng_blocks(const float* X, bool xOnDevice, const float* epsList, int nEps, int minPts, bool optics,
                              int32_t* labelsOut, int32_t* nclOut);

    static float* f32(DevBuf& b) { return static_cast<float*>(b.ptr); }
    static int32_t* i32(DevBuf& b) { return static_cast<int32_t*>(b.ptr); }
    static int64_t* i64(DevBuf& b) { return static_cast<int64_t*>(b.ptr); }
};
