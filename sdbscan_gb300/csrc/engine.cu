// The engine behind the C ABI (include/sdbscan_gb300.h): device buffers,
// host-side random numbers, the stage pipeline of fit_sDbscan / fit_sOptics,
// and the output accessors.
//
// Pipeline of one fit (all on the engine's stream; the only host syncs are
// at the end of the fit and in the accessors):
//   upload X -> [L1/L2: pad copy, random Fourier features]
//   -> k_colstats + k_project   transform, embedding, 3 x (signs + FWHT), top-k,
//                               projections, chunk extremes
//   -> top-m                    thresholds, collect, exact select (+ fallback)
//   -> index                    list members (inverted top-k), tiles, hub lists
//   -> k_dist                   grouped gathered distances, eps masks, in-counts
//   -> core                     de-duplicated neighbourhood sizes, core flags
//   -> cluster                  union-find labels   |  sOPTICS: core distance,
//                                                    neighbour lists, ordering
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/sdbscan_gb300.h"
#include "common.cuh"
#include "engine_internal.h"

namespace sdb {
int launch_tile_offsets(const IndexArgs& a, cudaStream_t st);
int launch_i32_to_i64(const int32_t* in, int64_t* out, int n, cudaStream_t st);
int dist_tile_rows();
int dist_tile_cols();
int launch_pad_copy(const float* X, int n, int d, float* Xt, int ld, cudaStream_t st);
}  // namespace sdb

using namespace sdb;

namespace {

// Point chunks per super-chunk of the tensor-core distance kernel's tile order
// (launch_tile_order_list), and the key count of that order's counting sort.
constexpr int kSuperChunk = 8;
size_t kTcKeys(int n, int L) {
    const int nChunks = (n + 4095) / 4096;
    return (size_t)((nChunks + kSuperChunk - 1) / kSuperChunk) * L + 1;
}

const char* dist_name(int d) {
    switch (d) {
        case SDB_COSINE: return "Cosine";
        case SDB_L1: return "L1";
        case SDB_L2: return "L2";
        case SDB_CHI2: return "Chi2";
        case SDB_JS: return "JS";
    }
    return "?";
}

}  // namespace

// ---------------------------------------------------------------------------
// device buffer helpers
// ---------------------------------------------------------------------------
bool sdb_engine::ensure(DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return true;
    if (dbgDeviceCap > 0 && devBytes - b.bytes + bytes > dbgDeviceCap) {
        fail(SDB_ERR_NOMEM, std::string("device allocation of ") + std::to_string(bytes) +
                                " bytes is over the engine's device memory cap of " + std::to_string(dbgDeviceCap));
        return false;
    }
    if (b.ptr) cudaFree(b.ptr);
    devBytes -= b.bytes;
    b.ptr = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(SDB_ERR_NOMEM, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " +
                                cudaGetErrorString(e));
        return false;
    }
    b.bytes = bytes;
    devBytes += bytes;
    return true;
}

sdb_status sdb_engine::fail(sdb_status s, const std::string& msg) {
    err = msg;
    return s;
}

sdb_status sdb_engine::cuda_fail(cudaError_t e, const char* where) {
    return fail(SDB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

void sdb_engine::free_all() {
    for (DevBuf* b : all_bufs())
        if (b->ptr) {
            cudaFree(b->ptr);
            b->ptr = nullptr;
            b->bytes = 0;
        }
    devBytes = 0;
}

std::vector<DevBuf*> sdb_engine::all_bufs() {
    return {&Xin, &Xt, &scale, &P, &topK, &chunkMax, &chunkMin, &thr, &cand, &candCount, &topM, &listCount,
            &listOff, &members, &tileOff, &tileList, &hubCount, &hubOff, &hubLists, &masks, &inRaw,
            &aCount, &degree, &core, &parent, &border, &rootFlag, &labels, &nClusters, &scanTmp, &errFlags,
            &counters, &E, &Rt, &signs, &compCosh, &dists, &coreDist, &nbOff, &nbIdx, &nbDist, &nbFill, &hubIdx,
            &kMask, &firstMasks, &Xb, &queue, &sweepLabels, &sweepNcl, &sig, &Rb, &newMasks, &coreEps, &sampleFlag,
            &noiseFlag, &noiseCores, &noisePts, &PcT, &numCore, &pairRound, &sngCols, &sngMult, &sngColOf, &sngExtras,
            &sngExtraPass, &sngMask, &rowDeg, &colCnt, &sngUb, &sngHeavy, &chunkOff, &tileKey, &keyOff, &tilePerm,
            &Cb, &tileKeyTc, &keyOffTc, &tilePermTc, &sngWords, &hashOffB, &hashIdB, &hashDistB, &sqNorm, &multiMask};
}

// ---------------------------------------------------------------------------
// parameters and host random numbers
// ---------------------------------------------------------------------------
sdb_status sdb_engine::derive() {
    const sdb_params& p = prm;
    if (p.n_proj < 1 || p.topK < 1 || p.topM < 1) return fail(SDB_ERR_ARG, "n_proj, topK and topM must be >= 1");
    if (p.topK > p.n_proj) return fail(SDB_ERR_ARG, "topK must be <= n_proj");
    if (p.topM > n) return fail(SDB_ERR_ARG, "topM must be <= n_points");
    if (p.distance < SDB_COSINE || p.distance > SDB_JS) return fail(SDB_ERR_ARG, "unknown distance");
    if (p.clusterNoise < 0 || p.clusterNoise > 2)
        return fail(SDB_ERR_ARG, "clusterNoise must be 0, 1 (sDbscan-1NN) or 2 (neighbour heuristic)");
    if (p.precision != SDB_PREC_FP32 && p.precision != SDB_PREC_BF16) return fail(SDB_ERR_ARG, "unknown precision");
    ker = p.distance == SDB_COSINE ? d : p.ker_n_features;  // src/sDbscan.h:102-104
    if (ker < 1) return fail(SDB_ERR_ARG, "ker_n_features must be >= 1");
    if ((p.distance == SDB_L1 || p.distance == SDB_L2) && ker % 2) return fail(SDB_ERR_ARG, "ker_n_features must be even for L1/L2");
    // embedChi2 / embedJS fill the first d slots of a ker-long vector
    // (src/Utilities.h:140-145): the reference requires ker >= d (src/sDbscan.cpp:54)
    if ((p.distance == SDB_CHI2 || p.distance == SDB_JS) && ker < d)
        return fail(SDB_ERR_ARG, "ker_n_features must be >= n_features for Chi2/JS");
    const int mx = std::max(p.n_proj, ker);
    fhtDim = 1 << (int)std::ceil(std::log2((double)mx));  // src/sDbscan.h:107
    if (fhtDim < 16) return fail(SDB_ERR_ARG, "max(n_proj, ker_n_features) must be >= 9");
    // vectors up to 2048 live in a warp's registers (k_project), up to 16384 in
    // a CTA's shared memory (k_project_smem); n_proj stays within 2048
    if (fhtDim > 16384) return fail(SDB_ERR_ARG, "max(n_proj, ker_n_features) must be <= 16384");
    if (p.n_proj > 2048) return fail(SDB_ERR_ARG, "n_proj must be <= 2048");
    if (p.topK > 31) return fail(SDB_ERR_ARG, "topK must be <= 31");
    if ((int64_t)n * 2 * p.topK >= ((int64_t)1 << 31))
        return fail(SDB_ERR_ARG, "n_points * 2 * topK must stay below 2^31 (32-bit member indexing)");
    ld = (d + 3) & ~3;
    return SDB_OK;
}

void sdb_engine::host_random(int seedUsed) {
    // bitHD3Generator (src/Utilities.h:47-64): fhtDim * 3 bits, one draw each.
    std::default_random_engine gen((unsigned)seedUsed);
    std::uniform_int_distribution<uint32_t> u(0, 1);
    const int nbits = 3 * fhtDim;
    hostSigns.assign((nbits + 31) / 32, 0u);
    for (int i = 0; i < nbits; ++i)
        if (u(gen) & 1) hostSigns[i >> 5] |= 1u << (i & 31);
    // gaussGenerator / cauchyGenerator (src/Utilities.h:76-122), (ker/2) x d,
    // column first; stored transposed (row r = R(r, :)) with row stride ld.
    hostRt.clear();
    if (prm.distance == SDB_L1 || prm.distance == SDB_L2) {
        const int h = ker / 2;
        hostRt.assign((size_t)h * ld, 0.0f);
        std::default_random_engine g2((unsigned)seedUsed);
        if (prm.distance == SDB_L2) {
            std::normal_distribution<float> nd(0.0f, 1.0f / prm.ker_sigma);
            for (int c = 0; c < d; ++c)
                for (int r = 0; r < h; ++r) hostRt[(size_t)r * ld + c] = nd(g2);
        } else {
            std::cauchy_distribution<float> cd(0.0f, 1.0f / prm.ker_sigma);
            for (int c = 0; c < d; ++c)
                for (int r = 0; r < h; ++r) hostRt[(size_t)r * ld + c] = cd(g2);
        }
    }
    // Chi2 / JS constants (src/Utilities.h:134-160, :176-204) evaluated on the host.
    hostCosh.clear();
    if (prm.distance == SDB_CHI2 || prm.distance == SDB_JS) {
        const int comps = ((ker / d) - 1) / 2;
        const double PI = 3.141592653589793238460;
        for (int c = 1; c <= comps; ++c) hostCosh.push_back(std::cosh(PI * c * (double)prm.ker_intervalSampling));
    }
    ln4 = std::log(4.0);
}

// ---------------------------------------------------------------------------
// the fit pipeline
// ---------------------------------------------------------------------------
sdb_status sdb_engine::fit(const float* X, bool xOnDevice, float eps, int minPts, bool optics, const SweepSpec* sw) {
    if (!paramsSet) return fail(SDB_ERR_STATE, "set_params must be called before a fit");
    const bool sweep = sw != nullptr, capture = sw != nullptr && sw->capture;
    if (sweep && (optics || sw->nEps < 1 || !sw->eps || !sw->labelsDev || !sw->nclDev))
        return fail(SDB_ERR_ARG, "invalid eps sweep");
    haveLabels = haveOptics = false;
    if (optics && minPts < 2) return fail(SDB_ERR_ARG, "minPts must be >= 2 for sOPTICS");
    if (X == nullptr) return fail(SDB_ERR_ARG, "X is null");
    sdb_status s = derive();
    if (s != SDB_OK) return s;
    const sdb_params& p = prm;
    const int k = p.topK, m = p.topM, D = p.n_proj;
    if (!capture) {
        seedUsed = p.random_seed >= 0 ? p.random_seed
                                      : (int)(unsigned)std::chrono::system_clock::now().time_since_epoch().count();
        host_random(seedUsed);
    }
    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");

    const int TMr = dist_tile_rows(), TNc = dist_tile_cols();
    const int nct = (m + TNc - 1) / TNc;
    const int W = (m + 63) / 64;
    const int L = 2 * D;
    // top-m threshold chunks: six chunks per projection block of one full
    // wave (project_wave_chunks), so the grid-stride blocks end together, and
    // at least 4m chunks so the chunk maxima bound the m-th value
    const int chunksWanted = std::max(project_wave_chunks() * 6, 4 * m);
    const int chunk = std::max(8, (n + chunksWanted - 1) / chunksWanted);
    const int G = (n + chunk - 1) / chunk;
    int cap = 256;
    while (cap < 8 * m) cap <<= 1;
    const int64_t maxTiles = ((int64_t)n * 2 * k / TMr + L) * nct;
    const bool rff = p.distance == SDB_L1 || p.distance == SDB_L2;
    // BF16 tensor-core screening of the candidate distances: Cosine sDBSCAN
    // fits and eps sweeps of up to kMaxScreenedSweep values (the projection
    // kernel writes the BF16 copy of the rows when it runs its register path),
    // and L2 sDBSCAN fits (split-BF16 rows, made for the embedding GEMM)
    const bool screen = p.precision == SDB_PREC_BF16 && !optics &&
                        ((p.distance == SDB_COSINE && (!sweep || sw->nEps <= kMaxScreenedSweep)) ||
                         (p.distance == SDB_L2 && !sweep));
    const int ldb = (d + 63) / 64 * 64;
    const bool fuseXb = screen && p.distance == SDB_COSINE && fhtDim <= 2048 && ldb <= fhtDim;

    // allocations (grow-only)
    bool ok = true;
    if (!xOnDevice) ok &= ensure(Xin, sizeof(float) * (size_t)n * d);
    ok &= ensure(Xt, sizeof(float) * (size_t)n * ld) && ensure(scale, sizeof(float) * n) &&
          ensure(P, sizeof(float) * (size_t)n * D) && ensure(topK, sizeof(int32_t) * (size_t)n * 2 * k) &&
          ensure(chunkMax, sizeof(float) * (size_t)G * D) && ensure(chunkMin, sizeof(float) * (size_t)G * D) &&
          ensure(thr, sizeof(float) * 2 * D) && ensure(cand, sizeof(uint64_t) * (size_t)L * cap) &&
          ensure(candCount, sizeof(int32_t) * L) && ensure(topM, sizeof(int32_t) * (size_t)D * 2 * m) &&
          ensure(listCount, sizeof(int64_t) * (L + 1)) && ensure(listOff, sizeof(int64_t) * (L + 1)) &&
          ensure(members, sizeof(int2) * (size_t)n * 2 * k) &&
          ensure(tileOff, sizeof(int64_t) * (L + 1)) && ensure(tileList, sizeof(int32_t) * (size_t)maxTiles) &&
          ensure(hubCount, sizeof(int32_t) * n) && ensure(hubOff, sizeof(int64_t) * (n + 1)) &&
          ensure(hubLists, sizeof(int32_t) * (size_t)L * m) &&
          ensure(masks, sizeof(uint64_t) * (size_t)n * 2 * k * W) && ensure(inRaw, sizeof(int32_t) * n) &&
          ensure(firstMasks, sizeof(uint64_t) * (size_t)n * 2 * k * W) &&
          ensure(aCount, sizeof(int32_t) * n) && ensure(degree, sizeof(int32_t) * n) && ensure(core, n) &&
          ensure(parent, sizeof(int32_t) * n) && ensure(border, sizeof(int32_t) * n) &&
          ensure(rootFlag, sizeof(int64_t) * (n + 1)) && ensure(labels, sizeof(int32_t) * n) &&
          ensure(nClusters, sizeof(int32_t) * 4) &&
          ensure(scanTmp, sizeof(int64_t) * scan_tmp_elems(std::max<size_t>((size_t)std::max(n + 1, L + 1),
                                                                             kTcKeys(n, L)))) &&
          ensure(errFlags, sizeof(int32_t) * kErrSlots) && ensure(counters, sizeof(unsigned long long) * 8) &&
          ensure(signs, sizeof(uint32_t) * hostSigns.size()) &&
          ensure(compCosh, sizeof(double) * std::max<size_t>(1, hostCosh.size()));
    const int chunkPts = 4096, nChunks = (n + chunkPts - 1) / chunkPts;
    ok &= ensure(chunkOff, sizeof(int32_t) * (size_t)L * nChunks) && ensure(tileKey, sizeof(int32_t) * maxTiles) &&
          ensure(keyOff, sizeof(int64_t) * ((size_t)nChunks + 1)) && ensure(tilePerm, sizeof(int32_t) * maxTiles);
    const int maskWords = (L + 31) / 32;
    const size_t maxHubs = std::min<size_t>((size_t)n, (size_t)L * m);
    ok &= ensure(hubIdx, sizeof(int32_t) * n) && ensure(kMask, sizeof(uint32_t) * maxHubs * maskWords) &&
          ensure(sig, 16 * (size_t)L * m) && ensure(multiMask, sizeof(uint64_t) * (size_t)L * W);
    if (rff) ok &= ensure(E, sizeof(float) * (size_t)n * ker) && ensure(Rt, sizeof(float) * hostRt.size());
    if (optics || sweep) ok &= ensure(dists, sizeof(float) * (size_t)n * 2 * k * m);
    if (optics) ok &= ensure(coreDist, sizeof(float) * n);
    if (!ok) return SDB_ERR_NOMEM;

    cudaStream_t st = stream;
    int launches = 0;
    auto L_ = [&](int r) {
        if (r < 0) ok = false;
        else launches += r;
    };
#define SDB_CK(call)                                     \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

    if (!capture) SDB_CK(cudaEventRecord(ev[0], st));
    const float* Xd = X;
    // host input without an embedding GEMM: the upload runs in segments on the
    // copy stream and overlaps stage 1 (the "upload" stage time then reads 0)
    const bool overlapUpload = !xOnDevice && !rff && !capture;
    if (!xOnDevice) {
        Xd = static_cast<const float*>(Xin.ptr);
        if (!overlapUpload)
            SDB_CK(cudaMemcpyAsync(Xin.ptr, X, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
    }
    if (!capture) SDB_CK(cudaEventRecord(ev[1], st));
    if (!capture) {  // a captured sweep reuses the signs its sizing run uploaded
        SDB_CK(cudaMemcpyAsync(signs.ptr, hostSigns.data(), sizeof(uint32_t) * hostSigns.size(),
                               cudaMemcpyHostToDevice, st));
        if (!hostCosh.empty())
            SDB_CK(cudaMemcpyAsync(compCosh.ptr, hostCosh.data(), sizeof(double) * hostCosh.size(),
                                   cudaMemcpyHostToDevice, st));
    }
    SDB_CK(cudaMemsetAsync(errFlags.ptr, 0, sizeof(int32_t) * kErrSlots, st));
    SDB_CK(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8, st));
    unsigned long long* ctr = static_cast<unsigned long long*>(counters.ptr);

    // ---- stage 1: transform, embedding, projection, top-k ------------------
    ProjectArgs pa{};
    pa.X = Xd;
    pa.ldx = d;
    pa.Xt = f32(Xt);
    pa.ld = ld;
    pa.n = n;
    pa.d = d;
    pa.dist = p.distance;
    pa.ker = ker;
    pa.kerSam = p.ker_intervalSampling;
    pa.E = nullptr;
    pa.signs = static_cast<const uint32_t*>(signs.ptr);
    pa.fhtDim = fhtDim;
    pa.nproj = D;
    pa.k = k;
    pa.P = f32(P);
    pa.topK = i32(topK);
    pa.chunkMax = f32(chunkMax);
    pa.chunkMin = f32(chunkMin);
    pa.chunk = chunk;
    pa.err = i32(errFlags);
    pa.ties = ctr + 0;
    pa.do_transform = 1;
    pa.scale = f32(scale);
    pa.compCosh = static_cast<const double*>(compCosh.ptr);
    pa.ln4 = ln4;
    if (fuseXb) {
        if (!ensure(Xb, sizeof(uint16_t) * (size_t)n * ldb)) return SDB_ERR_NOMEM;
        pa.Xb = static_cast<uint16_t*>(Xb.ptr);
        pa.ldb = ldb;
    }
    if (rff) {
        if (!capture)
            SDB_CK(cudaMemcpyAsync(Rt.ptr, hostRt.data(), sizeof(float) * hostRt.size(), cudaMemcpyHostToDevice, st));
        L_(launch_pad_copy(Xd, n, d, f32(Xt), ld, st));
        const int h = ker / 2;
        int tcr = -1;
        if (p.precision == SDB_PREC_BF16) {
            // the embedding GEMM on the tensor cores from split-BF16 copies of X
            // and R; the FP32 kernel after it runs only if the tensor-core one failed
            if (!ensure(Xb, sizeof(uint16_t) * (size_t)n * 2 * ldb) ||
                !ensure(Rb, sizeof(uint16_t) * (size_t)h * 2 * ldb))
                return SDB_ERR_NOMEM;
            L_(launch_to_bf16_split(f32(Xt), ld, n, Xb.ptr, ldb, st));
            L_(launch_to_bf16_split(f32(Rt), ld, h, Rb.ptr, ldb, st));
            tcr = launch_rff_tc(Xb.ptr, Rb.ptr, n, h, ldb, f32(E), i32(errFlags) + 5, dbgStallSpins, st);
            if (tcr > 0) launches += tcr;
        }
        L_(launch_rff(f32(Xt), ld, n, d, f32(Rt), h, f32(E), st, tcr > 0 ? i32(errFlags) + 5 : nullptr));
        pa.X = f32(Xt);
        pa.ldx = ld;
        pa.E = f32(E);
        pa.do_transform = 0;
    }
    if (overlapUpload) {
        const int segs = std::min(kUploadSegs, G);
        SDB_CK(cudaEventRecord(segEv[kUploadSegs], st));  // Xin is free once the stream got here
        for (int c = 0; c < kCopyStreams; ++c) SDB_CK(cudaStreamWaitEvent(copyStream[c], segEv[kUploadSegs], 0));
        // every copy is queued before the first projection launch, so a delay
        // of the host thread while it queues the launches cannot starve the
        // copy engine
        for (int sgi = 0; sgi < segs; ++sgi) {
            const int cb = (int)((int64_t)G * sgi / segs), ce = (int)((int64_t)G * (sgi + 1) / segs);
            const size_t pb = (size_t)cb * chunk, pe = std::min<size_t>((size_t)n, (size_t)ce * chunk);
            cudaStream_t cs = copyStream[sgi % kCopyStreams];  // one cudaMemcpyAsync per segment
            SDB_CK(cudaMemcpyAsync(static_cast<float*>(Xin.ptr) + pb * d, X + pb * d, sizeof(float) * (pe - pb) * d,
                                   cudaMemcpyHostToDevice, cs));
            SDB_CK(cudaEventRecord(segEv[sgi], cs));
        }
        for (int sgi = 0; sgi < segs; ++sgi) {
            SDB_CK(cudaStreamWaitEvent(st, segEv[sgi], 0));
            pa.chunkBase = (int)((int64_t)G * sgi / segs);
            pa.chunkEnd = (int)((int64_t)G * (sgi + 1) / segs);
            L_(launch_project(pa, st));
        }
        pa.chunkBase = pa.chunkEnd = 0;
    } else {
        L_(launch_project(pa, st));
    }
    if (!ok) return fail(SDB_ERR_CUDA, std::string("projection launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (!capture) SDB_CK(cudaEventRecord(ev[2], st));

    // ---- stage 2: per-vector top-m -----------------------------------------
    TopMArgs ta{};
    ta.P = f32(P);
    ta.n = n;
    ta.nproj = D;
    ta.m = m;
    ta.chunkMax = f32(chunkMax);
    ta.chunkMin = f32(chunkMin);
    ta.G = G;
    ta.thrMax = f32(thr);
    ta.thrMin = f32(thr) + D;
    ta.cand = static_cast<uint64_t*>(cand.ptr);
    ta.candCount = i32(candCount);
    ta.cap = cap;
    ta.topM = i32(topM);
    ta.ties = ctr + 1;
    ta.errFlag = i32(errFlags) + 3;
    SDB_CK(cudaMemsetAsync(candCount.ptr, 0, sizeof(int32_t) * L, st));
    L_(launch_topm_thresholds(ta, st));
    L_(launch_topm_collect(ta, st));
    L_(launch_topm_select(ta, st));
    if (!ok) return fail(SDB_ERR_CUDA, std::string("top-m launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (!capture) SDB_CK(cudaEventRecord(ev[3], st));

    // ---- stage 3: inverted index, tiles, hub lists ---------------------------
    IndexArgs ia{};
    ia.topK = i32(topK);
    ia.n = n;
    ia.k = k;
    ia.nproj = D;
    ia.m = m;
    ia.topM = i32(topM);
    ia.listCount = i64(listCount);
    ia.listOff = i64(listOff);
    ia.members = static_cast<int2*>(members.ptr);
    ia.TM = TMr;
    ia.nct = nct;
    ia.tileOff = i64(tileOff);
    ia.tileList = i32(tileList);
    ia.hubCount = i32(hubCount);
    ia.hubOff = i64(hubOff);
    ia.hubLists = i32(hubLists);
    ia.scanTmp = i64(scanTmp);
    ia.chunkPts = chunkPts;
    ia.nChunks = nChunks;
    ia.chunkOff = i32(chunkOff);
    ia.tileKey = i32(tileKey);
    ia.keyOff = i64(keyOff);
    ia.tilePerm = i32(tilePerm);
    ia.maxTiles = maxTiles;
    SDB_CK(cudaMemsetAsync(listCount.ptr, 0, sizeof(int64_t) * (L + 1), st));
    SDB_CK(cudaMemsetAsync(hubCount.ptr, 0, sizeof(int32_t) * n, st));
    SDB_CK(cudaMemsetAsync(hubOff.ptr, 0, sizeof(int64_t) * (n + 1), st));
    L_(launch_index_count(ia, st));
    L_(launch_scan_i64(i64(listCount), i64(listOff), (size_t)L + 1, i64(scanTmp), st));
    L_(launch_index_scatter(ia, st));
    L_(launch_tile_offsets(ia, st));
    L_(launch_tiles(ia, 0, st));
    L_(launch_tile_order(ia, st));
    L_(launch_hubs_count(ia, st));
    L_(launch_i32_to_i64(i32(hubCount), i64(hubOff), n, st));
    L_(launch_scan_i64(i64(hubOff), i64(hubOff), (size_t)n + 1, i64(scanTmp), st));
    SDB_CK(cudaMemsetAsync(hubCount.ptr, 0, sizeof(int32_t) * n, st));
    L_(launch_hubs_scatter(ia, st));
    L_(launch_slot_sigs(i32(topM), D, m, i64(hubOff), i32(hubLists), sig.ptr, static_cast<uint64_t*>(multiMask.ptr), W,
                        st));
    if (!ok) return fail(SDB_ERR_CUDA, std::string("index launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (!capture) SDB_CK(cudaEventRecord(ev[4], st));

    // ---- stage 4: distances + eps --------------------------------------------
    DistArgs da{};
    da.Xt = f32(Xt);
    da.ld = ld;
    da.d = d;
    da.dist = p.distance;
    da.n = n;
    da.members = static_cast<const int2*>(members.ptr);
    da.listOff = i64(listOff);
    da.tileList = i32(tileList);
    da.tileOff = i64(tileOff);
    da.nTiles = maxTiles;
    da.tileTotal = i64(tileOff) + L;
    da.tilePerm = i32(tilePerm);
    da.topM = i32(topM);
    da.nproj = D;
    da.m = m;
    da.k = k;
    da.W = W;
    da.nct = nct;
    da.eps = eps;
    if (sweep) da.eps = *std::max_element(sw->eps, sw->eps + sw->nEps);
    da.masks = static_cast<uint64_t*>(masks.ptr);
    da.inRaw = i32(inRaw);
    da.dists = (optics || sweep) ? f32(dists) : nullptr;
    da.pairs = ctr + 3;
    da.topKmat = i32(topK);
    da.variant = distVariant;
    da.waitErr = i32(errFlags) + 8;
    da.stallSpins = dbgStallSpins;
    SDB_CK(cudaMemsetAsync(inRaw.ptr, 0, sizeof(int32_t) * n, st));
    // BF16 tensor-core screening + exact FP32 re-decision near eps.  The
    // plain kernel is launched after it in every case and runs only if the
    // screening raised its flag (queue overflow or a timed-out wait), so the
    // stage needs no host synchronisation and can be captured in a graph.
    if (screen) {
        if (sweep) {  // ascending, as the rounds run
            da.nSweep = sw->nEps;
            for (int e = 0; e < sw->nEps; ++e) da.sweepEps[e] = sw->eps[e];
            std::sort(da.sweepEps, da.sweepEps + sw->nEps);
        }
        const int64_t qcap = dbgQueueCap > 0 ? dbgQueueCap : std::max<int64_t>(1 << 20, (int64_t)n * 2 * k * m / 8);
        const bool l2 = p.distance == SDB_L2;  // split rows [hi | lo] from stage 1, squared norms
        if (!ensure(Xb, sizeof(uint16_t) * (size_t)n * (l2 ? 2 : 1) * ldb) ||
            !ensure(queue, sizeof(uint64_t) * (size_t)qcap) || !ensure(Cb, dist_tc_cand_bytes(da, ldb)) ||
            (l2 && !ensure(sqNorm, sizeof(float) * (size_t)n)))
            return SDB_ERR_NOMEM;
        if (l2) {
            L_(launch_sq_norms(f32(Xt), ld, n, f32(sqNorm), st));
            da.sqNorm = f32(sqNorm);
        } else if (!fuseXb) {
            L_(launch_to_bf16(f32(Xt), ld, n, Xb.ptr, ldb, st));
        }
        // the tensor-core kernel takes the tiles by (super-chunk, list): the
        // rows of 8 point chunks stay in L2 while every list passes over them
        const size_t nKeys = tile_order_list_keys(ia, kSuperChunk);
        if (!ensure(tileKeyTc, sizeof(int32_t) * (size_t)maxTiles) || !ensure(keyOffTc, sizeof(int64_t) * nKeys) ||
            !ensure(tilePermTc, sizeof(int32_t) * (size_t)maxTiles))
            return SDB_ERR_NOMEM;
        L_(launch_tile_order_list(ia, kSuperChunk, i32(tileKeyTc), i64(keyOffTc), i32(tilePermTc), st));
        DistArgs dtc = da;
        dtc.tilePerm = i32(tilePermTc);
        L_(launch_dist_tc(dtc, Xb.ptr, ldb, Cb.ptr, static_cast<uint64_t*>(queue.ptr), qcap, ctr + 4,
                          i32(errFlags) + 4, st));
        L_(launch_recheck(da, static_cast<const uint64_t*>(queue.ptr), ctr + 4, qcap, st));
        da.gate = i32(errFlags) + 4;
        L_(launch_screen_reset(da, st));
        if (!ok) return fail(SDB_ERR_CUDA, std::string("tensor-core distance launch failed: ") +
                                               cudaGetErrorString(cudaGetLastError()));
    }
    L_(launch_dist(da, st));
    if (!ok) return fail(SDB_ERR_CUDA, std::string("distance launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (!capture) SDB_CK(cudaEventRecord(ev[5], st));

    // ---- stage 5: neighbourhood sizes, core flags -----------------------------
    CoreArgs ca{};
    ca.n = n;
    ca.k = k;
    ca.m = m;
    ca.W = W;
    ca.nproj = D;
    ca.minPts = minPts;
    ca.masks = static_cast<const uint64_t*>(masks.ptr);
    ca.topK = i32(topK);
    ca.topM = i32(topM);
    ca.hubCount = i32(hubCount);
    ca.hubOff = i64(hubOff);
    ca.hubLists = i32(hubLists);
    ca.multi = static_cast<const uint64_t*>(multiMask.ptr);
    ca.inRaw = i32(inRaw);
    ca.aCount = i32(aCount);
    ca.degree = i32(degree);
    ca.core = static_cast<uint8_t*>(core.ptr);
    ca.dists = optics ? f32(dists) : nullptr;
    ca.coreDist = optics ? f32(coreDist) : nullptr;
    ca.hubIdx = i32(hubIdx);
    ca.kMask = static_cast<const uint32_t*>(kMask.ptr);
    ca.firstMasks = static_cast<uint64_t*>(firstMasks.ptr);
    SDB_CK(cudaMemsetAsync(kMask.ptr, 0, sizeof(uint32_t) * maxHubs * maskWords, st));
    L_(launch_hub_masks(ca, i32(hubIdx), i64(rootFlag), static_cast<uint32_t*>(kMask.ptr), i64(scanTmp),
                        reinterpret_cast<int64_t*>(ctr + 5), st));
    const int rounds = sweep ? sw->nEps : 1;
    // an eps sweep runs in ascending eps: each round adds the pairs with
    // previous eps < d <= eps to the degrees, the first-occurrence masks and
    // the union-find of the round before (neighbourhoods only grow with eps)
    std::vector<int> ord(rounds, 0);
    if (sweep) {
        for (int i = 0; i < rounds; ++i) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return sw->eps[x] < sw->eps[y]; });
        if (rounds <= kMaxScreenedSweep) {  // one byte per pair: the round in which it joins
            da.nSweep = rounds;
            for (int e = 0; e < rounds; ++e) da.sweepEps[e] = sw->eps[ord[e]];
            if (!ensure(pairRound, (size_t)n * 2 * k * W * 64)) return SDB_ERR_NOMEM;
            L_(launch_pair_rounds(da, static_cast<uint8_t*>(pairRound.ptr), st));
            da.pairRound = static_cast<const uint8_t*>(pairRound.ptr);
        }
        if (!ensure(newMasks, sizeof(uint64_t) * (size_t)n * 2 * k * W) || !ensure(coreEps, sizeof(int32_t) * n))
            return SDB_ERR_NOMEM;
        SDB_CK(cudaMemsetAsync(degree.ptr, 0, sizeof(int32_t) * n, st));
        SDB_CK(cudaMemsetAsync(core.ptr, 0, n, st));
        SDB_CK(cudaMemsetAsync(coreEps.ptr, 0xFF, sizeof(int32_t) * n, st));
        SDB_CK(cudaMemsetAsync(firstMasks.ptr, 0, sizeof(uint64_t) * (size_t)n * 2 * k * W, st));
        ca.accumulate = 1;
        ca.newMasks = static_cast<uint64_t*>(newMasks.ptr);
        ca.coreEps = i32(coreEps);
    }
    for (int ei = 0; ei < rounds; ++ei) {
    const int eo = ord[ei];  // the eps value (and output slot) of this round
    if (sweep) {  // this eps: new pairs' masks and reverse counts from the stored distances
        da.eps = sw->eps[eo];
        da.epsLo = ei > 0 ? sw->eps[ord[ei - 1]] : -INFINITY;
        da.round = ei;
        ca.round = ei;
        SDB_CK(cudaMemsetAsync(inRaw.ptr, 0, sizeof(int32_t) * n, st));
        L_(launch_masks_from_dists(da, st));
    }
    L_(launch_core_dedupe(ca, sig.ptr, st));
    L_(launch_core_finish(ca, st));
    if (!ok) return fail(SDB_ERR_CUDA, std::string("core launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (!capture) SDB_CK(cudaEventRecord(ev[6], st));

    // ---- stage 6: clusters or sOPTICS ------------------------------------------
    if (!optics) {
        ClusterArgs ka{};
        ka.n = n;
        ka.k = k;
        ka.m = m;
        ka.W = W;
        ka.masks = static_cast<const uint64_t*>(firstMasks.ptr);
        ka.topK = i32(topK);
        ka.topM = i32(topM);
        ka.members = static_cast<const int2*>(members.ptr);
        ka.listOff = i64(listOff);
        ka.tileList = i32(tileList);
        ka.tileOff = i64(tileOff);
        ka.tileTotal = i64(tileOff) + L;
        ka.tilePerm = i32(tilePerm);
        ka.nTiles = maxTiles;
        ka.TM = TMr;
        ka.nct = nct;
        ka.nproj = D;
        ka.core = static_cast<const uint8_t*>(core.ptr);
        ka.parent = i32(parent);
        ka.border = i32(border);
        ka.rootFlag = i64(rootFlag);
        ka.scanTmp = i64(scanTmp);
        ka.labels = i32(labels);
        ka.nClusters = i32(nClusters);
        if (sweep) {
            ka.carry = 1;
            ka.round = ei;
            ka.newMasks = static_cast<const uint64_t*>(newMasks.ptr);
            ka.coreEps = i32(coreEps);
        }
        L_(launch_cluster(ka, st));
        if (p.clusterNoise == 1) {  // sDbscan-1NN labels for the points left as noise
            const float sp = p.samplingProb;
            const int sMax = (int)std::min<double>((double)n, 2.0 * std::max(0.0f, sp) * n + 4096.0);
            if (!ensure(sampleFlag, sizeof(int64_t) * (n + 1)) || !ensure(noiseFlag, sizeof(int64_t) * (n + 1)) ||
                !ensure(noiseCores, sizeof(int32_t) * sMax) || !ensure(noisePts, sizeof(int32_t) * n) ||
                !ensure(PcT, sizeof(float) * (size_t)D * sMax) || !ensure(numCore, sizeof(int32_t)))
                return SDB_ERR_NOMEM;
            NoiseArgs na{};
            na.n = n;
            na.nproj = D;
            na.k = k;
            na.P = f32(P);
            na.topK = i32(topK);
            na.core = static_cast<const uint8_t*>(core.ptr);
            na.labels = i32(labels);
            na.samplingProb = sp;
            na.seed = (uint32_t)seedUsed;
            na.sMax = sMax;
            na.sampleFlag = i64(sampleFlag);
            na.noiseFlag = i64(noiseFlag);
            na.cores = i32(noiseCores);
            na.noise = i32(noisePts);
            na.PcT = f32(PcT);
            na.numCore = i32(numCore);
            na.scanTmp = i64(scanTmp);
            L_(launch_label_noise(na, st));
        }
        if (!ok) return fail(SDB_ERR_CUDA, std::string("cluster launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    } else {
        s = optics_stage(ca, launches);
        if (s != SDB_OK) return s;
    }
    if (sweep) {
        SDB_CK(cudaMemcpyAsync(sw->labelsDev + (size_t)eo * n, labels.ptr, sizeof(int32_t) * n,
                               cudaMemcpyDeviceToDevice, st));
        SDB_CK(cudaMemcpyAsync(sw->nclDev + eo, nClusters.ptr, sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
    }
    }  // eps rounds
    if (!capture) SDB_CK(cudaEventRecord(ev[7], st));
    SDB_CK(cudaMemcpyAsync(hostErr, errFlags.ptr, sizeof(int32_t) * kErrSlots, cudaMemcpyDeviceToHost, st));
    SDB_CK(cudaMemcpyAsync(hostCounters, counters.ptr, sizeof(unsigned long long) * 8, cudaMemcpyDeviceToHost, st));
    launchCount = launches;
    if (capture) return SDB_OK;  // flags are read by check_flags() after the graph has run
    SDB_CK(cudaEventRecord(ev[8], st));
    SDB_CK(cudaStreamSynchronize(st));
#undef SDB_CK
    for (int i = 0; i < 8; ++i) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        stageMs[i] = ms;
    }
    {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[0], ev[8]);
        stageMs[8] = ms;
    }
    s = check_flags();
    if (s != SDB_OK) return s;
    if (optics) haveOptics = true;
    else haveLabels = true;
    haveFit = true;
    lastOptics = optics;
    lastSng = false;
    if (p.verbose) {
        std::printf("sdbscan_gb300 %s fit: n=%d d=%d D=%d k=%d m=%d dist=%s eps=%g minPts=%d\n",
                    optics ? "sOPTICS" : "sDBSCAN", n, d, D, k, m, dist_name(p.distance), eps, minPts);
        const char* names[9] = {"upload", "project+topk", "topm", "index", "distances", "core", "cluster/optics",
                                "readback", "total"};
        for (int i = 0; i < 9; ++i) std::printf("  %-14s %9.3f ms\n", names[i], stageMs[i]);
    }
    err.clear();
    return SDB_OK;
}

// Error flags the kernels raised during the last (synchronised) fit.
sdb_status sdb_engine::check_flags() {
    if (hostErr[4]) fallbacks += 1;  // the screened stage was redone on the plain path
    if (hostErr[5]) fallbacks += 1;  // the tensor-core embedding was redone in FP32
    if (hostErr[7]) fallbacks += 1;  // the sngDbscan block was redone in FP32
    if (hostErr[0]) return fail(SDB_ERR_NEGATIVE, "X is not non-negative (Chi2/JS need nonnegative data)");
    if (hostErr[1])
        return fail(SDB_ERR_ZERO_POINT, prm.distance == SDB_COSINE ? "X has a point of zero norm (Cosine)"
                                                                   : "X has a point of zero sum (Chi2/JS)");
    if (hostErr[2]) return fail(SDB_ERR_ARG, "X has a non-finite value");
    if (hostErr[3]) return fail(SDB_ERR_INTERNAL, "top-m selection found fewer candidates than topM");
    if (hostErr[8]) return fail(SDB_ERR_INTERNAL, "a bounded wait of the distance kernel ran out");
    return SDB_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void sdb_params_default(sdb_params* p) {
    if (!p) return;
    p->n_proj = 1024;
    p->topK = 10;
    p->topM = 50;
    p->distance = SDB_COSINE;
    p->ker_n_features = 1024;
    p->ker_sigma = 1.0f;
    p->ker_intervalSampling = 0.4f;
    p->clusterNoise = 0;
    p->samplingProb = 0.01f;
    p->verbose = 0;
    p->n_threads = -1;
    p->random_seed = -1;
    p->precision = SDB_PREC_FP32;
}

sdb_status sdb_engine_create(int32_t n_points, int32_t n_features, int32_t device, sdb_engine** out) {
    if (!out) return SDB_ERR_ARG;
    *out = nullptr;
    if (n_points < 1 || n_features < 1) return SDB_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return SDB_ERR_CUDA;
    }
    if (device < 0 || device >= count) return SDB_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SDB_ERR_CUDA;
    sdb_engine* e = new sdb_engine();
    e->n = n_points;
    e->d = n_features;
    e->device = device;
    sdb_params_default(&e->prm);
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        sdb_engine_destroy(e);
        return SDB_ERR_CUDA;
    }
    for (int c = 0; c < sdb_engine::kCopyStreams; ++c)
        if (cudaStreamCreateWithFlags(&e->copyStream[c], cudaStreamNonBlocking) != cudaSuccess) {
            sdb_engine_destroy(e);
            return SDB_ERR_CUDA;
        }
    for (int i = 0; i <= sdb_engine::kUploadSegs; ++i)
        if (cudaEventCreateWithFlags(&e->segEv[i], cudaEventDisableTiming) != cudaSuccess) {
            sdb_engine_destroy(e);
            return SDB_ERR_CUDA;
        }
    for (int i = 0; i < 9; ++i)
        if (cudaEventCreate(&e->ev[i]) != cudaSuccess) {
            sdb_engine_destroy(e);
            return SDB_ERR_CUDA;
        }
    if (cudaMallocHost(&e->hostErr, sizeof(int32_t) * kErrSlots) != cudaSuccess ||
        cudaMallocHost(&e->hostCounters, sizeof(unsigned long long) * 8) != cudaSuccess) {
        sdb_engine_destroy(e);
        return SDB_ERR_CUDA;
    }
    *out = e;
    return SDB_OK;
}

void sdb_engine_destroy(sdb_engine* e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (cudaStream_t cs : e->copyStream)
        if (cs) cudaStreamSynchronize(cs);
    e->free_all();
    for (int i = 0; i < 9; ++i)
        if (e->ev[i]) cudaEventDestroy(e->ev[i]);
    for (int i = 0; i <= sdb_engine::kUploadSegs; ++i)
        if (e->segEv[i]) cudaEventDestroy(e->segEv[i]);
    for (cudaStream_t cs : e->copyStream)
        if (cs) cudaStreamDestroy(cs);
    if (e->hostErr) cudaFreeHost(e->hostErr);
    if (e->hostCounters) cudaFreeHost(e->hostCounters);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

sdb_status sdb_set_params(sdb_engine* e, const sdb_params* p) {
    if (!e || !p) return SDB_ERR_ARG;
    e->prm = *p;
    e->paramsSet = true;
    sdb_status s = e->derive();
    if (s != SDB_OK) e->paramsSet = false;
    return s;
}

sdb_status sdb_set_tile_variant(sdb_engine* e, int32_t variant) {
    if (!e) return SDB_ERR_ARG;
    if (variant < 0 || variant > 5) return e->fail(SDB_ERR_ARG, "tile variant must be 0..5");
    e->distVariant = variant;
    return SDB_OK;
}

sdb_status sdb_set_debug_limits(sdb_engine* e, int64_t stall_spins, int64_t queue_cap, int64_t device_bytes_cap) {
    if (!e) return SDB_ERR_ARG;
    if (stall_spins < 0 || queue_cap < 0 || device_bytes_cap < 0)
        return e->fail(SDB_ERR_ARG, "debug limits must be >= 0 (0 = off)");
    e->dbgStallSpins = stall_spins;
    e->dbgQueueCap = queue_cap;
    e->dbgDeviceCap = (size_t)device_bytes_cap;
    return SDB_OK;
}

sdb_status sdb_set_precision(sdb_engine* e, int32_t precision) {
    if (!e) return SDB_ERR_ARG;
    if (precision != SDB_PREC_FP32 && precision != SDB_PREC_BF16) return e->fail(SDB_ERR_ARG, "unknown precision");
    e->prm.precision = precision;
    return SDB_OK;
}

sdb_status sdb_fit_sdbscan(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit(X, false, eps, minPts, false) : SDB_ERR_ARG;
}
sdb_status sdb_fit_sdbscan_device(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit(X, true, eps, minPts, false) : SDB_ERR_ARG;
}
sdb_status sdb_fit_soptics(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit(X, false, eps, minPts, true) : SDB_ERR_ARG;
}
sdb_status sdb_fit_soptics_device(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit(X, true, eps, minPts, true) : SDB_ERR_ARG;
}

sdb_status sdb_fit_sdbscan_sweep(sdb_engine* e, const float* X, const float* eps, int32_t n_eps, int32_t minPts,
                                 int32_t* labels, int32_t* n_clusters) {
    if (!e) return SDB_ERR_ARG;
    if (!eps || n_eps < 1 || !labels || !n_clusters) return e->fail(SDB_ERR_ARG, "eps list and outputs are required");
    cudaSetDevice(e->device);
    if (!e->ensure(e->sweepLabels, sizeof(int32_t) * (size_t)n_eps * e->n) ||
        !e->ensure(e->sweepNcl, sizeof(int32_t) * n_eps))
        return SDB_ERR_NOMEM;
    SweepSpec sw;
    sw.eps = eps;
    sw.nEps = n_eps;
    sw.labelsDev = static_cast<int32_t*>(e->sweepLabels.ptr);
    sw.nclDev = static_cast<int32_t*>(e->sweepNcl.ptr);
    sdb_status s = e->fit(X, false, eps[0], minPts, false, &sw);
    if (s != SDB_OK) return s;
    cudaError_t c = cudaMemcpyAsync(labels, sw.labelsDev, sizeof(int32_t) * (size_t)n_eps * e->n,
                                    cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess)
        c = cudaMemcpyAsync(n_clusters, sw.nclDev, sizeof(int32_t) * n_eps, cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    return c == cudaSuccess ? SDB_OK : e->cuda_fail(c, "sweep download");
}

sdb_status sdb_get_labels(sdb_engine* e, int32_t* labels, int32_t* n_clusters) {
    if (!e) return SDB_ERR_ARG;
    if (!e->haveLabels) return e->fail(SDB_ERR_STATE, "no sDbscan result: call sdb_fit_sdbscan first");
    cudaSetDevice(e->device);
    if (labels) {
        cudaError_t c = cudaMemcpyAsync(labels, e->labels.ptr, sizeof(int32_t) * e->n, cudaMemcpyDeviceToHost, e->stream);
        if (c != cudaSuccess) return e->cuda_fail(c, "labels download");
    }
    int32_t nc = 0;
    cudaError_t c = cudaMemcpyAsync(&nc, e->nClusters.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream);
    if (c != cudaSuccess) return e->cuda_fail(c, "n_clusters download");
    c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return e->cuda_fail(c, "labels sync");
    if (n_clusters) *n_clusters = nc;
    return SDB_OK;
}

sdb_status sdb_get_optics(sdb_engine* e, int32_t* ordering, float* reach) {
    if (!e) return SDB_ERR_ARG;
    if (!e->haveOptics) return e->fail(SDB_ERR_STATE, "no sOPTICS result: call sdb_fit_soptics first");
    if (ordering) std::memcpy(ordering, e->hostOrdering.data(), sizeof(int32_t) * e->hostOrdering.size());
    if (reach) std::memcpy(reach, e->hostReach.data(), sizeof(float) * e->hostReach.size());
    return SDB_OK;
}

sdb_status sdb_clear(sdb_engine* e) {
    if (!e) return SDB_ERR_ARG;
    e->haveLabels = e->haveOptics = e->haveFit = false;
    e->hostOrdering.clear();
    e->hostReach.clear();
    return SDB_OK;
}

static sdb_status download(sdb_engine* e, void* dst, const DevBuf& b, size_t bytes) {
    if (!e->haveFit) return e->fail(SDB_ERR_STATE, "no fit yet");
    if (!dst) return SDB_ERR_ARG;
    cudaSetDevice(e->device);
    cudaError_t c = cudaMemcpyAsync(dst, b.ptr, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    return c == cudaSuccess ? SDB_OK : e->cuda_fail(c, "download");
}

static sdb_status no_index(sdb_engine* e) {
    return e->fail(SDB_ERR_STATE, "the last fit was sngDbscan / sngOptics, which builds no index");
}
sdb_status sdb_get_topk(sdb_engine* e, int32_t* out) {
    if (!e) return SDB_ERR_ARG;
    if (e->lastSng) return no_index(e);
    return download(e, out, e->topK, sizeof(int32_t) * (size_t)e->n * 2 * e->prm.topK);
}
sdb_status sdb_get_topm(sdb_engine* e, int32_t* out) {
    if (!e) return SDB_ERR_ARG;
    if (e->lastSng) return no_index(e);
    return download(e, out, e->topM, sizeof(int32_t) * (size_t)e->prm.n_proj * 2 * e->prm.topM);
}
sdb_status sdb_get_core(sdb_engine* e, uint8_t* core, int32_t* degree) {
    if (!e) return SDB_ERR_ARG;
    sdb_status s = SDB_OK;
    if (core) s = download(e, core, e->core, e->n);
    if (s == SDB_OK && degree) s = download(e, degree, e->degree, sizeof(int32_t) * e->n);
    return s;
}
sdb_status sdb_get_core_dist(sdb_engine* e, float* out) {
    if (!e) return SDB_ERR_ARG;
    if (!e->lastOptics) return e->fail(SDB_ERR_STATE, "core distances exist after an OPTICS fit only");
    return download(e, out, e->coreDist, sizeof(float) * e->n);
}
sdb_status sdb_get_projections(sdb_engine* e, float* out) {
    if (!e) return SDB_ERR_ARG;
    if (e->lastSng) return no_index(e);
    return download(e, out, e->P, sizeof(float) * (size_t)e->n * e->prm.n_proj);
}
sdb_status sdb_get_counters(sdb_engine* e, int64_t* out, int32_t n_out) {
    if (!e || !out) return SDB_ERR_ARG;
    int64_t v[8] = {(int64_t)e->hostCounters[0], (int64_t)e->hostCounters[1], (int64_t)e->launchCount,
                    (int64_t)e->hostCounters[3], (int64_t)e->hostCounters[4], (int64_t)e->fallbacks,
                    (int64_t)e->sngColsLast, (int64_t)e->sngExtraLast};
    for (int i = 0; i < n_out && i < 8; ++i) out[i] = v[i];
    return SDB_OK;
}
sdb_status sdb_get_stage_ms(sdb_engine* e, float* ms, int32_t n_ms) {
    if (!e || !ms) return SDB_ERR_ARG;
    for (int i = 0; i < n_ms && i < 9; ++i) ms[i] = e->stageMs[i];
    return SDB_OK;
}
void* sdb_engine_stream(sdb_engine* e) { return e ? (void*)e->stream : nullptr; }
const char* sdb_last_error(sdb_engine* e) { return e ? e->err.c_str() : "null engine"; }

}  // extern "C"
