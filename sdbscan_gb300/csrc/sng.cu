// sngDbscan and sngOptics on the engine: fit_sngDbscan / test_sngDbscan
// (src/sDbscan.cpp:1131-1304) and fit_sngOptics (:1846-1880).
//
// Pipeline (engine stream): upload X -> transformData (k_colstats +
// k_transform_rows) -> the host's sample (columns, multiplicities, extra
// draws) uploaded -> k_sng_block, or with BF16 precision (Cosine sngDbscan)
// k_sng_tc + k_sng_recheck with the FP32 block as gated fallback
// (+ k_sng_extras) -> k_sng_degree ->
//   sngDbscan: union-find over the pass bits, border minima, labels;
//   sngOptics: second block pass into CSR lists, core distances, ordering.
//
// The sample.  sng_findCorePoints (:430-465) seeds each point's generator
// with random_seed when it is >= 0, so every point draws the same sequence
// d_0, d_1, ... of uniform_int_distribution(0, n - 1) over
// default_random_engine and keeps its first S = ceil(1.0 n samplingProb)
// draws that are not its own index.  A point that is not among d_0..d_{S-1}
// gets exactly those; a sampled point u, drawn c_u times there, continues
// with the first c_u values of d_S, d_S+1, ... that are not u.  The draws are
// made here with the same standard-library engine and distribution, so a
// seeded fit reproduces the reference's neighbourhoods.  samplingProb >= 1
// is the reference's exact DBSCAN (:466-479).  With random_seed < 0 the
// reference seeds each point from the clock; here one clock seed is drawn
// per fit and shared.
//
// sng_findCoreDist (:1490-1512) seeds every point from std::random_device and
// takes S = ceil(samplingProb n) (float product) draws, skipping its own
// index without replacing it; that sample cannot be reproduced, so the
// sngOptics fit draws the same shared sequence as sngDbscan (first S draws,
// own index skipped) and de-duplicates the lists as the reference does
// (:1537-1541).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "../../include/sdbscan_gb300.h"
#include "common.cuh"
#include "engine_internal.h"

namespace sdb {
int launch_i32_to_i64(const int32_t* in, int64_t* out, int n, cudaStream_t st);
int launch_core_dist(const CoreArgs& a, const int64_t* nbOff, const float* nbDist, cudaStream_t st);
}  // namespace sdb

using namespace sdb;

namespace {

struct SngSample {
    std::vector<int32_t> cols, mult;  // distinct drawn ids (ascending) and their draw counts
    std::vector<int2> extras;         // (sampled point u, its replacement draw)
    bool exact = false;
};

void sng_sample(int n, float prob, unsigned seed, bool optics, SngSample& s) {
    s = SngSample();
    if (!optics && !(prob < 1.0)) {  // exact DBSCAN: every other point is a candidate
        s.exact = true;
        s.cols.resize(n);
        for (int i = 0; i < n; ++i) s.cols[i] = i;
        return;
    }
    const double S = optics ? (double)std::ceil(prob * (float)n) : std::ceil(1.0 * n * prob);
    if (!(S >= 1.0)) return;
    std::default_random_engine gen(seed);
    std::uniform_int_distribution<> distrib(0, n - 1);
    std::vector<int32_t> cnt(n, 0);
    for (long long i = 0; i < (long long)S; ++i) ++cnt[distrib(gen)];
    for (int v = 0; v < n; ++v)
        if (cnt[v]) {
            s.cols.push_back(v);
            s.mult.push_back(cnt[v]);
        }
    if (optics) return;
    std::vector<int32_t> more;  // d_S, d_S+1, ... continued from the same generator
    for (size_t c = 0; c < s.cols.size(); ++c) {
        const int u = s.cols[c];
        int need = s.mult[c];
        for (size_t i = 0; need > 0; ++i) {
            while (more.size() <= i) more.push_back(distrib(gen));
            if (more[i] != u) {
                s.extras.push_back(make_int2(u, more[i]));
                --need;
            }
        }
    }
}

const char* dist_label(int d) {
    static const char* names[] = {"Cosine", "L1", "L2", "Chi2", "JS"};
    return d >= 0 && d <= 4 ? names[d] : "?";
}

}  // namespace

sdb_status sdb_engine::fit_sng(const float* X, bool xOnDevice, const float* epsList, int nEps, int minPts,
                               bool optics, int32_t* labelsOut, int32_t* nclOut) {
    if (!paramsSet && !sngParamsSet) return fail(SDB_ERR_STATE, "set_sngParams must be called before a fit");
    if (X == nullptr) return fail(SDB_ERR_ARG, "X is null");
    if (epsList == nullptr || nEps < 1 || (optics && nEps != 1)) return fail(SDB_ERR_ARG, "invalid eps list");
    if (optics && minPts < 2) return fail(SDB_ERR_ARG, "minPts must be >= 2 for sngOptics");
    const sdb_params& p = prm;
    if (p.distance < SDB_COSINE || p.distance > SDB_JS) return fail(SDB_ERR_ARG, "unknown distance");
    if (n < 2 && !optics && p.samplingProb < 1.0 && std::ceil(1.0 * n * p.samplingProb) >= 1.0)
        return fail(SDB_ERR_ARG, "sngDbscan with samplingProb < 1 needs n_points >= 2 (every draw of a single point "
                                 "is itself, which the reference's draw loop never gets past)");
    haveLabels = haveOptics = haveFit = false;
    ld = (d + 3) & ~3;
    seedUsed = p.random_seed >= 0 ? p.random_seed
                                  : (int)(unsigned)std::chrono::system_clock::now().time_since_epoch().count();
    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");

    // independent samples per block of points: the reference's law when its
    // points draw apart (random_seed < 0), or when asked for
    // (sngOptics: the reference draws every point's sample from its own
    // std::random_device, so blocks unless a shared sample is asked for)
    if (optics ? sngSampling != 1
               : p.samplingProb < 1.0 && (sngSampling == 2 || (sngSampling == 0 && p.random_seed < 0)))
        return fit_sng_blocks(X, xOnDevice, epsList, nEps, minPts, optics, labelsOut, nclOut);

    SngSample smp;
    sng_sample(n, p.samplingProb, (unsigned)seedUsed, optics, smp);
    const int nU = (int)smp.cols.size();
    const int nct = (nU + 63) / 64;
    const int nExtra = (int)smp.extras.size();
    sngColsLast = nU;
    sngExtraLast = nExtra;

    bool ok = true;
    if (!xOnDevice) ok &= ensure(Xin, sizeof(float) * (size_t)n * d);
    ok &= ensure(Xt, sizeof(float) * (size_t)n * ld) && ensure(scale, sizeof(float) * n) &&
          ensure(errFlags, sizeof(int32_t) * kErrSlots) && ensure(counters, sizeof(unsigned long long) * 8) &&
          ensure(sngCols, sizeof(int32_t) * std::max(nU, 1)) && ensure(sngMult, sizeof(int32_t) * std::max(nU, 1)) &&
          ensure(sngColOf, sizeof(int32_t) * n) && ensure(sngExtras, sizeof(int2) * std::max(nExtra, 1)) &&
          ensure(sngExtraPass, std::max(nExtra, 1)) && ensure(rowDeg, sizeof(int32_t) * n) &&
          ensure(colCnt, sizeof(int32_t) * std::max(nU, 1)) && ensure(degree, sizeof(int32_t) * n) &&
          ensure(core, n) && ensure(scanTmp, sizeof(int64_t) * scan_tmp_elems((size_t)n + 1));
    if (!optics)
        ok &= ensure(sngMask, sizeof(uint64_t) * std::max<size_t>(1, (size_t)nct * n)) &&
              ensure(parent, sizeof(int32_t) * n) && ensure(border, sizeof(int32_t) * n) &&
              ensure(rootFlag, sizeof(int64_t) * (n + 1)) && ensure(labels, sizeof(int32_t) * n) &&
              ensure(nClusters, sizeof(int32_t) * 4);
    else
        ok &= ensure(nbOff, sizeof(int64_t) * (n + 1)) && ensure(nbFill, sizeof(int32_t) * n) &&
              ensure(coreDist, sizeof(float) * n);
    if (!ok) return SDB_ERR_NOMEM;

    cudaStream_t st = stream;
    int launches = 0;
    auto L_ = [&](int r) {
        if (r < 0) ok = false;
        else launches += r;
    };
#define SDB_CK(call)                                        \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

    SDB_CK(cudaEventRecord(ev[0], st));
    const float* Xd = X;
    if (!xOnDevice) {
        Xd = static_cast<const float*>(Xin.ptr);
        SDB_CK(cudaMemcpyAsync(Xin.ptr, X, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
    }
    SDB_CK(cudaEventRecord(ev[1], st));
    SDB_CK(cudaMemsetAsync(errFlags.ptr, 0, sizeof(int32_t) * kErrSlots, st));
    SDB_CK(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8, st));
    unsigned long long* ctr = static_cast<unsigned long long*>(counters.ptr);
    ProjectArgs pa{};
    pa.X = Xd;
    pa.ldx = d;
    pa.Xt = f32(Xt);
    pa.ld = ld;
    pa.n = n;
    pa.d = d;
    pa.dist = p.distance;
    pa.scale = f32(scale);
    pa.err = i32(errFlags);
    L_(launch_transform(pa, st));
    SDB_CK(cudaEventRecord(ev[2], st));
    SDB_CK(cudaEventRecord(ev[3], st));
    if (nU) {
        SDB_CK(cudaMemcpyAsync(sngCols.ptr, smp.cols.data(), sizeof(int32_t) * nU, cudaMemcpyHostToDevice, st));
        if (!smp.mult.empty())
            SDB_CK(cudaMemcpyAsync(sngMult.ptr, smp.mult.data(), sizeof(int32_t) * nU, cudaMemcpyHostToDevice, st));
    }
    if (nExtra)
        SDB_CK(cudaMemcpyAsync(sngExtras.ptr, smp.extras.data(), sizeof(int2) * nExtra, cudaMemcpyHostToDevice, st));

    SngArgs sa{};
    sa.Xt = f32(Xt);
    sa.ld = ld;
    sa.d = d;
    sa.dist = p.distance;
    sa.n = n;
    sa.cols = i32(sngCols);
    sa.mult = (!optics && !smp.exact) ? i32(sngMult) : nullptr;
    sa.colOf = i32(sngColOf);
    sa.nU = nU;
    sa.nct = nct;
    sa.mask = optics ? nullptr : static_cast<uint64_t*>(sngMask.ptr);
    sa.rowDeg = i32(rowDeg);
    sa.colCnt = i32(colCnt);
    sa.pairs = ctr + 3;
    sa.extras = static_cast<const int2*>(sngExtras.ptr);
    sa.extraPass = static_cast<uint8_t*>(sngExtraPass.ptr);
    sa.nExtra = nExtra;
    sa.err = i32(errFlags) + 6;
    sa.stallSpins = dbgStallSpins;
    L_(launch_sng_col_of(sa, i32(sngColOf), st));
    // BF16 screening of the block (Cosine sngDbscan): BF16 copies of every
    // row and of the sampled rows, a queue for the pairs near eps
    const bool screen = !optics && p.precision == SDB_PREC_BF16 && p.distance == SDB_COSINE && nU > 0;
    const int ldb = (d + 63) / 64 * 64;
    int64_t qcap = 0;
    std::vector<uint64_t> heavy;  // per 64-column word: the columns drawn more than once
    if (screen) {
        qcap = std::min<int64_t>((int64_t)1 << 31, std::max<int64_t>((int64_t)1 << 22, (int64_t)n * nU / 16));
        if (dbgQueueCap > 0) qcap = dbgQueueCap;
        if (!ensure(Xb, sizeof(uint16_t) * (size_t)n * ldb) || !ensure(sngUb, sizeof(uint16_t) * (size_t)nU * ldb) ||
            !ensure(queue, sizeof(uint64_t) * (size_t)qcap) || !ensure(sngHeavy, sizeof(uint64_t) * nct))
            return SDB_ERR_NOMEM;
        L_(launch_to_bf16(f32(Xt), ld, n, Xb.ptr, ldb, st));
        L_(launch_sng_gather_bf16(sa, sngUb.ptr, ldb, st));
        if (sa.mult != nullptr) {
            heavy.assign(nct, 0ull);
            for (int c = 0; c < nU; ++c)
                if (smp.mult[c] > 1) heavy[c >> 6] |= 1ull << (c & 63);
            SDB_CK(cudaMemcpyAsync(sngHeavy.ptr, heavy.data(), sizeof(uint64_t) * nct, cudaMemcpyHostToDevice, st));
            sa.heavy = static_cast<const uint64_t*>(sngHeavy.ptr);
        }
    }
    if (!ok) return fail(SDB_ERR_CUDA, "sample setup launch failed");
    SDB_CK(cudaEventRecord(ev[4], st));

    for (int ei = 0; ei < nEps; ++ei) {
        sa.eps = epsList[ei];
        SDB_CK(cudaMemsetAsync(rowDeg.ptr, 0, sizeof(int32_t) * n, st));
        SDB_CK(cudaMemsetAsync(colCnt.ptr, 0, sizeof(int32_t) * std::max(nU, 1), st));
        bool plain = nct > 0;
        if (screen) {
            // the FP32 block runs after the screening only if its flag was
            // raised (queue overflow or a timed-out wait): one small readback
            SDB_CK(cudaMemsetAsync(ctr + 4, 0, sizeof(unsigned long long), st));
            L_(launch_sng_tc(sa, Xb.ptr, sngUb.ptr, ldb, static_cast<uint64_t*>(queue.ptr), qcap, ctr + 4,
                             i32(errFlags) + 7, st));
            if (!ok) return fail(SDB_ERR_CUDA, "tensor-core sample distance launch failed");
            SDB_CK(cudaMemcpyAsync(hostErr + 7, i32(errFlags) + 7, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            SDB_CK(cudaStreamSynchronize(st));
            plain = hostErr[7] != 0;
        }
        if (plain) L_(launch_sng_block(sa, st));
        L_(launch_sng_extras(sa, st));
        if (!ok) return fail(SDB_ERR_CUDA, "sample distance launch failed");
        if (ei == 0) SDB_CK(cudaEventRecord(ev[5], st));
        L_(launch_sng_degree(sa, smp.exact ? 1 : 0, optics ? 1 : 0, minPts, i32(degree),
                             static_cast<uint8_t*>(core.ptr), st));
        if (ei == 0) SDB_CK(cudaEventRecord(ev[6], st));
        if (!optics) {
            ClusterArgs ka{};
            ka.n = n;
            ka.core = static_cast<const uint8_t*>(core.ptr);
            ka.parent = i32(parent);
            ka.border = i32(border);
            ka.rootFlag = i64(rootFlag);
            ka.scanTmp = i64(scanTmp);
            ka.labels = i32(labels);
            ka.nClusters = i32(nClusters);
            L_(launch_uf_init(i32(parent), i32(border), n, st));
            L_(launch_sng_union(sa, ka.core, i32(parent), st));
            L_(launch_uf_compress(ka, st));
            L_(launch_sng_border(sa, ka.core, i32(parent), i32(border), st));
            L_(launch_cluster_labels(ka, st));
            if (!ok) return fail(SDB_ERR_CUDA, "cluster launch failed");
            if (labelsOut) {
                SDB_CK(cudaMemcpyAsync(labelsOut + (size_t)ei * n, labels.ptr, sizeof(int32_t) * n,
                                       cudaMemcpyDeviceToHost, st));
                SDB_CK(cudaMemcpyAsync(nclOut + ei, nClusters.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            }
        }
    }
    if (optics) {
        // distinct neighbour lists: offsets from the degrees, then the pairs again
        SDB_CK(cudaMemsetAsync(nbOff.ptr, 0, sizeof(int64_t) * (n + 1), st));
        L_(launch_i32_to_i64(i32(degree), i64(nbOff), n, st));
        L_(launch_scan_i64(i64(nbOff), i64(nbOff), (size_t)n + 1, i64(scanTmp), st));
        if (!ok) return fail(SDB_ERR_CUDA, "neighbour offsets launch failed");
        int64_t total = 0;
        SDB_CK(cudaMemcpyAsync(&total, i64(nbOff) + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SDB_CK(cudaStreamSynchronize(st));
        if (!ensure(nbIdx, sizeof(int32_t) * std::max<int64_t>(total, 1)) ||
            !ensure(nbDist, sizeof(float) * std::max<int64_t>(total, 1)))
            return SDB_ERR_NOMEM;
        SDB_CK(cudaMemsetAsync(nbFill.ptr, 0, sizeof(int32_t) * n, st));
        sa.nbOff = i64(nbOff);
        sa.nbFill = i32(nbFill);
        sa.nbIdx = i32(nbIdx);
        sa.nbDist = f32(nbDist);
        if (nct) L_(launch_sng_emit(sa, st));
        CoreArgs ca{};
        ca.n = n;
        ca.minPts = minPts;
        ca.core = static_cast<uint8_t*>(core.ptr);
        ca.coreDist = f32(coreDist);
        L_(launch_core_dist(ca, i64(nbOff), f32(nbDist), st));
        if (!ok) return fail(SDB_ERR_CUDA, "neighbour list launch failed");
        SDB_CK(cudaMemcpyAsync(hostErr, errFlags.ptr, sizeof(int32_t) * kErrSlots, cudaMemcpyDeviceToHost, st));
        SDB_CK(cudaStreamSynchronize(st));
        if (hostErr[6]) return fail(SDB_ERR_INTERNAL, "sngOptics neighbour list overflow");
        sdb_status s = optics_order(total);
        if (s != SDB_OK) return s;
    }
    SDB_CK(cudaEventRecord(ev[7], st));
    SDB_CK(cudaMemcpyAsync(hostErr, errFlags.ptr, sizeof(int32_t) * kErrSlots, cudaMemcpyDeviceToHost, st));
    SDB_CK(cudaMemcpyAsync(hostCounters, counters.ptr, sizeof(unsigned long long) * 8, cudaMemcpyDeviceToHost, st));
    SDB_CK(cudaEventRecord(ev[8], st));
    SDB_CK(cudaStreamSynchronize(st));
#undef SDB_CK
    launchCount = launches;
    for (int i = 0; i < 8; ++i) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        stageMs[i] = ms;
    }
    cudaEventElapsedTime(&stageMs[8], ev[0], ev[8]);
    sdb_status s = check_flags();
    if (s != SDB_OK) return s;
    if (hostErr[6]) return fail(SDB_ERR_INTERNAL, "sngOptics neighbour list overflow");
    haveFit = true;
    lastOptics = optics;
    lastSng = true;
    if (optics) haveOptics = true;
    else haveLabels = true;
    if (p.verbose) {
        std::printf("sdbscan_gb300 %s fit: n=%d d=%d dist=%s samplingProb=%g sampled=%d extra=%d eps=%g minPts=%d%s\n",
                    optics ? "sngOPTICS" : "sngDBSCAN", n, d, dist_label(p.distance), p.samplingProb, nU, nExtra,
                    epsList[0], minPts, screen ? " (BF16 screening)" : "");
        const char* names[9] = {"upload", "transform", "-", "sample", "distances", "core", "cluster/optics",
                                "readback", "total"};
        for (int i = 0; i < 9; ++i) std::printf("  %-14s %9.3f ms\n", names[i], stageMs[i]);
    }
    err.clear();
    return SDB_OK;
}

// sngDbscan with independent samples per block of sng_block_rows() points
// (k_sng_blocks.cu): transform, then per eps the pass words, degrees and core
// flags, the union-find over the core-core passes, border minima and labels.
sdb_status sdb_engine::fit_sng_blocks(const float* X, bool xOnDevice, const float* epsList, int nEps, int minPts,
                                      bool optics, int32_t* labelsOut, int32_t* nclOut) {
    const sdb_params& p = prm;
    const int BR = sng_block_rows();
    // draws per point: ceil(1.0 n prob) in double (src/sDbscan.cpp:432), for
    // sngOptics ceil(prob n) in float (:1490)
    const int64_t S = optics ? (int64_t)std::ceil(p.samplingProb * (float)n)
                             : (int64_t)std::ceil(1.0 * n * p.samplingProb);
    const int64_t nb = (n + BR - 1) / BR;
    sngColsLast = 0;
    sngExtraLast = 0;
    bool ok = true;
    if (!xOnDevice) ok &= ensure(Xin, sizeof(float) * (size_t)n * d);
    ok &= ensure(Xt, sizeof(float) * (size_t)n * ld) && ensure(scale, sizeof(float) * n) &&
          ensure(errFlags, sizeof(int32_t) * kErrSlots) && ensure(counters, sizeof(unsigned long long) * 8) &&
          ensure(degree, sizeof(int32_t) * n) && ensure(core, n) && ensure(parent, sizeof(int32_t) * n) &&
          ensure(border, sizeof(int32_t) * n) && ensure(rootFlag, sizeof(int64_t) * (n + 1)) &&
          ensure(labels, sizeof(int32_t) * n) && ensure(nClusters, sizeof(int32_t) * 4) &&
          ensure(scanTmp, sizeof(int64_t) * scan_tmp_elems((size_t)n + 1)) &&
          ensure(sngWords, sizeof(uint32_t) * std::max<size_t>(1, (size_t)nb * (size_t)std::max<int64_t>(S, 0)));
    if (optics)
        ok &= ensure(nbOff, sizeof(int64_t) * (n + 1)) && ensure(coreDist, sizeof(float) * n) &&
              ensure(hashOffB, sizeof(int64_t) * (n + 1));
    if (!ok) return SDB_ERR_NOMEM;
    cudaStream_t st = stream;
    int launches = 0;
    auto L_ = [&](int r) {
        if (r < 0) ok = false;
        else launches += r;
    };
#define SDB_CK(call)                                        \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)
    SDB_CK(cudaEventRecord(ev[0], st));
    const float* Xd = X;
    if (!xOnDevice) {
        Xd = static_cast<const float*>(Xin.ptr);
        SDB_CK(cudaMemcpyAsync(Xin.ptr, X, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, st));
    }
    SDB_CK(cudaEventRecord(ev[1], st));
    SDB_CK(cudaMemsetAsync(errFlags.ptr, 0, sizeof(int32_t) * kErrSlots, st));
    SDB_CK(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8, st));
    unsigned long long* ctr = static_cast<unsigned long long*>(counters.ptr);
    ProjectArgs pa{};
    pa.X = Xd;
    pa.ldx = d;
    pa.Xt = f32(Xt);
    pa.ld = ld;
    pa.n = n;
    pa.d = d;
    pa.dist = p.distance;
    pa.scale = f32(scale);
    pa.err = i32(errFlags);
    L_(launch_transform(pa, st));
    SDB_CK(cudaEventRecord(ev[2], st));
    SDB_CK(cudaEventRecord(ev[3], st));
    SDB_CK(cudaEventRecord(ev[4], st));
    // splitmix64 of the seed, the key of every block's draws
    uint64_t key = (uint64_t)(uint32_t)seedUsed + 0x9E3779B97F4A7C15ull;
    key = (key ^ (key >> 30)) * 0xBF58476D1CE4E5B9ull;
    key = (key ^ (key >> 27)) * 0x94D049BB133111EBull;
    key ^= key >> 31;
    SngBlockArgs ba{};
    ba.Xt = f32(Xt);
    ba.ld = ld;
    ba.d = d;
    ba.dist = p.distance;
    ba.n = n;
    ba.S = std::max<int64_t>(S, 0);
    ba.key = key;
    ba.words = static_cast<uint32_t*>(sngWords.ptr);
    ba.degree = i32(degree);
    ba.pairs = ctr + 3;
    ba.err = i32(errFlags) + 6;
    if (optics) {
        // passes with repeats -> table sizes -> the emitting pass into the
        // tables -> distinct lists, core flags and core distances -> ordering
        ba.eps = epsList[0];
        SDB_CK(cudaMemsetAsync(degree.ptr, 0, sizeof(int32_t) * n, st));
        L_(launch_sngb_pass(ba, minPts, static_cast<uint8_t*>(core.ptr), st));
        L_(launch_sngb_caps(ba, i64(hashOffB), st));
        L_(launch_scan_i64(i64(hashOffB), i64(hashOffB), (size_t)n + 1, i64(scanTmp), st));
        if (!ok) return fail(SDB_ERR_CUDA, "sampled-block launch failed");
        int64_t slots = 0;
        SDB_CK(cudaMemcpyAsync(&slots, i64(hashOffB) + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SDB_CK(cudaStreamSynchronize(st));
        if (!ensure(hashIdB, sizeof(int32_t) * std::max<int64_t>(slots, 1)) ||
            !ensure(hashDistB, sizeof(float) * std::max<int64_t>(slots, 1)))
            return SDB_ERR_NOMEM;
        SDB_CK(cudaMemsetAsync(hashIdB.ptr, 0xFF, sizeof(int32_t) * std::max<int64_t>(slots, 1), st));
        ba.hashOff = i64(hashOffB);
        ba.hashId = i32(hashIdB);
        ba.hashDist = f32(hashDistB);
        L_(launch_sngb_emit(ba, st));
        SDB_CK(cudaEventRecord(ev[5], st));
        L_(launch_sngb_distinct(ba, minPts, i32(degree), static_cast<uint8_t*>(core.ptr), st));
        SDB_CK(cudaMemsetAsync(nbOff.ptr, 0, sizeof(int64_t) * (n + 1), st));
        L_(launch_i32_to_i64(i32(degree), i64(nbOff), n, st));
        L_(launch_scan_i64(i64(nbOff), i64(nbOff), (size_t)n + 1, i64(scanTmp), st));
        if (!ok) return fail(SDB_ERR_CUDA, "sampled-block launch failed");
        int64_t total = 0;
        SDB_CK(cudaMemcpyAsync(&total, i64(nbOff) + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SDB_CK(cudaStreamSynchronize(st));
        if (!ensure(nbIdx, sizeof(int32_t) * std::max<int64_t>(total, 1)) ||
            !ensure(nbDist, sizeof(float) * std::max<int64_t>(total, 1)))
            return SDB_ERR_NOMEM;
        L_(launch_sngb_compact(ba, i64(nbOff), i32(nbIdx), f32(nbDist), st));
        CoreArgs ca{};
        ca.n = n;
        ca.minPts = minPts;
        ca.core = static_cast<uint8_t*>(core.ptr);
        ca.coreDist = f32(coreDist);
        L_(launch_core_dist(ca, i64(nbOff), f32(nbDist), st));
        SDB_CK(cudaEventRecord(ev[6], st));
        if (!ok) return fail(SDB_ERR_CUDA, "sampled-block launch failed");
        SDB_CK(cudaMemcpyAsync(hostErr, errFlags.ptr, sizeof(int32_t) * kErrSlots, cudaMemcpyDeviceToHost, st));
        SDB_CK(cudaStreamSynchronize(st));
        if (hostErr[6]) return fail(SDB_ERR_INTERNAL, "sngOptics neighbour table overflow");
        sdb_status so = optics_order(total);
        if (so != SDB_OK) return so;
    }
    for (int ei = 0; ei < nEps && !optics; ++ei) {
        ba.eps = epsList[ei];
        SDB_CK(cudaMemsetAsync(degree.ptr, 0, sizeof(int32_t) * n, st));
        L_(launch_sngb_pass(ba, minPts, static_cast<uint8_t*>(core.ptr), st));
        if (ei == 0) SDB_CK(cudaEventRecord(ev[5], st));
        if (ei == 0) SDB_CK(cudaEventRecord(ev[6], st));
        ClusterArgs ka{};
        ka.n = n;
        ka.core = static_cast<const uint8_t*>(core.ptr);
        ka.parent = i32(parent);
        ka.border = i32(border);
        ka.rootFlag = i64(rootFlag);
        ka.scanTmp = i64(scanTmp);
        ka.labels = i32(labels);
        ka.nClusters = i32(nClusters);
        L_(launch_uf_init(i32(parent), i32(border), n, st));
        if (ba.S > 0) L_(launch_sngb_union(ba, ka.core, i32(parent), st));
        L_(launch_uf_compress(ka, st));
        if (ba.S > 0) L_(launch_sngb_border(ba, ka.core, i32(parent), i32(border), st));
        L_(launch_cluster_labels(ka, st));
        if (!ok) return fail(SDB_ERR_CUDA, "sampled-block launch failed");
        if (labelsOut) {
            SDB_CK(cudaMemcpyAsync(labelsOut + (size_t)ei * n, labels.ptr, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                   st));
            SDB_CK(cudaMemcpyAsync(nclOut + ei, nClusters.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        }
    }
    SDB_CK(cudaEventRecord(ev[7], st));
    SDB_CK(cudaMemcpyAsync(hostErr, errFlags.ptr, sizeof(int32_t) * kErrSlots, cudaMemcpyDeviceToHost, st));
    SDB_CK(cudaMemcpyAsync(hostCounters, counters.ptr, sizeof(unsigned long long) * 8, cudaMemcpyDeviceToHost, st));
    SDB_CK(cudaEventRecord(ev[8], st));
    SDB_CK(cudaStreamSynchronize(st));
#undef SDB_CK
    launchCount = launches;
    for (int i = 0; i < 8; ++i) cudaEventElapsedTime(&stageMs[i], ev[i], ev[i + 1]);
    cudaEventElapsedTime(&stageMs[8], ev[0], ev[8]);
    sdb_status s = check_flags();
    if (s != SDB_OK) return s;
    haveFit = true;
    if (optics) haveOptics = true;
    else haveLabels = true;
    lastOptics = optics;
    lastSng = true;
    if (p.verbose) {
        std::printf("sdbscan_gb300 %s fit (independent samples per %d-point block): n=%d d=%d dist=%s "
                    "samplingProb=%g draws=%lld eps=%g minPts=%d\n",
                    optics ? "sngOPTICS" : "sngDBSCAN", BR, n, d, dist_label(p.distance), p.samplingProb,
                    (long long)ba.S, epsList[0], minPts);
        const char* names[9] = {"upload", "transform", "-", "-", "distances", "-", "cluster", "readback", "total"};
        for (int i = 0; i < 9; ++i) std::printf("  %-14s %9.3f ms\n", names[i], stageMs[i]);
    }
    err.clear();
    return SDB_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

sdb_status sdb_set_sng_sampling(sdb_engine* e, int32_t mode) {
    if (!e) return SDB_ERR_ARG;
    if (mode < 0 || mode > 2) return e->fail(SDB_ERR_ARG, "sng sampling must be 0 (by seed), 1 (shared) or 2 (blocks)");
    e->sngSampling = mode;
    return SDB_OK;
}

sdb_status sdb_set_sng_params(sdb_engine* e, int32_t distance, float samplingProb, int32_t clusterNoise,
                              int32_t verbose, int32_t n_threads, int32_t random_seed) {
    if (!e) return SDB_ERR_ARG;
    if (distance < SDB_COSINE || distance > SDB_JS) return e->fail(SDB_ERR_ARG, "unknown distance");
    e->prm.distance = distance;
    e->prm.samplingProb = samplingProb;
    if (clusterNoise > 0) e->prm.clusterNoise = 2;  // src/sDbscan.h:133-134
    e->prm.verbose = verbose;
    e->prm.n_threads = n_threads;
    e->prm.random_seed = random_seed;
    e->sngParamsSet = true;
    return SDB_OK;
}

sdb_status sdb_fit_sngdbscan(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    if (!e) return SDB_ERR_ARG;
    e->prm.clusterNoise = 0;  // fit_sngDbscan switches noise labelling off (src/sDbscan.cpp:1157)
    return e->fit_sng(X, false, &eps, 1, minPts, false);
}
sdb_status sdb_fit_sngdbscan_device(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    if (!e) return SDB_ERR_ARG;
    e->prm.clusterNoise = 0;
    return e->fit_sng(X, true, &eps, 1, minPts, false);
}
sdb_status sdb_fit_sngdbscan_sweep(sdb_engine* e, const float* X, const float* eps, int32_t n_eps, int32_t minPts,
                                   int32_t* labels, int32_t* n_clusters) {
    if (!e) return SDB_ERR_ARG;
    if (!eps || n_eps < 1 || !labels || !n_clusters) return e->fail(SDB_ERR_ARG, "eps list and outputs are required");
    return e->fit_sng(X, false, eps, n_eps, minPts, false, labels, n_clusters);
}
sdb_status sdb_fit_sngoptics(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit_sng(X, false, &eps, 1, minPts, true) : SDB_ERR_ARG;
}
sdb_status sdb_fit_sngoptics_device(sdb_engine* e, const float* X, float eps, int32_t minPts) {
    return e ? e->fit_sng(X, true, &eps, 1, minPts, true) : SDB_ERR_ARG;
}

}  // extern "C"
