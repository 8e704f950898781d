// Shared device helpers and the internal launcher interface between the
// kernel translation units and the engine (engine.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#define SDB_DEV __device__ __forceinline__

namespace sdb {

constexpr int kWarp = 32;
constexpr float kNegInfReach = -2147483648.0f;  // NEG_INF of src/Header.h:20

// Order-preserving map float -> uint32 (larger float -> larger key).  -0 is
// folded onto +0 first so that keys are equal exactly when the floats compare
// equal (the reference's heaps compare floats).
SDB_DEV uint32_t key_of(float v) {
    uint32_t u = __float_as_uint(v + 0.0f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
SDB_DEV float float_of_key(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

SDB_DEV unsigned lane_id() { return threadIdx.x & 31u; }

template <typename T> SDB_DEV T shfl_xor(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

SDB_DEV uint64_t shfl_xor_u64(uint64_t v, int m) {
    uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    lo = __shfl_xor_sync(0xffffffffu, lo, m);
    hi = __shfl_xor_sync(0xffffffffu, hi, m);
    return ((uint64_t)hi << 32) | lo;
}
SDB_DEV uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        uint64_t o = shfl_xor_u64(v, m);
        v = o > v ? o : v;
    }
    return v;
}
SDB_DEV int warp_sum(int v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

// Calls f(i) on the warp's lanes for every candidate i of point p that passed
// eps (bit set in p's mask words).  The 2k top-k ids and mask words are
// fetched up front, two slots per lane; candidates come in lane-parallel
// batches of up to 32.
template <typename F>
SDB_DEV void for_each_passing(const int32_t* __restrict__ topK, const int32_t* __restrict__ topM,
                              const uint64_t* __restrict__ masks, int k, int m, int W, int p, F&& f) {
    const unsigned l = lane_id();
    const int slots = 2 * k;
    const unsigned long long* mk64 = reinterpret_cast<const unsigned long long*>(masks);
    int rA = 0, rB = 0;
    uint64_t mA = 0, mB = 0;
    if ((int)l < slots) {
        rA = __ldg(topK + (size_t)p * slots + l);
        mA = __ldg(mk64 + ((size_t)p * slots + l) * W);
    }
    if ((int)l + 32 < slots) {
        rB = __ldg(topK + (size_t)p * slots + l + 32);
        mB = __ldg(mk64 + ((size_t)p * slots + l + 32) * W);
    }
    for (int jj = 0; jj < slots; ++jj) {
        const int src = jj & 31;
        const int r = __shfl_sync(0xffffffffu, jj < 32 ? rA : rB, src);
        const int side = jj >= k;
        const int32_t* lst = topM + (size_t)r * 2 * m + side * m;
        for (int wd = 0; wd < W; ++wd) {
            uint64_t mk;
            if (wd == 0) {
                const uint64_t mine = jj < 32 ? mA : mB;
                const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)mine, src);
                const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(mine >> 32), src);
                mk = ((uint64_t)hi << 32) | lo;
            } else {
                mk = __ldg(mk64 + ((size_t)p * slots + jj) * W + wd);
            }
            if (!mk) continue;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int bit = half * 32 + (int)l;
                if ((mk >> bit) & 1ull) f(__ldg(lst + wd * 64 + bit));
            }
        }
    }
}

// Distance codes (sdb_distance in include/sdbscan_gb300.h).
enum { DIST_COSINE = 0, DIST_L1 = 1, DIST_L2 = 2, DIST_CHI2 = 3, DIST_JS = 4 };

}  // namespace sdb

// -------------------------------------------------------------------------
// Launchers (host functions) implemented by the kernel translation units.
// All run on `st`; none synchronizes.  Each returns the number of kernel
// launches it made (for the launch counter) or a negative value on a launch
// error.
// -------------------------------------------------------------------------
namespace sdb {

// Streaming multiprocessors of the current device, queried once per device;
// grid sizes are multiples of it.
inline int sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1;
    }
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
            cudaGetLastError();
            v = 1;
        }
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

struct ProjectArgs {
    const float* X;      // input rows (n x d, row stride ldx)
    int ldx;
    float* Xt;           // transformed rows out (n x ld), may alias nothing
    int ld;              // padded row stride of Xt (multiple of 4)
    int n, d, dist;
    int ker;             // embedding width (== d for Cosine)
    float kerSam;        // Chi2/JS interval sampling
    const float* E;      // precomputed embedding rows (L1/L2), n x ker, or null
    const uint32_t* signs;  // 3 x fhtDim/32 words of sign bits (bit = 1 -> +1)
    int fhtDim, nproj, k;
    float* P;            // n x nproj projections out
    int32_t* topK;       // n x 2k out
    float* chunkMax;     // G x nproj
    float* chunkMin;     // G x nproj
    int chunk;           // points per chunk (G = ceil(n / chunk))
    int chunkBase, chunkEnd;  // chunks this launch covers (chunkEnd 0: all G)
    int32_t* err;        // device flags: [0] negative input, [1] zero point
    unsigned long long* ties;  // top-k boundary tie counter
    int do_transform;    // 1: apply transformData; 0: X already transformed
    float* scale;        // n: per-point norm / sum (scratch)
    const double* compCosh;  // Chi2/JS: cosh(PI * c * L) for c = 1..components (host-computed)
    double ln4;              // JS: log(4.0) as the host computes it
    uint16_t* Xb;            // Cosine, fhtDim <= 2048: BF16 copy of Xt (n x ldb, zero padded), or null
    int ldb;                 // its row stride, <= fhtDim
};
int launch_project(const ProjectArgs& a, cudaStream_t st);
// Blocks in one full wave of k_project (six blocks per SM; each walks its
// launch's chunks grid-stride).
inline int project_wave_chunks() { return sm_count() * 6; }
// transformData alone into Xt (uses X, ldx, Xt, ld, n, d, dist, scale, err).
int launch_transform(const ProjectArgs& a, cudaStream_t st);

// Random Fourier features for L1/L2: E[p] = [cos(R x_p), sin(R x_p)].
// gate (optional): run only if *gate != 0 (the tensor-core embedding failed).
int launch_rff(const float* Xt, int ld, int n, int d, const float* R, int h, float* E, cudaStream_t st,
               const int32_t* gate = nullptr);
// BF16 mode: the same embedding on the tensor cores from split-BF16 copies
// ([hi | lo] per row) of the points (n x 2 ldb) and of R (h x 2 ldb); err set
// on a timed-out wait.
// stallSpins > 0: the stall test (sdb_set_debug_limits).
int launch_rff_tc(const void* Xb, const void* Rb, int n, int h, int ldb, float* E, int32_t* err, long long stallSpins,
                  cudaStream_t st);

struct TopMArgs {
    const float* P;
    int n, nproj, m;
    const float* chunkMax;
    const float* chunkMin;
    int G;
    float* thrMax;       // nproj
    float* thrMin;       // nproj
    uint64_t* cand;      // 2*nproj lists x cap entries of (key<<32 | ~index)
    int32_t* candCount;  // 2*nproj
    int cap;
    int32_t* topM;       // nproj x 2m out
    int32_t* overflow;   // list ids that overflowed (2*nproj), count in overflow_n
    int32_t* overflow_n;
    unsigned long long* ties;
    int32_t* errFlag;    // set when an internal invariant fails
};
int launch_topm_thresholds(const TopMArgs& a, cudaStream_t st);
int launch_topm_collect(const TopMArgs& a, cudaStream_t st);
int launch_topm_select(const TopMArgs& a, cudaStream_t st);

// Exclusive scan of n int64 values (in place allowed); tmp needs
// scan_tmp_elems(n) entries.
size_t scan_tmp_elems(size_t n);
int launch_scan_i64(const int64_t* in, int64_t* out, size_t n, int64_t* tmp, cudaStream_t st);

struct IndexArgs {
    const int32_t* topK;  // n x 2k
    int n, k, nproj, m;
    const int32_t* topM;  // nproj x 2m
    int64_t* listCount;   // 2*nproj + 1
    int64_t* listOff;     // 2*nproj + 1
    int2* members;        // n*2k (point, slot)
    int TM;               // member rows per distance tile
    int nct;              // candidate tiles per list
    int64_t* tileOff;     // 2*nproj + 1 (tiles per list, scanned)
    int32_t* tileList;    // total tiles
    int32_t* hubCount;    // n: number of top-m lists containing the point
    int64_t* hubOff;      // n + 1
    int32_t* hubLists;    // 2*nproj*m: list ids per hub point
    int64_t* scanTmp;
    // members in point-chunk order and tiles in chunk order (L2 locality of
    // the gathered rows: the tiles in flight cover a narrow range of points)
    int chunkPts, nChunks;  // points per chunk; chunks
    int32_t* chunkOff;      // 2*nproj x nChunks: members of the list from each chunk, scanned per list
    int32_t* tileKey;       // total tiles: chunk of the tile's first member
    int64_t* keyOff;        // nChunks + 1 (counts, then scanned, then used as cursors)
    int32_t* tilePerm;      // total tiles: tiles in chunk order
    int64_t maxTiles;       // grid bound of the tile kernels
};
// Members of every list ordered by point chunk (CTA per chunk).
int launch_index_count(const IndexArgs& a, cudaStream_t st);
int launch_index_scatter(const IndexArgs& a, cudaStream_t st);
// tilePerm: the tiles sorted by the chunk of their first member.
int launch_tile_order(const IndexArgs& a, cudaStream_t st);
// tilePerm for the tensor-core distance kernel: tiles by (super-chunk of
// superChunk point chunks, list); keys: total tiles, keyOff:
// tile_order_list_keys() entries (scanTmp must cover that many).
size_t tile_order_list_keys(const IndexArgs& a, int superChunk);
int launch_tile_order_list(const IndexArgs& a, int superChunk, int32_t* keys, int64_t* keyOff, int32_t* perm,
                           cudaStream_t st);
// Tile id of the b-th launched tile (identity without a permutation).
__device__ __forceinline__ int64_t tile_at(const int32_t* perm, int64_t b) { return perm != nullptr ? perm[b] : b; }
int launch_tiles(const IndexArgs& a, int64_t total_tiles, cudaStream_t st);
int launch_hubs_count(const IndexArgs& a, cudaStream_t st);
int launch_hubs_scatter(const IndexArgs& a, cudaStream_t st);

struct DistArgs {
    const float* Xt;
    int ld, d, dist, n;
    const int2* members;
    const int64_t* listOff;
    const int32_t* tileList;
    const int64_t* tileOff;
    int64_t nTiles;       // launch grid (an upper bound)
    const int64_t* tileTotal;  // device: actual number of tiles
    const int32_t* tilePerm;   // optional: launch order of the tiles (tile_at)
    const int32_t* topM;
    int nproj, m, k, W;   // W = 64-bit mask words per (point, slot)
    int nct;              // candidate tiles per list
    float eps;
    float epsLo;          // eps sweeps: k_masks_from_dists keeps epsLo < d <= eps
    const uint8_t* pairRound;  // eps sweeps (optional): per pair, the first round whose eps >= d (rows of W x 64 bytes)
    int round;
    int variant;               // plain distance tiles: 0 by m, 1: 128 x 64 (256 threads), 2-3: 128 x 50 (160 threads; k_dist.cu)
    uint64_t* masks;      // n x 2k x W
    int32_t* inRaw;       // n
    float* dists;         // n x 2k x m (optional)
    unsigned long long* pairs;  // pass counter
    const int32_t* topKmat;     // n x 2k (the re-decision kernel maps slots back to lists)
    const int32_t* gate;        // optional: k_dist runs only if *gate != 0 (screening failed)
    int32_t* waitErr;           // set by the persistent plain kernel when a bounded wait ran out
    long long stallSpins;       // > 0: the stall test (sdb_set_debug_limits)
    int nSweep;                 // BF16 sweep: eps values whose margins are re-decided exactly
    float sweepEps[16];
    const float* sqNorm;        // L2 BF16 screening: per point, the squared norm of its row of Xt
};
constexpr int kMaxScreenedSweep = 16;
int launch_dist(const DistArgs& a, cudaStream_t st);
// The persistent warp-specialised plain kernel (k_dist_ws.cu): variant 4 or 5.
int launch_dist_ws(const DistArgs& a, int variant, cudaStream_t st);
int launch_masks_from_dists(const DistArgs& a, cudaStream_t st);
// Eps sweeps: each pair's round (index of the first of the nSweep ascending
// sweepEps values >= its distance; nSweep when none; 255 for the point's own
// entry and padding), n x 2k rows of W x 64 bytes.
int launch_pair_rounds(const DistArgs& a, uint8_t* rounds, cudaStream_t st);
int launch_to_bf16(const float* Xt, int ld, int n, void* Xb, int ldb, cudaStream_t st);
int launch_to_bf16_split(const float* Xt, int ld, int n, void* Xs, int ldb, cudaStream_t st);
int launch_screen_reset(const DistArgs& a, cudaStream_t st);
// BF16 screening: Cb (dist_tc_cand_bytes) receives the lists' candidate rows.
// Cosine: Xb holds the BF16 rows (stride ldb); L2: the split [hi | lo] rows
// (stride 2 ldb, launch_to_bf16_split) and a.sqNorm the squared row norms.
size_t dist_tc_cand_bytes(const DistArgs& a, int ldb);
// Squared norms of the rows of Xt (n x ld), any summation order (screening only).
int launch_sq_norms(const float* Xt, int ld, int n, float* out, cudaStream_t st);
int launch_dist_tc(const DistArgs& a, const void* Xb, int ldb, void* Cb, uint64_t* queue, int64_t qcap,
                   unsigned long long* qcount, int32_t* err, cudaStream_t st);
int launch_recheck(const DistArgs& a, const uint64_t* queue, const unsigned long long* qcount, int64_t qcap,
                   cudaStream_t st);

struct CoreArgs {
    int n, k, m, W, nproj, minPts;
    const uint64_t* masks;
    const int32_t* topK;
    const int32_t* topM;
    const int32_t* hubCount;
    const int64_t* hubOff;
    const int32_t* hubLists;
    int32_t* inRaw;
    int32_t* aCount;
    int32_t* degree;
    uint8_t* core;
    const float* dists;   // sOPTICS: n x 2k x m distances, or null
    float* coreDist;      // sOPTICS: n (0 for non-core), or null
    const int32_t* hubIdx;   // n: dense index of hub points, -1 for others
    const uint32_t* kMask;   // hubs x ceil(2D/32): bit l set when the hub meets list l (its top-k)
    uint64_t* firstMasks;    // n x 2k x W: the mask bits of each point's first occurrence of a candidate
    // eps sweeps, processed in ascending eps: the masks hold only the pairs new
    // at this eps (previous eps < d <= eps); degrees accumulate, core flags only
    // grow, firstMasks accumulate and newMasks receive this round's bits
    int accumulate, round;
    uint64_t* newMasks;      // n x 2k x W (accumulate only)
    int32_t* coreEps;        // n: round at which the point became core, -1 before (accumulate only)
    const uint64_t* multi;   // 2D x W: slots whose point another list holds too (launch_slot_sigs)
};
// Per-slot signatures (sig, 2D x m int4) and the multi-list slot bits (multi, 2D x W).
int launch_slot_sigs(const int32_t* topM, int D, int m, const int64_t* hubOff, const int32_t* hubLists, void* sig,
                     uint64_t* multi, int W, cudaStream_t st);
int launch_core_dedupe(const CoreArgs& a, const void* sig, cudaStream_t st);
// hubIdx from hubOff (a scan of hub flags into idxTmp) and the hubs' list masks.
int launch_hub_masks(const CoreArgs& a, int32_t* hubIdx, int64_t* idxTmp, uint32_t* kMask, int64_t* scanTmp,
                     int64_t* nHubsDev, cudaStream_t st);
int launch_core_finish(const CoreArgs& a, cudaStream_t st);

struct ClusterArgs {
    int n, k, m, W;
    const uint64_t* masks;   // first-occurrence masks: each distinct candidate once per point
    const int32_t* topK;
    const int32_t* topM;
    // the distance stage's tiles (list l, 128 member rows, 64 candidate columns)
    const int2* members;
    const int64_t* listOff;
    const int32_t* tileList;
    const int64_t* tileOff;
    const int64_t* tileTotal;  // device: actual number of tiles
    const int32_t* tilePerm;   // optional: launch order of the tiles (tile_at)
    int64_t nTiles;            // launch grid (an upper bound)
    int TM, nct, nproj;
    // eps sweeps: the union-find carries over from the previous (smaller) eps,
    // and only rows with a new edge or a newly core endpoint are united
    int carry, round;
    const uint64_t* newMasks;  // this round's first-occurrence bits
    const int32_t* coreEps;    // round at which each point became core
    const uint8_t* core;
    int32_t* parent;
    int32_t* border;
    int64_t* rootFlag;    // n + 1, scanned into cluster ids
    int64_t* scanTmp;
    int32_t* labels;
    int32_t* nClusters;   // device scalar
};
int launch_cluster(const ClusterArgs& a, cudaStream_t st);
// Pieces of launch_cluster for callers with their own edge kernels: parent[p]
// = p and border[p] = INT_MAX; parents of core points set to their roots;
// cluster ids and labels from core, parent and border (uses n, core, parent,
// border, rootFlag, scanTmp, labels, nClusters).
int launch_uf_init(int32_t* parent, int32_t* border, int n, cudaStream_t st);
int launch_uf_compress(const ClusterArgs& a, cudaStream_t st);
int launch_cluster_labels(const ClusterArgs& a, cudaStream_t st);

// sngDbscan / sngOptics (src/sDbscan.cpp:416-504, :1484-1583) over one
// shared sample of columns: every point is a row, every distinct sampled
// point a column.
struct SngArgs {
    const float* Xt;
    int ld, d, dist, n;
    const int32_t* cols;   // nU distinct sampled point ids, ascending
    const int32_t* mult;   // nU: times each was drawn (null: weight 1)
    const int32_t* colOf;  // n: the point's column, -1 when not sampled
    int nU, nct;           // columns; 64-column tiles
    float eps;
    uint64_t* mask;        // nct x n pass bits (tile-major: word ct * n + p), or null
    int32_t* rowDeg;       // n: weighted passes of the point's row (atomic adds)
    int32_t* colCnt;       // nU: passes of each column over all rows
    unsigned long long* pairs;  // pass counter
    // extra draws of the sampled points (sngDbscan): (point, drawn point) pairs
    const int2* extras;
    uint8_t* extraPass;
    int nExtra;
    // sngOptics neighbour lists (CSR filled by the second block pass)
    const int64_t* nbOff;
    int32_t* nbFill;
    int32_t* nbIdx;
    float* nbDist;
    int32_t* err;          // set when a list would overflow its slots
    const uint64_t* heavy; // nct words: bit set for the columns drawn more than once (null: none)
    long long stallSpins;  // > 0: the stall test of k_sng_tc (sdb_set_debug_limits)
};
// First block pass: pass bits (mask may be null), row degrees, column counts.
int launch_sng_block(const SngArgs& a, cudaStream_t st);
// Second block pass (sngOptics): every passing pair into the CSR lists.
int launch_sng_emit(const SngArgs& a, cudaStream_t st);
int launch_sng_extras(const SngArgs& a, cudaStream_t st);
// BF16 screening of the block (Cosine, sngDbscan): Ub = BF16 sampled rows
// (nU x ldb); then the tensor-core block, the exact re-decision of the queued
// pairs and, when the screening failed (*gate != 0), the reset of the counts
// before the gated FP32 block.
int launch_sng_gather_bf16(const SngArgs& a, void* Ub, int ldb, cudaStream_t st);
int launch_sng_tc(const SngArgs& a, const void* Xb, const void* Ub, int ldb, uint64_t* queue, int64_t qcap,
                  unsigned long long* qcount, int32_t* gate, cudaStream_t st);
int launch_sng_col_of(const SngArgs& a, int32_t* colOf, cudaStream_t st);
// degree / core flags: sngDbscan counts draws (weights), sngOptics distinct neighbours
int launch_sng_degree(const SngArgs& a, int exact, int optics, int minPts, int32_t* degree, uint8_t* core,
                      cudaStream_t st);
// union-find over the core-core pass pairs and border minima (parents of core
// points compressed in between by the caller)
int launch_sng_union(const SngArgs& a, const uint8_t* core, int32_t* parent, cudaStream_t st);
int launch_sng_border(const SngArgs& a, const uint8_t* core, const int32_t* parent, int32_t* border,
                      cudaStream_t st);

// sngDbscan with independent samples per block of sng_block_rows() points
// (k_sng_blocks.cu): draw j of block b is the point
// floor(hi32(splitmix64(key + b S + j)) n / 2^32), key = splitmix64(seed).
struct SngBlockArgs {
    const float* Xt;
    int ld, d, dist, n;
    int64_t S;             // draws per block
    uint64_t key;
    float eps;
    uint32_t* words;       // blocks x S pass words (bit i: point 32 b + i)
    int32_t* degree;       // n, zeroed by the caller: passes with repeats, both sides
    unsigned long long* pairs;
    // sngOptics: per-point open-addressing tables of distinct neighbours
    const int64_t* hashOff;  // n + 1
    int32_t* hashId;         // -1 = empty
    float* hashDist;
    int32_t* err;            // set if a table overflows (cannot happen by construction)
};
int sng_block_rows();
// pass words, degrees and core flags
int launch_sngb_pass(const SngBlockArgs& a, int minPts, uint8_t* core, cudaStream_t st);
int launch_sngb_union(const SngBlockArgs& a, const uint8_t* core, int32_t* parent, cudaStream_t st);
int launch_sngb_border(const SngBlockArgs& a, const uint8_t* core, const int32_t* parent, int32_t* border,
                       cudaStream_t st);
// sngOptics under the same rule: table sizes (n + 1 entries into cap) from
// the pass's degrees, the emitting pass, distinct counts + core flags, and the
// tables compacted into CSR lists.
int launch_sngb_caps(const SngBlockArgs& a, int64_t* cap, cudaStream_t st);
int launch_sngb_emit(const SngBlockArgs& a, cudaStream_t st);
int launch_sngb_distinct(const SngBlockArgs& a, int minPts, int32_t* distinct, uint8_t* core, cudaStream_t st);
int launch_sngb_compact(const SngBlockArgs& a, const int64_t* nbOff, int32_t* nbIdx, float* nbDist, cudaStream_t st);

// sDbscan-1NN noise labelling (clusterNoise = 1), after the cluster labels.
struct NoiseArgs {
    int n, nproj, k;
    const float* P;          // n x nproj projections
    const int32_t* topK;     // n x 2k
    const uint8_t* core;
    int32_t* labels;         // in/out
    float samplingProb;
    uint32_t seed;
    int sMax;                // capacity of the sampled-core list
    int64_t* sampleFlag;     // n + 1 (scanned into indices)
    int64_t* noiseFlag;      // n + 1
    int32_t* cores;          // sMax: sampled core point ids, ascending
    int32_t* noise;          // n: noise point ids
    float* PcT;              // nproj x sMax
    int32_t* numCore;        // device scalar
    int64_t* scanTmp;
};
int launch_label_noise(const NoiseArgs& a, cudaStream_t st);

}  // namespace sdb
