// sngDbscan with independent samples (sng_findCorePoints,
// src/sDbscan.cpp:416-504, when every point's generator is seeded apart: the
// reference seeds each point from the clock when random_seed < 0, :437-440).
//
// One shared sample (the fixed-seed case, k_sng.cu) gives every sampled
// point about n reverse draws and the others none, which is not the
// reference's law when the points draw independently: then every point has S
// forward draws and about S reverse ones.  Here each block of BR = 32
// consecutive points draws its own S columns, which keeps that law (only the
// variance of the reverse count grows with the block size), and the block is
// still a dense tile: 128 draws x the block's 32 points.
//
// Draw j of block b: q = floor(hi32(splitmix64(splitmix64(seed) + b S + j)) n
// / 2^32), generated in the kernel (no draw array); a draw equal to the point
// itself is skipped.  Per pass (p, q), dist <= eps, both directions count once
// per draw (repeats counted, :459-464).  The pass bits are kept as one 32-bit
// word per (block, draw) over the block's points; the union-find and border
// passes walk the words.
//
// The distance tile is the candidate stage's FP32 tile (dist_tile.cuh): every
// distance is the CPU path's bits, so the result equals the oracle's
// restatement of the same rule (orc_fit_sngdbscan_blocks).
#include "dist_tile.cuh"
#include "uf.cuh"

#include <algorithm>
#include <climits>

namespace sdb {
namespace {

using namespace dtile;

constexpr int BR = 32;                       // points per sampled block
constexpr int BTX = 8, BCN = 4, BNT = 16 * BTX;  // 128 draws x 32 points on 128 threads

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ int block_draw(uint64_t key, int64_t S, int64_t b, int64_t j, int n) {
    const uint64_t z = splitmix64(key + (uint64_t)(b * S + j));
    return (int)(((z >> 32) * (uint64_t)n) >> 32);
}

size_t tile_smem() {
    return sizeof(float) * (STAGES * (TM + BTX * BCN) * LDS) + sizeof(int) * (TM + BTX * BCN);
}

// sngOptics: q into p's open-addressing table of distinct neighbours (ids,
// -1 = empty, with the pair's distance), linear probing from a
// multiplicative hash.
__device__ __forceinline__ void hash_insert(const SngBlockArgs& a, int p, int q, float dist) {
    const int64_t o = a.hashOff[p];
    const int cap = (int)(a.hashOff[p + 1] - o);
    if (cap == 0) {
        atomicExch(a.err, 1);
        return;
    }
    uint32_t h = ((uint32_t)q * 0x9E3779B1u) & (uint32_t)(cap - 1);
    for (int probe = 0; probe < cap; ++probe, h = (h + 1) & (uint32_t)(cap - 1)) {
        const int old = atomicCAS(a.hashId + o + h, -1, q);
        if (old == -1) {  // first occurrence of q in p's list
            a.hashDist[o + h] = dist;
            return;
        }
        if (old == q) return;  // a repeat: dist(p, q) is the same value every time
    }
    atomicExch(a.err, 1);  // full table (cannot happen: cap >= 2 x the entries)
}

// One tile (block b, draws dt * 128 ..) per CTA.  Tiles of a block are
// consecutive: the block's 32 rows stay in L1/L2 while its draws stream past.
// EMIT (sngOptics): the pass is repeated and every passing pair goes into
// both points' tables instead of the pass words and degrees.
template <int DIST, bool EMIT>
__global__ void __launch_bounds__(BNT, 4) k_sngb_tile(SngBlockArgs a) {
    extern __shared__ __align__(16) float sm[];
    float* As = sm;                              // STAGES x TM x LDS (the draws)
    float* Bs = As + STAGES * TM * LDS;          // STAGES x 32 x LDS (the block's points)
    int* rowPoint = reinterpret_cast<int*>(Bs + STAGES * (BTX * BCN) * LDS);
    int* colPoint = rowPoint + TM;
    __shared__ uint32_t sword[TM];
    __shared__ int colCount[BR];
    __shared__ int passTotal;

    const int tid = threadIdx.x;
    const int64_t nT = (a.S + TM - 1) / TM;
    const int64_t b = (int64_t)blockIdx.x / nT;
    const int64_t j0 = ((int64_t)blockIdx.x % nT) * TM;
    for (int r = tid; r < TM; r += BNT) {
        const int64_t j = j0 + r;
        rowPoint[r] = j < a.S ? block_draw(a.key, a.S, b, j, a.n) : -1;
        sword[r] = 0;
    }
    if (tid < BR) {
        const int64_t p = b * BR + tid;
        colPoint[tid] = p < a.n ? (int)p : -1;
        colCount[tid] = 0;
    }
    if (tid == 0) passTotal = 0;
    __syncthreads();

    float acc[8][BCN];
    accumulate<DIST, BTX, BCN>(a.Xt, a.ld, a.d, rowPoint, colPoint, As, Bs, acc);
    int ty, tx;
    tile_coords<BTX>(tid, ty, tx);
    int colPass[BCN] = {0, 0, 0, 0};
    int myPass = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int row = ty + 16 * i;
        const int q = rowPoint[row];
        uint32_t bits = 0;
#pragma unroll
        for (int jj = 0; jj < BCN; ++jj) {
            const int col = tx + BTX * jj;
            const int p = colPoint[col];
            const float dist = finish<DIST>(acc[i][jj]);
            const bool pass = q >= 0 && p >= 0 && p != q && dist <= a.eps;
            if (pass) {
                if (EMIT) {
                    hash_insert(a, p, q, dist);
                    hash_insert(a, q, p, dist);
                }
                bits |= 1u << col;
                colPass[jj] += 1;
                ++myPass;
            }
        }
        if (!EMIT && bits) atomicOr(&sword[row], bits);
    }
    if constexpr (!EMIT) {
#pragma unroll
        for (int jj = 0; jj < BCN; ++jj)
            if (colPass[jj]) atomicAdd(&colCount[tx + BTX * jj], colPass[jj]);
        const int wp = warp_sum(myPass);
        if ((tid & 31) == 0 && wp) atomicAdd(&passTotal, wp);
        __syncthreads();
        for (int r = tid; r < TM; r += BNT) {
            const int64_t j = j0 + r;
            if (j >= a.S) continue;
            const uint32_t w = sword[r];
            a.words[b * a.S + j] = w;
            if (w) atomicAdd(a.degree + rowPoint[r], __popc(w));  // the draw's side: once per passing point
        }
        if (tid < BR && colCount[tid]) atomicAdd(a.degree + colPoint[tid], colCount[tid]);  // the points' side
        if (tid == 0 && passTotal) atomicAdd(a.pairs, (unsigned long long)passTotal);
    }
}

__global__ void k_sngb_core(SngBlockArgs a, int minPts, uint8_t* __restrict__ core) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < a.n) core[p] = a.degree[p] >= minPts - 1 ? 1 : 0;
}

// Union of every passing core-core pair: a thread per (block, draw) word.
__global__ void k_sngb_union(SngBlockArgs a, const uint8_t* __restrict__ core, int32_t* parent) {
    const int64_t nb = (a.n + BR - 1) / BR, total = nb * a.S;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t w = __ldg(a.words + i);
        if (!w) continue;
        const int64_t b = i / a.S, j = i % a.S;
        const int q = block_draw(a.key, a.S, b, j, a.n);
        if (!core[q]) continue;
        while (w) {
            const int p = (int)(b * BR) + __ffs(w) - 1;
            w &= w - 1;
            if (core[p]) unite(parent, p, q);
        }
    }
}

// Border minima (parents of core points are roots by now): a non-core point
// takes the smallest root among its passing core neighbours, either side.
__global__ void k_sngb_border(SngBlockArgs a, const uint8_t* __restrict__ core, const int32_t* __restrict__ parent,
                              int32_t* border) {
    const int64_t nb = (a.n + BR - 1) / BR, total = nb * a.S;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t w = __ldg(a.words + i);
        if (!w) continue;
        const int64_t b = i / a.S, j = i % a.S;
        const int q = block_draw(a.key, a.S, b, j, a.n);
        const bool cq = core[q];
        const int rq = cq ? __ldcg(parent + q) : INT_MAX;
        int best = INT_MAX;
        while (w) {
            const int p = (int)(b * BR) + __ffs(w) - 1;
            w &= w - 1;
            const bool cp = core[p];
            if (cq && !cp) atomicMin(border + p, rq);
            if (cp && !cq) best = min(best, __ldcg(parent + p));
        }
        if (best != INT_MAX) atomicMin(border + q, best);
    }
}

// Hash table sizes: a power of two >= 2 x the point's passes with repeats.
__global__ void k_sngb_caps(SngBlockArgs a, int64_t* __restrict__ cap) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > a.n) return;
    int64_t c = 0;
    if (p < a.n && a.degree[p] > 0) {
        c = 2;
        while (c < 2 * (int64_t)a.degree[p]) c <<= 1;
    }
    cap[p] = c;
}

// Distinct neighbours per point (sngOptics, src/sDbscan.cpp:1537-1541): the
// filled slots of its table; degree = their count, core >= minPts - 1.
__global__ void k_sngb_distinct(SngBlockArgs a, int minPts, int32_t* __restrict__ distinct,
                                uint8_t* __restrict__ core) {
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned l = threadIdx.x & 31u;
    if (p >= a.n) return;
    int c = 0;
    for (int64_t t = a.hashOff[p] + l; t < a.hashOff[p + 1]; t += 32) c += a.hashId[t] >= 0;
    c = warp_sum(c);
    if (l == 0) {
        distinct[p] = c;
        core[p] = c >= minPts - 1 ? 1 : 0;
    }
}

// The tables compacted into the CSR lists (nbOff from a scan of distinct).
__global__ void k_sngb_compact(SngBlockArgs a, const int64_t* __restrict__ nbOff, int32_t* __restrict__ nbIdx,
                               float* __restrict__ nbDist) {
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned l = threadIdx.x & 31u;
    if (p >= a.n) return;
    int64_t out = nbOff[p];
    for (int64_t t0 = a.hashOff[p]; t0 < a.hashOff[p + 1]; t0 += 32) {
        const int64_t t = t0 + l;
        const bool have = t < a.hashOff[p + 1] && a.hashId[t] >= 0;
        const unsigned m = __ballot_sync(0xffffffffu, have);
        if (have) {
            const int64_t o = out + __popc(m & ((1u << l) - 1u));
            nbIdx[o] = a.hashId[t];
            nbDist[o] = a.hashDist[t];
        }
        out += __popc(m);
    }
}

template <int DIST, bool EMIT> int launch_tile_t(const SngBlockArgs& a, cudaStream_t st) {
    const size_t sm = tile_smem();
    if (cudaFuncSetAttribute(k_sngb_tile<DIST, EMIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess)
        return -1;
    const int64_t nb = (a.n + BR - 1) / BR, nT = (a.S + TM - 1) / TM;
    const int64_t tiles = nb * nT;
    if (tiles <= 0) return 0;
    if (tiles > (int64_t)INT_MAX) return -1;
    k_sngb_tile<DIST, EMIT><<<(unsigned)tiles, BNT, sm, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <bool EMIT> int launch_tiles(const SngBlockArgs& a, cudaStream_t st) {
    switch (a.dist) {
        case DIST_COSINE: return launch_tile_t<DIST_COSINE, EMIT>(a, st);
        case DIST_L1: return launch_tile_t<DIST_L1, EMIT>(a, st);
        case DIST_L2: return launch_tile_t<DIST_L2, EMIT>(a, st);
        case DIST_CHI2: return launch_tile_t<DIST_CHI2, EMIT>(a, st);
        case DIST_JS: return launch_tile_t<DIST_JS, EMIT>(a, st);
    }
    return -1;
}

int grid_words(const SngBlockArgs& a) {
    const int64_t total = (int64_t)((a.n + BR - 1) / BR) * a.S;
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16));
}

}  // namespace

int sng_block_rows() { return BR; }

int launch_sngb_pass(const SngBlockArgs& a, int minPts, uint8_t* core, cudaStream_t st) {
    const int r = launch_tiles<false>(a, st);
    if (r < 0) return -1;
    k_sngb_core<<<(a.n + 255) / 256, 256, 0, st>>>(a, minPts, core);
    return cudaPeekAtLastError() == cudaSuccess ? r + 1 : -1;
}

int launch_sngb_union(const SngBlockArgs& a, const uint8_t* core, int32_t* parent, cudaStream_t st) {
    k_sngb_union<<<grid_words(a), 256, 0, st>>>(a, core, parent);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sngb_border(const SngBlockArgs& a, const uint8_t* core, const int32_t* parent, int32_t* border,
                       cudaStream_t st) {
    k_sngb_border<<<grid_words(a), 256, 0, st>>>(a, core, parent, border);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// sngOptics: table sizes from the pass's degrees (cap: n + 1 entries, scanned
// by the caller into hashOff), then the emitting pass into the tables.
int launch_sngb_caps(const SngBlockArgs& a, int64_t* cap, cudaStream_t st) {
    k_sngb_caps<<<(a.n + 1 + 255) / 256, 256, 0, st>>>(a, cap);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sngb_emit(const SngBlockArgs& a, cudaStream_t st) { return launch_tiles<true>(a, st); }

int launch_sngb_distinct(const SngBlockArgs& a, int minPts, int32_t* distinct, uint8_t* core, cudaStream_t st) {
    k_sngb_distinct<<<(a.n + 7) / 8, 256, 0, st>>>(a, minPts, distinct, core);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sngb_compact(const SngBlockArgs& a, const int64_t* nbOff, int32_t* nbIdx, float* nbDist, cudaStream_t st) {
    k_sngb_compact<<<(a.n + 7) / 8, 256, 0, st>>>(a, nbOff, nbIdx, nbDist);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
