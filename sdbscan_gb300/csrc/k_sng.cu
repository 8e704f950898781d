// sngDbscan / sngOptics: neighbourhoods from random samples
// (sng_findCorePoints, src/sDbscan.cpp:416-504; sng_findCoreDist, :1484-1583).
//
// In the reference every point draws its sample from its own generator.
// With a fixed seed (sngDbscan, random_seed >= 0, :437-440) every point's
// generator is seeded alike, so all points draw the same index sequence and
// differ only in skipping their own index.  The host splits that sequence
// into one shared multiset of columns (the first S draws: distinct ids with
// their multiplicities) and, for each sampled point, the few extra draws that
// replace its own occurrences.  The GPU work is then a dense block: every
// point (row) against every distinct sampled point (column), computed with
// the FP32 distance tile of the candidate stage (same rounding sequence as
// the CPU path), plus a short list of extra pairs.
//
// Per pass (p, q), p != q, dist <= eps:
//  - sngDbscan, sampled (:446-464): p's list gets q and q's list gets p once
//    per draw of q, so deg(p) += mult(q) and deg(q) += mult(q);
//  - sngDbscan, exact (samplingProb >= 1, :466-479): only the row side,
//    deg(p) += 1 (the relation is symmetric by itself);
//  - sngOptics (:1493-1555): lists are de-duplicated (:1537-1541); p's
//    distinct neighbours are its row when p is not sampled, and its column
//    when it is (its row is a subset of its column: the distance is
//    symmetric), each with its distance.
// Pass bits are kept tile-major (word ct * n + p) so that the first pass
// writes and the cluster kernels read them coalesced.
#include "dist_tile.cuh"
#include "uf.cuh"

#include <algorithm>
#include <climits>

namespace sdb {
namespace {

using namespace dtile;

constexpr int kTX = 16, kCN = 4, kNT = 16 * kTX, kTNK = kTX * kCN;  // 128 x 64 tiles on 256 threads

size_t block_smem() {
    return sizeof(float) * (STAGES * (TM + kTNK) * LDS) + sizeof(int) * (2 * TM + 3 * kTNK + 2 * TM);
}

// One 128-row x 64-column tile of the block per CTA; tiles of a row block are
// consecutive so that a wave shares its rows in L2 and the sampled columns
// (a few MB) stay L2-resident.
template <int DIST, bool EMIT>
__global__ void __launch_bounds__(kNT, 2) k_sng_block(SngArgs a) {
    extern __shared__ __align__(16) float sm[];
    float* As = sm;                           // STAGES x TM x LDS
    float* Bs = As + STAGES * TM * LDS;       // STAGES x 64 x LDS
    int* rowPoint = reinterpret_cast<int*>(Bs + STAGES * kTNK * LDS);
    int* rowSampled = rowPoint + TM;
    int* colPoint = rowSampled + TM;
    int* colW = colPoint + kTNK;
    int* colCount = colW + kTNK;
    unsigned* smask = reinterpret_cast<unsigned*>(colCount + kTNK);  // TM x 2
    __shared__ int passTotal;

    const int tid = threadIdx.x;
    const int64_t t = blockIdx.x;
    const int rb = (int)(t / a.nct), ct = (int)(t % a.nct);
    const int p0 = rb * TM;
    for (int i = tid; i < TM; i += kNT) {
        const int p = p0 + i;
        rowPoint[i] = p < a.n ? p : -1;
        rowSampled[i] = (EMIT && p < a.n) ? (__ldg(a.colOf + p) >= 0) : 0;
        smask[2 * i] = 0;
        smask[2 * i + 1] = 0;
    }
    for (int j = tid; j < kTNK; j += kNT) {
        const int c = ct * kTNK + j;
        colPoint[j] = c < a.nU ? __ldg(a.cols + c) : -1;
        colW[j] = (c < a.nU && a.mult != nullptr) ? __ldg(a.mult + c) : 1;
        colCount[j] = 0;
    }
    if (tid == 0) passTotal = 0;
    __syncthreads();

    float acc[8][kCN];
    accumulate<DIST, kTX, kCN>(a.Xt, a.ld, a.d, rowPoint, colPoint, As, Bs, acc);
    int ty, tx;
    tile_coords<kTX>(tid, ty, tx);

    int myPass = 0;
    int colPass[kCN];
#pragma unroll
    for (int j = 0; j < kCN; ++j) colPass[j] = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int row = ty + 16 * i;
        const int p = rowPoint[row];
        unsigned lo = 0, hi = 0;
#pragma unroll
        for (int j = 0; j < kCN; ++j) {
            const int col = tx + kTX * j;
            const int q = colPoint[col];
            const float dist = finish<DIST>(acc[i][j]);
            const bool pass = p >= 0 && q >= 0 && p != q && dist <= a.eps;
            if (!pass) continue;
            if (EMIT) {
                if (!rowSampled[row]) {  // p's own list: its row
                    const int s = atomicAdd(a.nbFill + p, 1);
                    const int64_t o = a.nbOff[p] + s;
                    if (o < a.nbOff[p + 1]) {
                        a.nbIdx[o] = q;
                        a.nbDist[o] = dist;
                    } else {
                        atomicExch(a.err, 1);
                    }
                }
                const int s = atomicAdd(a.nbFill + q, 1);  // q's list: its column
                const int64_t o = a.nbOff[q] + s;
                if (o < a.nbOff[q + 1]) {
                    a.nbIdx[o] = p;
                    a.nbDist[o] = dist;
                } else {
                    atomicExch(a.err, 1);
                }
            } else {
                if (col < 32) lo |= 1u << col;
                else hi |= 1u << (col - 32);
                colPass[j] += 1;
                ++myPass;
            }
        }
        if constexpr (!EMIT) {
            if (lo) atomicOr(&smask[2 * row], lo);
            if (hi) atomicOr(&smask[2 * row + 1], hi);
        }
    }
    if constexpr (!EMIT) {
#pragma unroll
        for (int j = 0; j < kCN; ++j)
            if (colPass[j]) atomicAdd(&colCount[tx + kTX * j], colPass[j]);
        const int wp = warp_sum(myPass);
        if ((tid & 31) == 0 && wp) atomicAdd(&passTotal, wp);
        __syncthreads();
        for (int row = tid; row < TM; row += kNT) {
            const int p = rowPoint[row];
            if (p < 0) continue;
            const uint64_t w = ((uint64_t)smask[2 * row + 1] << 32) | smask[2 * row];
            if (a.mask != nullptr) a.mask[(size_t)ct * a.n + p] = w;
            if (w) {
                int s = 0;
                uint64_t b = w;
                while (b) {
                    s += colW[__ffsll((long long)b) - 1];
                    b &= b - 1;
                }
                atomicAdd(a.rowDeg + p, s);
            }
        }
        for (int j = tid; j < kTNK; j += kNT)
            if (colCount[j]) atomicAdd(a.colCnt + ct * kTNK + j, colCount[j]);
        if (tid == 0 && passTotal) atomicAdd(a.pairs, (unsigned long long)passTotal);
    }
}

// The extra draws of sampled points: one thread per (point, drawn point).
template <int DIST>
__global__ void k_sng_extras(SngArgs a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nExtra; i += gridDim.x * blockDim.x) {
        const int2 e = a.extras[i];
        const float dist = pair_distance<DIST>(a.Xt + (size_t)e.x * a.ld, a.Xt + (size_t)e.y * a.ld, a.d);
        const bool pass = dist <= a.eps;
        a.extraPass[i] = pass ? 1 : 0;
        if (pass) {
            atomicAdd(a.rowDeg + e.x, 1);
            atomicAdd(a.rowDeg + e.y, 1);
            atomicAdd(a.pairs, 1ull);
        }
    }
}

__global__ void k_sng_col_of(const int32_t* __restrict__ cols, int nU, int32_t* __restrict__ colOf) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nU) colOf[cols[c]] = c;
}

__global__ void k_sng_degree(SngArgs a, int exact, int optics, int minPts, int32_t* __restrict__ degree,
                             uint8_t* __restrict__ core) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int c = a.colOf[p];
    int deg;
    if (optics) deg = c >= 0 ? a.colCnt[c] : a.rowDeg[p];
    else deg = a.rowDeg[p] + ((c >= 0 && !exact) ? a.mult[c] * a.colCnt[c] : 0);
    degree[p] = deg;
    core[p] = deg >= minPts - 1 ? 1 : 0;
}

// The cluster kernels run on a 2-D grid: 256 consecutive rows (a thread per
// row) x a group of kGroup consecutive mask words.  A CTA loads its rows'
// words at once, finds the roots of the group's 64 kGroup columns in parallel
// and caches them in shared memory; the many independent CTAs hide the
// latency of the finds.  A core row unites only where its own root differs
// from a passing core column's cached root.  A cached value is an ancestor
// of its column (parents only move up), so equality proves the same set; a
// stale value only costs a redundant unite.
constexpr int kGroup = 8;

__global__ void __launch_bounds__(256) k_sng_union(SngArgs a, const uint8_t* __restrict__ core, int32_t* parent) {
    __shared__ int croot[kGroup][kTNK];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < a.n && core[p];
    const int ct0 = blockIdx.y * kGroup, nw = min(kGroup, a.nct - ct0);
    uint64_t w[kGroup];
    bool any = false;
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
        w[k] = (active && k < nw)
                   ? __ldg(reinterpret_cast<const unsigned long long*>(a.mask) + (size_t)(ct0 + k) * a.n + p)
                   : 0ull;
        any |= w[k] != 0;
    }
    if (!__syncthreads_or(any)) return;
    for (int e = threadIdx.x; e < nw * kTNK; e += blockDim.x) {
        const int c = ct0 * kTNK + e;
        const int q = c < a.nU ? __ldg(a.cols + c) : -1;
        croot[e / kTNK][e % kTNK] = (q >= 0 && core[q]) ? find_root(parent, q) : -1;
    }
    __syncthreads();
    if (!any) return;
    int rp = find_root(parent, p);
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
        uint64_t bits = w[k];
        while (bits) {
            const int j = __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const int cr = croot[k][j];
            if (cr < 0 || cr == rp) continue;
            unite(parent, rp, cr);
            rp = find_root(parent, rp);
        }
    }
}

__global__ void k_sng_extras_union(SngArgs a, const uint8_t* __restrict__ core, int32_t* parent) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nExtra; i += gridDim.x * blockDim.x) {
        const int2 e = a.extras[i];
        if (a.extraPass[i] && core[e.x] && core[e.y]) unite(parent, e.x, e.y);
    }
}

// Border minima (parents of core points are roots here), on the same 2-D
// grid: a non-core row takes the smallest root among its passing core
// columns; the roots that core rows offer to a non-core column are reduced in
// shared memory first, one global atomic per column and CTA.
__global__ void __launch_bounds__(256) k_sng_border(SngArgs a, const uint8_t* __restrict__ core,
                                                   const int32_t* __restrict__ parent, int32_t* border) {
    __shared__ int croot[kGroup][kTNK], cbest[kGroup][kTNK];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.n;
    const bool pc = valid && core[p];
    const int rp = pc ? __ldcg(parent + p) : INT_MAX;
    const int ct0 = blockIdx.y * kGroup, nw = min(kGroup, a.nct - ct0);
    uint64_t w[kGroup];
    bool any = false;
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
        w[k] = (valid && k < nw)
                   ? __ldg(reinterpret_cast<const unsigned long long*>(a.mask) + (size_t)(ct0 + k) * a.n + p)
                   : 0ull;
        any |= w[k] != 0;
    }
    if (!__syncthreads_or(any)) return;
    for (int e = threadIdx.x; e < nw * kTNK; e += blockDim.x) {
        const int c = ct0 * kTNK + e;
        const int q = c < a.nU ? __ldg(a.cols + c) : -1;
        croot[e / kTNK][e % kTNK] = (q >= 0 && core[q]) ? __ldcg(parent + q) : INT_MAX;
        cbest[e / kTNK][e % kTNK] = INT_MAX;
    }
    __syncthreads();
    int best = INT_MAX;
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
        uint64_t bits = w[k];
        while (bits) {
            const int j = __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const int cr = croot[k][j];
            if (pc) {
                if (cr == INT_MAX) atomicMin(&cbest[k][j], rp);  // a non-core column (set bits are valid columns)
            } else {
                best = min(best, cr);
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nw * kTNK; e += blockDim.x)
        if (cbest[e / kTNK][e % kTNK] != INT_MAX)
            atomicMin(border + __ldg(a.cols + ct0 * kTNK + e), cbest[e / kTNK][e % kTNK]);
    if (best != INT_MAX) atomicMin(border + p, best);
}

__global__ void k_sng_extras_border(SngArgs a, const uint8_t* __restrict__ core, const int32_t* __restrict__ parent,
                                    int32_t* border) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nExtra; i += gridDim.x * blockDim.x) {
        if (!a.extraPass[i]) continue;
        const int2 e = a.extras[i];
        const bool cx = core[e.x], cy = core[e.y];
        if (cx && !cy) atomicMin(border + e.y, __ldcg(parent + e.x));
        if (cy && !cx) atomicMin(border + e.x, __ldcg(parent + e.y));
    }
}

template <int DIST, bool EMIT>
int launch_block_t(const SngArgs& a, cudaStream_t st) {
    const size_t sm = block_smem();
    if (cudaFuncSetAttribute(k_sng_block<DIST, EMIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess)
        return -1;
    const int64_t tiles = (int64_t)((a.n + TM - 1) / TM) * a.nct;
    if (tiles <= 0) return 0;
    if (tiles > (int64_t)INT_MAX) return -1;
    k_sng_block<DIST, EMIT><<<(unsigned)tiles, kNT, sm, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <bool EMIT>
int launch_block(const SngArgs& a, cudaStream_t st) {
    switch (a.dist) {
        case DIST_COSINE: return launch_block_t<DIST_COSINE, EMIT>(a, st);
        case DIST_L1: return launch_block_t<DIST_L1, EMIT>(a, st);
        case DIST_L2: return launch_block_t<DIST_L2, EMIT>(a, st);
        case DIST_CHI2: return launch_block_t<DIST_CHI2, EMIT>(a, st);
        case DIST_JS: return launch_block_t<DIST_JS, EMIT>(a, st);
    }
    return -1;
}

int grid_for(int64_t work, int threads) {
    const int64_t b = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm_count() * 8));
}

}  // namespace

int launch_sng_block(const SngArgs& a, cudaStream_t st) { return launch_block<false>(a, st); }
int launch_sng_emit(const SngArgs& a, cudaStream_t st) { return launch_block<true>(a, st); }

int launch_sng_extras(const SngArgs& a, cudaStream_t st) {
    if (a.nExtra <= 0) return 0;
    const int g = grid_for(a.nExtra, 128);
    switch (a.dist) {
        case DIST_COSINE: k_sng_extras<DIST_COSINE><<<g, 128, 0, st>>>(a); break;
        case DIST_L1: k_sng_extras<DIST_L1><<<g, 128, 0, st>>>(a); break;
        case DIST_L2: k_sng_extras<DIST_L2><<<g, 128, 0, st>>>(a); break;
        case DIST_CHI2: k_sng_extras<DIST_CHI2><<<g, 128, 0, st>>>(a); break;
        case DIST_JS: k_sng_extras<DIST_JS><<<g, 128, 0, st>>>(a); break;
        default: return -1;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sng_col_of(const SngArgs& a, int32_t* colOf, cudaStream_t st) {
    if (cudaMemsetAsync(colOf, 0xff, sizeof(int32_t) * (size_t)a.n, st) != cudaSuccess) return -1;
    if (a.nU <= 0) return 0;
    k_sng_col_of<<<(a.nU + 255) / 256, 256, 0, st>>>(a.cols, a.nU, colOf);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sng_degree(const SngArgs& a, int exact, int optics, int minPts, int32_t* degree, uint8_t* core,
                      cudaStream_t st) {
    k_sng_degree<<<(a.n + 255) / 256, 256, 0, st>>>(a, exact, optics, minPts, degree, core);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sng_union(const SngArgs& a, const uint8_t* core, int32_t* parent, cudaStream_t st) {
    int launches = 0;
    if (a.nct > 0) {
        k_sng_union<<<dim3((a.n + 255) / 256, (a.nct + kGroup - 1) / kGroup), 256, 0, st>>>(a, core, parent);
        ++launches;
    }
    if (a.nExtra > 0) {
        k_sng_extras_union<<<grid_for(a.nExtra, 256), 256, 0, st>>>(a, core, parent);
        ++launches;
    }
    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

int launch_sng_border(const SngArgs& a, const uint8_t* core, const int32_t* parent, int32_t* border,
                      cudaStream_t st) {
    int launches = 0;
    if (a.nct > 0) {
        k_sng_border<<<dim3((a.n + 255) / 256, (a.nct + kGroup - 1) / kGroup), 256, 0, st>>>(a, core, parent,
                                                                                          border);
        ++launches;
    }
    if (a.nExtra > 0) {
        k_sng_extras_border<<<grid_for(a.nExtra, 256), 256, 0, st>>>(a, core, parent, border);
        ++launches;
    }
    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

}  // namespace sdb
