// Stage 4: candidate distances and the eps test — the dominant loop of
// rp_findCorePoints / rp_findCoreDist (src/sDbscan.cpp:243-359, :1323-1412)
// with computeDist (src/Utilities.h:212-287).
//
// Formulation: a grouped, gathered GEMM.  Tile = (list l, 128 member rows,
// 64 candidate columns).  The member rows are gathered from the transformed
// data by point id, the candidate rows are the list's top-m points; both are
// staged through shared memory with cp.async (3 stages, 32 dimensions per
// stage).  Each of the 256 threads owns an 8 x 4 block of (member, candidate)
// pairs and accumulates over dimensions in ascending order with one fmaf per
// dimension — the same sequence of roundings as the oracle's dot product — so
// every distance, and so every eps decision, is bit-identical to the CPU path.
//
// Epilogue per tile:
//  - mask word per (member point, slot): bit s set when candidate s is within
//    eps and is not the point itself (src/sDbscan.cpp:272, :286);
//  - inRaw[candidate] += number of members of this tile that pass (the
//    reverse edges n -> candidate, src/sDbscan.cpp:293-294);
//  - optionally the distance of every (member, candidate) pair (sOPTICS).
#include "dist_tile.cuh"

namespace sdb {
namespace {

using namespace dtile;

// Candidate columns per tile are TX * CN (TX column groups of CN columns, 16
// row groups of 8 rows): <16, 4> gives 64 columns on 256 threads (any m, one
// 64-bit mask word per tile) and <10, 5> exactly 50 columns on 160 threads
// (m in 41..50, no padded columns).

// Shared memory of one k_dist CTA; CTAs per SM for the launch bounds (three
// 160-thread CTAs fit the register file at 128 registers; the smem of a
// third must leave room).
template <int TX, int CN, int KT, int NST> constexpr size_t dist_smem() {
    return sizeof(float) * (NST * (TM + TX * CN) * (KT + 4)) + sizeof(int) * (3 * TM + 2 * TX * CN + 2 * TM);
}
template <int TX, int CN, int KT, int NST> constexpr int dist_min_blocks() {
    return TX == 10 && dist_smem<TX, CN, KT, NST>() <= 74 * 1024 ? 3 : 2;
}

template <int DIST, int TX, int CN, int KT, int NST>
__global__ void __launch_bounds__(16 * TX, (dist_min_blocks<TX, CN, KT, NST>())) k_dist(DistArgs a) {
    constexpr int NT = 16 * TX, TNK = TX * CN;  // threads, candidate columns this kernel computes
    if (a.gate != nullptr && __ldg(a.gate) == 0) return;  // the BF16 screening succeeded
    extern __shared__ __align__(16) float sm[];
    float* As = sm;                                   // NST x TM x (KT + 4)
    float* Bs = As + NST * TM * (KT + 4);             // NST x TNK x (KT + 4)
    int* rowPoint = reinterpret_cast<int*>(Bs + NST * TNK * (KT + 4));
    int* rowSlot = rowPoint + TM;
    int* colPoint = rowSlot + TM;
    unsigned* smask = reinterpret_cast<unsigned*>(colPoint + TNK);  // TM x 2
    int* colCount = reinterpret_cast<int*>(smask + 2 * TM);           // TNK
    __shared__ int passTotal;

    const int tid = threadIdx.x;
    if ((int64_t)blockIdx.x >= *a.tileTotal) return;
    const int64_t t = tile_at(a.tilePerm, blockIdx.x);
    const int l = a.tileList[t];
    const int64_t ti = t - a.tileOff[l];
    const int mt = (int)(ti / a.nct), ct = (int)(ti % a.nct);
    const int64_t mbeg = a.listOff[l] + (int64_t)mt * TM;
    const int64_t mend = a.listOff[l + 1];
    const int r = l % a.nproj, side = l / a.nproj;
    const int32_t* cand = a.topM + (size_t)r * 2 * a.m + side * a.m;

    for (int i = tid; i < TM; i += NT) {
        const int64_t q = mbeg + i;
        if (q < mend) {
            const int2 mb = a.members[q];
            rowPoint[i] = mb.x;
            rowSlot[i] = mb.y;
        } else {
            rowPoint[i] = -1;
            rowSlot[i] = 0;
        }
        smask[2 * i] = 0;
        smask[2 * i + 1] = 0;
    }
    for (int j = tid; j < TNK; j += NT) {
        const int c = ct * TN + j;
        colPoint[j] = c < a.m ? cand[c] : -1;
        colCount[j] = 0;
    }
    if (tid == 0) passTotal = 0;
    __syncthreads();

    float acc[8][CN];
    accumulate<DIST, TX, CN, KT, NST>(a.Xt, a.ld, a.d, rowPoint, colPoint, As, Bs, acc);
    int ty, tx;
    tile_coords<TX>(tid, ty, tx);

    // epilogue
    int myPass = 0;
    int colPass[CN];
#pragma unroll
    for (int j = 0; j < CN; ++j) colPass[j] = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int row = ty + 16 * i;
        const int p = rowPoint[row];
        unsigned lo = 0, hi = 0;
#pragma unroll
        for (int j = 0; j < CN; ++j) {
            const int col = tx + TX * j;
            const int q = colPoint[col];
            const float dist = finish<DIST>(acc[i][j]);
            const bool pass = p >= 0 && q >= 0 && p != q && dist <= a.eps;
            if (pass) {
                if (col < 32) lo |= 1u << col;
                else hi |= 1u << (col - 32);
                colPass[j] += 1;
                ++myPass;
            }
            if (a.dists != nullptr && p >= 0 && q >= 0)
                a.dists[((size_t)p * 2 * a.k + rowSlot[row]) * a.m + ct * TN + col] = dist;
        }
        if (lo) atomicOr(&smask[2 * row], lo);
        if (hi) atomicOr(&smask[2 * row + 1], hi);
    }
#pragma unroll
    for (int j = 0; j < CN; ++j)
        if (colPass[j]) atomicAdd(&colCount[tx + TX * j], colPass[j]);
    const int wp = warp_sum(myPass);
    if ((tid & 31) == 0 && wp) atomicAdd(&passTotal, wp);
    __syncthreads();
    for (int row = tid; row < TM; row += NT) {
        const int p = rowPoint[row];
        if (p >= 0) {
            const uint64_t w = ((uint64_t)smask[2 * row + 1] << 32) | smask[2 * row];
            a.masks[((size_t)p * 2 * a.k + rowSlot[row]) * a.W + ct] = w;
        }
    }
    for (int j = tid; j < TNK; j += NT)
        if (colCount[j]) atomicAdd(a.inRaw + colPoint[j], colCount[j]);
    if (tid == 0 && passTotal) atomicAdd(a.pairs, (unsigned long long)passTotal);
}

template <int DIST, int TX, int CN, int KT = TK, int NST = STAGES> int launch_dist_v(const DistArgs& a, cudaStream_t st) {
    const size_t sm = dist_smem<TX, CN, KT, NST>();
    if (cudaFuncSetAttribute(k_dist<DIST, TX, CN, KT, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess)
        return -1;
    if (a.nTiles <= 0) return 0;
    k_dist<DIST, TX, CN, KT, NST><<<(unsigned)a.nTiles, 16 * TX, sm, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// Tile shape: the caller's (autotuned) choice, else exact 50-column tiles for
// m in 41..50 and 64-column tiles otherwise.  Variants: 1 = 128 x 64 (256
// threads, 32 dimensions per stage, 2 stages), 2 = 128 x 50 (160 threads, 32
// dimensions, 2 stages), 3 = 128 x 50 (160 threads, 16 dimensions, 4 stages:
// the same shared memory, half the work between barriers and twice the loads
// in flight; 3 % faster than 2 for Cosine at 1M x 784, 2.5 % slower for Chi2
// at 500K x 512, so the other distances run shape 2 for it).  The 50-column
// shapes need m <= 50.
template <int DIST> int launch_dist_t(const DistArgs& a, cudaStream_t st) {
    const bool fits50 = a.m <= 50;
    if (a.variant == 4 || a.variant == 5) return launch_dist_ws(a, a.variant, st);
    switch (a.variant) {
        case 2: if (fits50) return launch_dist_v<DIST, 10, 5>(a, st); break;
        case 3:  // the 4-stage shape is built for the FMA-bound Cosine tile only (Chi2: 2.5 % slower)
        case 0:
            if (fits50 && (a.variant == 3 || a.m > 40)) {
                if constexpr (DIST == DIST_COSINE) return launch_dist_v<DIST, 10, 5, 16, 4>(a, st);
                else return launch_dist_v<DIST, 10, 5>(a, st);
            }
            break;
        default: break;
    }
    return launch_dist_v<DIST, 16, 4>(a, st);
}

// eps masks and reverse counts from stored distances (eps sweeps: the
// distances are computed once per dataset and thresholded per eps, the
// pattern of the reference's test_sDbscan, src/sDbscan.cpp:1009-1038).
// Same tiles as k_dist; one warp per member row, lanes over candidates.
__global__ void k_masks_from_dists(DistArgs a) {
    __shared__ int colCount[TN];
    __shared__ int passTotal;
    if ((int64_t)blockIdx.x >= *a.tileTotal) return;
    const int64_t t = tile_at(a.tilePerm, blockIdx.x);
    const int l = a.tileList[t];
    const int64_t ti = t - a.tileOff[l];
    const int mt = (int)(ti / a.nct), ct = (int)(ti % a.nct);
    const int64_t mbeg = a.listOff[l] + (int64_t)mt * TM, mend = a.listOff[l + 1];
    const int r = l % a.nproj, side = l / a.nproj;
    const int32_t* cand = a.topM + (size_t)r * 2 * a.m + side * a.m;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int j = threadIdx.x; j < TN; j += blockDim.x) colCount[j] = 0;
    if (threadIdx.x == 0) passTotal = 0;
    __syncthreads();
    int myPass = 0;
    for (int row = warp; row < TM; row += warps) {
        const int64_t q = mbeg + row;
        if (q >= mend) break;
        const int2 mb = a.members[q];
        const int p = mb.x, slot = mb.y;
        uint32_t half[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int col = h * 32 + lane;
            const int c = ct * TN + col;
            bool pass = false;
            if (c < a.m) {
                const int cp = __ldg(cand + c);
                const size_t at = ((size_t)p * 2 * a.k + slot) * a.m + c;
                const float dd = __ldg(a.dists + at);
                pass = cp != p && dd <= a.eps && dd > a.epsLo;
                if (pass) {
                    atomicAdd(&colCount[col], 1);
                    ++myPass;
                }
            }
            half[h] = __ballot_sync(0xffffffffu, pass);
        }
        if (lane == 0) a.masks[((size_t)p * 2 * a.k + slot) * a.W + ct] = ((uint64_t)half[1] << 32) | half[0];
    }
    const int wp = warp_sum(myPass);
    if (lane == 0 && wp) atomicAdd(&passTotal, wp);
    __syncthreads();
    for (int j = threadIdx.x; j < TN; j += blockDim.x) {
        const int c = ct * TN + j;
        if (colCount[j]) atomicAdd(a.inRaw + cand[c], colCount[j]);
    }
    if (threadIdx.x == 0 && passTotal) atomicAdd(a.pairs, (unsigned long long)passTotal);
}

// One pass over the stored distances: the sweep round in which each pair
// joins (its distance's rank among the ascending eps values), so that every
// round reads one byte per pair instead of the distance.  Rows (point, slot)
// are padded to W * 64 bytes so a round reads them with aligned 16-byte
// loads; padding columns and the point's own entry (a candidate equal to the
// point, src/sDbscan.cpp:272) get 255, which no round matches.
__global__ void k_pair_rounds(const float* __restrict__ dists, DistArgs a, uint32_t* __restrict__ rounds) {
    const int g4 = a.W * 16;  // four-column groups per padded row
    const size_t count = (size_t)a.n * 2 * a.k * g4;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / g4;
        const int c0 = (int)(i % g4) * 4;
        const int p = (int)(row / (2 * a.k)), slot = (int)(row % (2 * a.k));
        const int32_t* cand = a.topM + (size_t)__ldg(a.topKmat + row) * 2 * a.m + (slot >= a.k ? a.m : 0);
        uint32_t out = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int c = c0 + b;
            int r = 255;
            if (c < a.m && __ldg(cand + c) != p) {
                const float d = __ldg(dists + row * a.m + c);
                r = 0;
                while (r < a.nSweep && a.sweepEps[r] < d) ++r;
            }
            out |= (uint32_t)r << (8 * b);
        }
        rounds[i] = out;
    }
}

// A round's masks from the pair rounds: thread per member row of a tile; the
// row's 64 round bytes for this tile come in as four 16-byte loads and are
// compared four at a time (__vcmpeq4), giving the row's mask word directly;
// the column counts (reverse edges) are reduced with one ballot per column.
__global__ void __launch_bounds__(TM) k_masks_from_rounds(DistArgs a) {
    __shared__ int colCount[TN];
    if ((int64_t)blockIdx.x >= *a.tileTotal) return;
    const int64_t t = tile_at(a.tilePerm, blockIdx.x);
    const int l = a.tileList[t];
    const int64_t ti = t - a.tileOff[l];
    const int mt = (int)(ti / a.nct), ct = (int)(ti % a.nct);
    const int64_t q = a.listOff[l] + (int64_t)mt * TM + threadIdx.x;
    const bool valid = q < a.listOff[l + 1];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < TN) colCount[threadIdx.x] = 0;
    __syncthreads();
    uint64_t w = 0;
    int2 mb = make_int2(0, 0);
    if (valid) {
        mb = a.members[q];
        const uint4* src = reinterpret_cast<const uint4*>(a.pairRound + ((size_t)mb.x * 2 * a.k + mb.y) * (a.W * 64) +
                                                          (size_t)ct * 64);
        const uint32_t rr = 0x01010101u * (uint32_t)a.round;
#pragma unroll
        for (int v4 = 0; v4 < 4; ++v4) {
            const uint4 x = __ldg(src + v4);
            const uint32_t words[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int k4 = 0; k4 < 4; ++k4) {
                // low bit of each equal byte, gathered into a nibble
                const uint32_t eq = __vcmpeq4(words[k4], rr) & 0x01010101u;
                w |= (uint64_t)((eq * 0x10204080u) >> 28) << (v4 * 16 + k4 * 4);
            }
        }
        a.masks[((size_t)mb.x * 2 * a.k + mb.y) * a.W + ct] = w;
    }
    int cc0 = 0, cc1 = 0;  // passes of columns lane and lane + 32 in this warp
#pragma unroll
    for (int col = 0; col < TN; ++col) {
        const int pc = __popc(__ballot_sync(0xffffffffu, (w >> col) & 1ull));
        if (lane == (col & 31)) {
            if (col < 32) cc0 += pc;
            else cc1 += pc;
        }
    }
    if (cc0) atomicAdd(&colCount[lane], cc0);
    if (cc1) atomicAdd(&colCount[lane + 32], cc1);
    const int wp = warp_sum(__popcll(w));
    if (lane == 0 && wp) atomicAdd(a.pairs, (unsigned long long)wp);
    __syncthreads();
    if (threadIdx.x < TN && colCount[threadIdx.x]) {
        const int r = l % a.nproj, side = l / a.nproj;
        const int c = ct * TN + threadIdx.x;
        atomicAdd(a.inRaw + __ldg(a.topM + (size_t)r * 2 * a.m + side * a.m + c), colCount[threadIdx.x]);
    }
}

}  // namespace

int launch_pair_rounds(const DistArgs& a, uint8_t* rounds, cudaStream_t st) {
    k_pair_rounds<<<sm_count() * 16, 256, 0, st>>>(a.dists, a, reinterpret_cast<uint32_t*>(rounds));
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_masks_from_dists(const DistArgs& a, cudaStream_t st) {
    if (a.nTiles <= 0) return 0;
    if (a.pairRound != nullptr) k_masks_from_rounds<<<(unsigned)a.nTiles, TM, 0, st>>>(a);
    else k_masks_from_dists<<<(unsigned)a.nTiles, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int dist_tile_rows() { return TM; }
int dist_tile_cols() { return TN; }

int launch_dist(const DistArgs& a, cudaStream_t st) {
    switch (a.dist) {
        case DIST_COSINE: return launch_dist_t<DIST_COSINE>(a, st);
        case DIST_L1: return launch_dist_t<DIST_L1>(a, st);
        case DIST_L2: return launch_dist_t<DIST_L2>(a, st);
        case DIST_CHI2: return launch_dist_t<DIST_CHI2>(a, st);
        case DIST_JS: return launch_dist_t<DIST_JS>(a, st);
    }
    return -1;
}

}  // namespace sdb
