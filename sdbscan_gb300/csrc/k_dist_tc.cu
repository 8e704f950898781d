// Stage 4, BF16 screening mode: candidate dot products on the tcgen05 tensor
// cores, with an exact FP32 re-decision of every pair near eps.
//
// Same grouped, gathered formulation as k_dist (tile = list l, 128 member
// rows, 64 candidate columns), with BF16 copies of the unit-norm rows as
// operands and FP32 accumulation in tensor memory.  Persistent and
// warp-specialised, one CTA per SM, 384 threads:
//   warps 0-1  gather the tile's 128 member rows (A), 64 dimensions per stage,
//              with cp.async into the 128-byte-swizzled K-major layout the MMA
//              reads (8-row x 128-byte atoms, 16-byte chunk c of row r at
//              chunk c ^ (r & 7)); each lane's copies arrive on the stage's
//              "full" mbarrier (cp.async.mbarrier.arrive.noinc) as they land;
//   warp 2     loads the list's 64 candidate rows (B) with one TMA tile load
//              (cp.async.bulk.tensor) per stage from the candidate matrix Cb,
//              the BF16 rows of every list's top-m points gathered once per
//              fit (k_gather_cand), completing bytes on the same barrier;
//   warp 3     issues tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = 64,
//              K = 16) into one of two 128 x 64 FP32 accumulators in tensor
//              memory and commits each stage back to its "empty" barrier, so
//              the loaders refill it while later stages compute;
//   warps 4-11 epilogue: tcgen05.ld of the other accumulator (warp w reads
//              TMEM lanes 32 (w % 4).. and one half of the 64 columns), the
//              eps decisions as bit words, the queue of pairs near eps, the
//              column counts; the eight warps work independently (each writes
//              its half of a row's mask word) and fetch the next tile's ids
//              while this tile's MMAs run.
// An 8-stage ring (24 KB per stage) runs ahead across tiles.  The CTA takes
// the launch order's tiles b, b + grid, ..., so the tiles in flight stay in
// one window of point chunks (L2 reuse of the gathered rows).
//
// Decision rule.  For unit vectors x, y and their BF16 roundings x', y'
// (relative error <= 2^-8 each), |x'.y' - x.y| <= (2^-7 + 2^-16) * sum|x_i y_i|
// <= 0.00783; FP32 accumulation of the exact products adds < 2^-10, and the
// FP32 reference's own rounding < 5e-5, 0.00886 in all.  A pair whose screened
// distance is farther than kMargin = 0.009 from eps is therefore on the same
// side of eps as the reference's FP32 distance; every other pair goes to a
// queue and is recomputed by k_recheck with the plain path's exact sequential
// FP32 dot.  The resulting masks are identical to the plain FP32 path's.
//
// L2 (single fits): the operands are split BF16 copies, x = hi + lo + r with
// |r| <= 2^-16 |x| elementwise; the member rows enter as [hi | lo | hi] and the
// candidate rows as [hi | hi | lo], so one K = 3 d GEMM gives
// hi.hi + lo.hi + hi.lo = x.y - e with |e| <= 3.02 * 2^-16 sum|x_i y_i|.  The
// screened squared distance nx + ny - 2 v (nx, ny: squared row norms in FP32)
// then differs from the reference's FP32 sum of squared differences by less
// than tolRel (nx + ny) + tolAbs, with tolRel covering the split, the
// tensor-core accumulation (K 2^-23), the norms (d 2^-23) and the FP32 updates,
// and tolAbs the reference's own rounding and its sqrt near eps
// (sum|x_i y_i| <= (nx + ny) / 2).  Pairs within that band of eps^2 are
// re-decided exactly, as for Cosine.
//
// Every wait on an mbarrier is bounded.  A wait that runs out stops every
// role (a shared abort flag) and raises the error flag, after which the plain
// FP32 kernel redoes the stage; before freeing its tensor memory the CTA waits
// for its own copies and MMAs.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dist_tile.cuh"
#include "tc_common.cuh"

namespace sdb {
namespace {

constexpr int TM = 128, TN = 64, TKB = 64;  // rows, candidate columns, bf16 per stage row (128 B)
constexpr int STAGES = 8;
constexpr int A_BYTES = TM * 128, B_BYTES = TN * 128, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int NT = 384, EPI0 = 4;               // warps 0-1 A, 2 B, 3 MMA, 4-11 epilogue
constexpr int A_LANES = 64;                     // threads gathering A
constexpr float kMargin = 0.009f;
constexpr uint32_t kTmemCols = 2 * TN;          // two accumulators
constexpr uint32_t kIdesc = tc::idesc_bf16(TM, TN);

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_arrive_noinc(uint32_t bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(bar) : "memory");
}
// Swizzled byte offset of 16-byte chunk c (0..7) of row r in an operand tile.
__device__ __forceinline__ uint32_t sw128(int r, int c) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

struct TileIds {
    int64_t mbeg, mend;
    int l, ct;
};
__device__ __forceinline__ TileIds tile_ids(const DistArgs& a, int64_t b) {
    const int64_t t = tile_at(a.tilePerm, b);
    TileIds r;
    r.l = a.tileList[t];
    const int64_t ti = t - a.tileOff[r.l];
    const int mt = (int)(ti / a.nct);
    r.ct = (int)(ti % a.nct);
    r.mbeg = a.listOff[r.l] + (int64_t)mt * TM;
    r.mend = a.listOff[r.l + 1];
    return r;
}

// SWEEP (Cosine): store the screened distance of every pair and queue the
// pairs near any of the sweep's eps values (masks follow per eps from the
// distances); otherwise decide against eps and write the masks.
template <int DIST, bool SWEEP>
__global__ void __launch_bounds__(NT, 1) k_dist_tc(const __grid_constant__ CUtensorMap tmC, DistArgs a,
                                                  const __nv_bfloat16* __restrict__ Xb, int ldb,
                                                  uint64_t* __restrict__ queue, int64_t qcap,
                                                  unsigned long long* __restrict__ qcount, int32_t* __restrict__ err,
                                                  float tolRel, float tolAbs) {
    static_assert(DIST == DIST_COSINE || (DIST == DIST_L2 && !SWEEP), "screened distances: Cosine, L2 fits");
    constexpr bool L2 = DIST == DIST_L2;
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ uint64_t fullA[STAGES], fullB[STAGES], emptyBar[STAGES], tfullBar[2], temptyBar[2], doneBar, neverBar;
    __shared__ uint32_t tmemBase;
    __shared__ int colPts[8][32];  // each epilogue warp's 32 column ids of its current tile
    __shared__ float colNrm[8][32];  // L2: their squared norms
    __shared__ volatile int abortFlag;
    __shared__ volatile long long bIssued, bUsed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t base = (tc::smem_u32(smraw) + 1023u) & ~1023u;  // 1024-aligned operand tiles
    const int nkb = ldb / TKB;              // stages per operand segment
    const int nk = (L2 ? 3 : 1) * nkb;      // L2: [hi | lo | hi] x [hi | hi | lo]
    const int ldx = (L2 ? 2 : 1) * ldb;     // row stride of Xb
    const int64_t total = *a.tileTotal;

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(tc::smem_u32(&fullA[s]), A_LANES);  // one noinc arrival per A lane
            tc::mbar_init(tc::smem_u32(&fullB[s]), 1);        // the B loader's expect_tx (+ the TMA bytes)
            tc::mbar_init(tc::smem_u32(&emptyBar[s]), 1);     // the MMA commit
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(tc::smem_u32(&tfullBar[b]), 1);
            tc::mbar_init(tc::smem_u32(&temptyBar[b]), 8);
        }
        tc::mbar_init(tc::smem_u32(&doneBar), 1);
        tc::mbar_init(tc::smem_u32(&neverBar), 1);  // the stall test's barrier: nothing arrives on it
        abortFlag = 0;
        bIssued = 0;
        bUsed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         tc::smem_u32(&tmemBase)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmemBase;
    auto stop = [&]() {
        abortFlag = 1;
        atomicExch(err, 1);
    };

    if (warp < 2) {
        // ---------------- A: member rows, gathered ----------------
        long long it = 0;
        for (int64_t b = blockIdx.x; b < total && !abortFlag; b += gridDim.x) {
            const TileIds ti = tile_ids(a, b);
            // copy u of this lane: chunk tid % 8 of row 8 u + tid / 8, so the
            // eight lanes of a row read its 128 contiguous bytes together
            const int c = tid & 7;
            const __nv_bfloat16* src[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int64_t q = ti.mbeg + 8 * u + (tid >> 3);
                src[u] = q < ti.mend ? Xb + (size_t)__ldg(&a.members[q].x) * ldx + c * 8 : nullptr;
            }
            bool bad = false;
            for (int kc = 0; kc < nk; ++kc, ++it) {
                const int s = (int)(it % STAGES);
                if (it >= STAGES && !tc::mbar_wait_or(tc::smem_u32(&emptyBar[s]),
                                                      (uint32_t)(((it / STAGES) - 1) & 1), &abortFlag)) {
                    bad = true;
                    break;
                }
                if (abortFlag) break;
                const uint32_t sA = base + s * STAGE_BYTES;
                const int ks = L2 && kc >= 2 * nkb ? kc - 2 * nkb : kc;  // the stage's source chunk of the row
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    const int row = 8 * u + (tid >> 3);
                    cp_async16(sA + sw128(row, c), src[u] != nullptr ? src[u] + ks * TKB : Xb, src[u] != nullptr);
                }
                cp_async_arrive_noinc(tc::smem_u32(&fullA[s]));
            }
            if (bad) {
                stop();
                break;
            }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
    } else if (warp == 2) {
        // ---------------- B: the list's candidate rows, one TMA tile per stage ----------------
        if (lane == 0) {
            long long it = 0;
            for (int64_t b = blockIdx.x; b < total && !abortFlag; b += gridDim.x) {
                const TileIds ti = tile_ids(a, b);
                const int y0 = (ti.l * a.nct + ti.ct) * TN;
                bool bad = false;
                for (int kc = 0; kc < nk; ++kc, ++it) {
                    const int s = (int)(it % STAGES);
                    if (it >= STAGES && !tc::mbar_wait_or(tc::smem_u32(&emptyBar[s]),
                                                          (uint32_t)(((it / STAGES) - 1) & 1), &abortFlag)) {
                        bad = true;
                        break;
                    }
                    if (abortFlag) break;
                    const uint32_t bar = tc::smem_u32(&fullB[s]);
                    tc::mbar_expect_tx(bar, B_BYTES);
                    tc::tma_load_2d(base + s * STAGE_BYTES + A_BYTES, &tmC, kc * TKB, y0, bar);
                    bIssued = it + 1;
                }
                if (bad) {
                    stop();
                    break;
                }
            }
        }
    } else if (warp == 3) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            long long it = 0;
            int i = 0;
            for (int64_t b = blockIdx.x; b < total && !abortFlag; b += gridDim.x, ++i) {
                const int buf = i & 1;
                if (i >= 2 && !tc::mbar_wait_or(tc::smem_u32(&temptyBar[buf]), (uint32_t)(((i >> 1) - 1) & 1),
                                                &abortFlag)) {
                    stop();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(buf * TN);
                // the stall test: a producer that never delivers, with copies and loads in flight
                bool bad = i == 0 && a.stallSpins > 0 && !tc::stall_wait(tc::smem_u32(&neverBar), a.stallSpins);
                for (int kc = 0; kc < nk && !bad; ++kc, ++it) {
                    const int s = (int)(it % STAGES);
                    if (!tc::mbar_wait_or(tc::smem_u32(&fullB[s]), (uint32_t)((it / STAGES) & 1), &abortFlag)) {
                        bad = true;
                        break;
                    }
                    bUsed = it + 1;
                    if (!tc::mbar_wait_or(tc::smem_u32(&fullA[s]), (uint32_t)((it / STAGES) & 1), &abortFlag)) {
                        bad = true;
                        break;
                    }
                    // cp.async writes to shared memory (generic proxy) before the MMA reads them (async proxy)
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t sA = base + s * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
                    for (int k = 0; k < TKB / 16; ++k)
                        tc::mma_bf16(acc, tc::smem_desc(sA + k * 32), tc::smem_desc(sB + k * 32), kIdesc,
                                     (kc > 0 || k > 0) ? 1u : 0u);
                    tc::mma_commit(tc::smem_u32(&emptyBar[s]));
                }
                if (bad) {
                    stop();
                    break;
                }
                tc::mma_commit(tc::smem_u32(&tfullBar[buf]));
            }
            tc::mma_commit(tc::smem_u32(&doneBar));  // arrives once every MMA issued above has completed
        }
    } else {
        // ---------------- epilogue: eight independent warps ----------------
        // Warp w reads TMEM lanes 32 (w % 4) .. + 31 (the tile's rows) and one
        // half of the 64 columns (w >= 8: the upper half); a thread owns one
        // row's 32 columns.  The next tile's ids are fetched while this tile's
        // MMAs run, and nothing is shared with the other epilogue warps.
        const int quarter = warp & 3, half = (warp - EPI0) >> 2;
        const int row = quarter * 32 + lane;  // TMEM lane = tile row
        int* colPt = colPts[warp - EPI0];
        float* colN = colNrm[warp - EPI0];
        long long myPairs = 0;
        auto fetch = [&](int64_t b, int& p, int& slot, int& cpt, TileIds& ti) {
            ti = tile_ids(a, b);
            const int64_t q = ti.mbeg + row;
            p = -1;
            slot = 0;
            if (q < ti.mend) {
                const int2 mm = a.members[q];
                p = mm.x;
                slot = mm.y;
            }
            const int side = ti.l / a.nproj, r = ti.l % a.nproj;
            const int c = ti.ct * TN + half * 32 + lane;
            cpt = c < a.m ? __ldg(a.topM + (size_t)r * 2 * a.m + side * a.m + c) : -1;
        };
        int nP = -1, nSlot = 0, nCol = -1;
        TileIds nTi{};
        if ((int64_t)blockIdx.x < total) fetch(blockIdx.x, nP, nSlot, nCol, nTi);
        int i = 0;
        for (int64_t b = blockIdx.x; b < total && !abortFlag; b += gridDim.x, ++i) {
            const int buf = i & 1;
            const int p = nP, mySlot = nSlot, ct = nTi.ct;
            __syncwarp();
            colPt[lane] = nCol;
            if constexpr (L2) colN[lane] = nCol >= 0 ? __ldg(a.sqNorm + nCol) : 0.0f;
            __syncwarp();
            const float nx = L2 && p >= 0 ? __ldg(a.sqNorm + p) : 0.0f;
            if (b + gridDim.x < total) fetch(b + gridDim.x, nP, nSlot, nCol, nTi);  // under this tile's MMAs
            if (!tc::mbar_wait_or(tc::smem_u32(&tfullBar[buf]), (uint32_t)((i >> 1) & 1), &abortFlag)) {
                stop();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t tacc =
                tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * TN + half * 32);
            const int cbase = ct * TN + half * 32;  // the tile's first column of this half, in list order
            if constexpr (SWEEP) {
#pragma unroll 1
                for (int c16 = 0; c16 < 2; ++c16) {
                    float v[16];
                    tc::tmem_ld16(tacc + (uint32_t)(c16 * 16), v);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int col = c16 * 16 + j;  // within the half
                        const int qq = colPt[col];
                        bool unsure = false;
                        if (p >= 0 && qq >= 0) {  // keep the screened distance, re-decide near any eps
                            const float dist = 1.0f - v[j];
                            a.dists[((size_t)p * 2 * a.k + mySlot) * a.m + cbase + col] = dist;
                            if (p != qq)
                                for (int e = 0; e < a.nSweep; ++e) unsure |= fabsf(dist - a.sweepEps[e]) <= kMargin;
                        }
                        const unsigned um = __ballot_sync(0xffffffffu, unsure);
                        if (um) {
                            const int leader = __ffs(um) - 1;
                            unsigned long long at0 = 0;
                            if (lane == leader) at0 = atomicAdd(qcount, (unsigned long long)__popc(um));
                            at0 = __shfl_sync(0xffffffffu, at0, leader);
                            if (unsure) {
                                const unsigned long long at = at0 + __popc(um & ((1u << lane) - 1u));
                                if ((int64_t)at < qcap)
                                    queue[at] = ((uint64_t)(uint32_t)p << 32) | ((uint32_t)mySlot << 16) |
                                                (uint32_t)(cbase + col);
                                else
                                    atomicExch(err, 2);
                            }
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(tc::smem_u32(&temptyBar[buf]));
            } else {
                // The row's 32 decisions as bit words: pass (screened distance
                // below eps - margin), unsure (within the margin), near zero (the
                // only place the point itself can be among the candidates); then
                // the columns that do not exist, the row's own point and empty
                // rows are masked out.
                uint32_t bits = 0, uw = 0, zw = 0;
#pragma unroll
                for (int c16 = 0; c16 < 2; ++c16) {
                    float v[16];
                    tc::tmem_ld16(tacc + (uint32_t)(c16 * 16), v);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        bool pass, near, zero;
                        if constexpr (L2) {
                            // squared distances against eps^2, within a per-pair band
                            const float ny = colN[c16 * 16 + j];
                            const float d2 = nx + ny - 2.0f * v[j];
                            const float tol = tolRel * (nx + ny) + tolAbs;
                            const float e2 = a.eps * a.eps;
                            pass = d2 <= e2 - tol;
                            near = d2 <= e2 + tol;
                            zero = d2 <= tol;
                        } else {
                            const float dist = 1.0f - v[j];
                            pass = dist <= a.eps - kMargin;
                            near = dist <= a.eps + kMargin;
                            zero = dist <= kMargin;
                        }
                        bits |= (uint32_t)pass << (c16 * 16 + j);
                        uw |= (uint32_t)(!pass && near) << (c16 * 16 + j);
                        zw |= (uint32_t)zero << (c16 * 16 + j);
                    }
                }
                // the accumulator is in registers: the MMAs may reuse it
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(tc::smem_u32(&temptyBar[buf]));
                const int nvalid = a.m - cbase;
                uint32_t keep = p < 0 || nvalid <= 0 ? 0u : (nvalid >= 32 ? ~0u : (1u << nvalid) - 1u);
                for (uint32_t z = zw & keep & (bits | uw); z; z &= z - 1) {  // rare: is the row's point a candidate?
                    const int col = __ffs(z) - 1;
                    if (colPt[col] == p) keep &= ~(1u << col);
                }
                bits &= keep;
                uw &= keep;
                if (__any_sync(0xffffffffu, uw != 0)) {  // pairs within the margin go to the queue
                    const int cnt = __popc(uw);
                    if (cnt) {
                        unsigned long long at = atomicAdd(qcount, (unsigned long long)cnt);
                        for (uint32_t u = uw; u; u &= u - 1, ++at) {
                            const int col = __ffs(u) - 1;
                            if ((int64_t)at < qcap)
                                queue[at] = ((uint64_t)(uint32_t)p << 32) | ((uint32_t)mySlot << 16) |
                                            (uint32_t)(cbase + col);
                            else
                                atomicExch(err, 2);
                        }
                    }
                }
                // this half of the row's 64-bit mask word (little endian: columns 0-31 low)
                if (p >= 0)
                    reinterpret_cast<uint32_t*>(a.masks)[(((size_t)p * 2 * a.k + mySlot) * a.W + ct) * 2 + half] = bits;
                myPairs += __popc(bits);
                int cc = 0;  // passes of column `lane` of this half over the warp's 32 rows
#pragma unroll
                for (int col = 0; col < 32; ++col) {
                    const int pc = __popc(__ballot_sync(0xffffffffu, (bits >> col) & 1u));
                    if (lane == col) cc = pc;
                }
                if (cc) atomicAdd(a.inRaw + colPt[lane], cc);
            }
        }
        const int wp = warp_sum((int)myPairs);
        if (lane == 0 && wp) atomicAdd(a.pairs, (unsigned long long)wp);
    }
    __syncthreads();
    if (tid == 0) {
        // a stopped CTA may still have TMA loads in flight into its shared memory
        for (long long it = bUsed; it < bIssued; ++it)
            tc::mbar_wait(tc::smem_u32(&fullB[it % STAGES]), (uint32_t)((it / STAGES) & 1));
        if (!tc::mbar_wait(tc::smem_u32(&doneBar), 0u)) atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// Cb: the BF16 rows of every list's candidates, list-major, nct * 64 rows per
// list (row ct * 64 + j = candidate ct * 64 + j of the list, zero past m), the
// B operand of k_dist_tc as plain tiles.  Cosine: rows of Xb (ldb wide); L2:
// [hi | hi | lo] from the split rows [hi | lo] of Xb (3 ldb wide).
__global__ void k_gather_cand(const DistArgs a, const __nv_bfloat16* __restrict__ Xb, int ldb, int segs,
                              __nv_bfloat16* __restrict__ Cb) {
    const int rowsPerList = a.nct * TN, ldc = segs * ldb, per = ldc / 8;
    const int ldx = segs == 3 ? 2 * ldb : ldb;
    const size_t total = (size_t)2 * a.nproj * rowsPerList * per;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / per;
        const int c8 = (int)(i % per) * 8;
        const int seg = c8 / ldb, off = c8 % ldb;
        const int srcCol = (segs == 3 && seg == 2 ? ldb : 0) + off;  // segments 0, 1: hi; 2: lo
        const int l = (int)(row / rowsPerList), j = (int)(row % rowsPerList);
        const int r = l % a.nproj, side = l / a.nproj;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (j < a.m) {
            const int q = __ldg(a.topM + (size_t)r * 2 * a.m + side * a.m + j);
            v = __ldg(reinterpret_cast<const uint4*>(Xb + (size_t)q * ldx + srcCol));
        }
        *reinterpret_cast<uint4*>(Cb + row * ldc + c8) = v;
    }
}

// Squared norm of each row of Xt: a warp per row, 16-byte loads.
__global__ void k_sq_norms(const float* __restrict__ Xt, int ld, int n, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += warps) {
        const float4* x = reinterpret_cast<const float4*>(Xt + (size_t)p * ld);
        float s = 0.0f;
        for (int c = lane; c < ld / 4; c += 32) {
            const float4 v = __ldg(x + c);
            s = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, s))));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[p] = s;
    }
}

// Exact re-decision of the queued pairs: a warp takes 32 queue entries, one
// per lane, and computes their distances with the plain path's sequential
// FP32 arithmetic (dtile::warp_staged), so the decision equals k_dist's.
constexpr int RC_WARPS = 4;

template <int DIST>
__global__ void __launch_bounds__(RC_WARPS * 32) k_recheck(DistArgs a, const uint64_t* __restrict__ queue,
                                                           const unsigned long long* __restrict__ qcount,
                                                           int64_t qcap) {
    __shared__ float tile[RC_WARPS][64][33];  // rows 0..31: the pairs' points, 32..63: their candidates
    __shared__ const float* rows[RC_WARPS][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nq = (int64_t)min((unsigned long long)qcap, *qcount);
    const int64_t warpsTotal = (int64_t)gridDim.x * RC_WARPS;
    for (int64_t base = ((int64_t)blockIdx.x * RC_WARPS + w) * 32; base < nq; base += warpsTotal * 32) {
        const int64_t e = base + lane;
        const bool valid = e < nq;
        int p = 0, q = 0, slot = 0, col = 0;
        if (valid) {
            const uint64_t v = queue[e];
            p = (int)(v >> 32);
            slot = (int)((v >> 16) & 0xFFFF);
            col = (int)(v & 0xFFFF);
            const int r = __ldg(a.topKmat + (size_t)p * 2 * a.k + slot);
            const int side = slot >= a.k;
            q = __ldg(a.topM + (size_t)r * 2 * a.m + side * a.m + col);
        }
        rows[w][lane] = a.Xt + (size_t)p * a.ld;
        rows[w][32 + lane] = a.Xt + (size_t)q * a.ld;
        __syncwarp();
        const float dist = dtile::warp_staged<DIST>(rows[w], tile[w], a.ld);
        if (a.dists != nullptr) {  // eps sweep: store the exact distance; masks follow per eps
            if (valid) a.dists[((size_t)p * 2 * a.k + slot) * a.m + col] = dist;
            __syncwarp();
            continue;
        }
        const bool pass = valid && dist <= a.eps;
        if (pass) {
            atomicOr(reinterpret_cast<unsigned long long*>(a.masks) + ((size_t)p * 2 * a.k + slot) * a.W + col / 64,
                     1ull << (col % 64));
            atomicAdd(a.inRaw + q, 1);
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        if (lane == 0 && pm) atomicAdd(a.pairs, (unsigned long long)__popc(pm));
        __syncwarp();
    }
}

// When screening failed (queue overflow or a timed-out wait) the plain path
// redoes the stage: clear what the screening counted.
__global__ void k_screen_reset(DistArgs a) {
    if (__ldg(a.gate) == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) a.inRaw[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.pairs = 0;
}

// Xt (FP32, row stride ld) -> Xb (BF16, row stride ldb, zero padded).
__global__ void k_to_bf16(const float* __restrict__ Xt, int ld, int n, __nv_bfloat16* __restrict__ Xb, int ldb) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = (size_t)ldb / 8;
    if (q >= (size_t)n * per) return;
    const int p = (int)(q / per), c0 = (int)(q % per) * 8;
    __align__(16) __nv_bfloat16 out[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int c = c0 + i;
        out[i] = __float2bfloat16_rn(c < ld ? Xt[(size_t)p * ld + c] : 0.0f);
    }
    *reinterpret_cast<uint4*>(Xb + (size_t)p * ldb + c0) = *reinterpret_cast<const uint4*>(out);
}

// Xt (FP32, row stride ld) -> [hi | lo] BF16 halves per row (row stride
// 2 ldb): hi = bf16(x), lo = bf16(x - hi), both zero past ld.
__global__ void k_to_bf16_split(const float* __restrict__ Xt, int ld, int n, __nv_bfloat16* __restrict__ Xs, int ldb) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = (size_t)ldb / 8;
    if (q >= (size_t)n * per) return;
    const int p = (int)(q / per), c0 = (int)(q % per) * 8;
    __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int c = c0 + i;
        const float x = c < ld ? Xt[(size_t)p * ld + c] : 0.0f;
        hi[i] = __float2bfloat16_rn(x);
        lo[i] = __float2bfloat16_rn(x - __bfloat162float(hi[i]));
    }
    *reinterpret_cast<uint4*>(Xs + (size_t)p * 2 * ldb + c0) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(Xs + (size_t)p * 2 * ldb + ldb + c0) = *reinterpret_cast<const uint4*>(lo);
}

}  // namespace

int launch_to_bf16_split(const float* Xt, int ld, int n, void* Xs, int ldb, cudaStream_t st) {
    const size_t total = (size_t)n * (ldb / 8);
    k_to_bf16_split<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(Xt, ld, n, static_cast<__nv_bfloat16*>(Xs), ldb);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_to_bf16(const float* Xt, int ld, int n, void* Xb, int ldb, cudaStream_t st) {
    const size_t total = (size_t)n * (ldb / 8);
    k_to_bf16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(Xt, ld, n, static_cast<__nv_bfloat16*>(Xb), ldb);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

static int cand_segs(const DistArgs& a) { return a.dist == DIST_L2 ? 3 : 1; }

size_t dist_tc_cand_bytes(const DistArgs& a, int ldb) {
    return sizeof(uint16_t) * (size_t)2 * a.nproj * a.nct * TN * cand_segs(a) * ldb;
}

int launch_dist_tc(const DistArgs& a, const void* Xb, int ldb, void* Cb, uint64_t* queue, int64_t qcap,
                   unsigned long long* qcount, int32_t* err, cudaStream_t st) {
    if (ldb % TKB != 0 || (reinterpret_cast<uintptr_t>(Xb) & 15) || (reinterpret_cast<uintptr_t>(Cb) & 15)) return -1;
    if (a.dist != DIST_COSINE && !(a.dist == DIST_L2 && a.dists == nullptr && a.sqNorm != nullptr)) return -1;
    const int segs = cand_segs(a);
    const int rows = 2 * a.nproj * a.nct * TN;
    k_gather_cand<<<sm_count() * 8, 256, 0, st>>>(a, static_cast<const __nv_bfloat16*>(Xb), ldb, segs,
                                                  static_cast<__nv_bfloat16*>(Cb));
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    CUtensorMap tmC;
    if (!tc::encode_bf16_2d(&tmC, Cb, rows, segs * ldb, TKB, TN)) return -1;
    const size_t sm = (size_t)STAGES * STAGE_BYTES + 1024;
    auto kern = a.dist == DIST_L2 ? k_dist_tc<DIST_L2, false>
                                  : (a.dists != nullptr ? k_dist_tc<DIST_COSINE, true> : k_dist_tc<DIST_COSINE, false>);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    // L2 band (see the decision rule above): split error, tensor-core
    // accumulation over K = 3 ldb, the FP32 norms over ld, the FP32 updates;
    // then the reference's own sum of squares and its sqrt at eps
    float tolRel = 0.0f, tolAbs = 0.0f;
    if (a.dist == DIST_L2) {
        const double u23 = std::ldexp(1.0, -23);
        tolRel = (float)(3.1 * std::ldexp(1.0, -16) + (3.0 * ldb + a.ld) * u23 + 4.0 * u23);
        tolAbs = (float)(((double)a.ld * u23 + 8.0 * u23) * (double)a.eps * a.eps * 1.01 + 1e-30);
    }
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(a.nTiles, (int64_t)sm_count()));
    kern<<<grid, NT, sm, st>>>(tmC, a, static_cast<const __nv_bfloat16*>(Xb), ldb, queue, qcap, qcount, err, tolRel,
                               tolAbs);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

int launch_sq_norms(const float* Xt, int ld, int n, float* out, cudaStream_t st) {
    if (n <= 0) return 0;
    if ((ld & 3) || (reinterpret_cast<uintptr_t>(Xt) & 15)) return -1;
    const int grid = (int)std::min<int64_t>(((int64_t)n + 7) / 8, (int64_t)sm_count() * 16);
    k_sq_norms<<<grid, 256, 0, st>>>(Xt, ld, n, out);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_screen_reset(const DistArgs& a, cudaStream_t st) {
    k_screen_reset<<<sm_count() * 4, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_recheck(const DistArgs& a, const uint64_t* queue, const unsigned long long* qcount, int64_t qcap,
                   cudaStream_t st) {
    if (a.dist == DIST_L2) k_recheck<DIST_L2><<<sm_count() * 8, RC_WARPS * 32, 0, st>>>(a, queue, qcount, qcap);
    else k_recheck<DIST_COSINE><<<sm_count() * 8, RC_WARPS * 32, 0, st>>>(a, queue, qcount, qcap);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int dist_tc_tile_rows() { return TM; }

}  // namespace sdb
