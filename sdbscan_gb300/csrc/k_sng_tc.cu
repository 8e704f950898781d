// sngDbscan, BF16 screening mode (Cosine): the dense block of dot products
// (every point x every distinct sampled point) on the tcgen05 tensor cores,
// with an exact FP32 re-decision of every pair near eps.  The decision rule
// is the candidate stage's (k_dist_tc.cu): for unit vectors the BF16 dot errs
// by at most 0.00886 from the reference's FP32 dot, so a pair whose screened
// distance is farther than kMargin = 0.009 from eps is on the reference's side
// of eps; every other pair is queued and recomputed by k_sng_recheck with the
// plain path's sequential FP32 dot.  Masks, row degrees and column counts are
// then identical to the FP32 block's (k_sng_block).
//
// Tile: 128 points x 256 sampled points, K in chunks of 64 BF16 (one 128-byte
// swizzle atom per row, written by TMA and read by the MMA's smem descriptor).
// Persistent and warp-specialised, one CTA per SM:
//   warp 0   TMA producer: a 4-stage ring (48 KB per stage) of A (point rows)
//            and B (sampled rows) chunks, running ahead across tiles;
//   warp 1   MMA issuer: tcgen05.mma.cta_group::1.kind::f16 (M = 128,
//            N = 256, K = 16) into one of two 128 x 256 FP32 accumulators in
//            tensor memory (all 512 columns), so one tile's MMAs run under
//            the previous tile's epilogue;
//   warps 2-9 epilogue: tcgen05.ld of the accumulator (two warps per 32-lane
//            quarter, one half of the columns each), the eps decision, pass
//            bits, row degrees, queued pairs; column counts are summed in
//            shared memory and flushed once per tile.
// The 256 columns of a tile are four 64-bit pass-bit words of the block's
// tile-major mask.  Tile t covers row block t / nbt and column tile t % nbt,
// so the CTAs in flight share a few row blocks in L2 and the sampled rows
// (nU x d BF16) stay L2-resident.
//
// Every wait is bounded (mbarriers only, no named barriers).  A timed-out
// wait stops all roles (a shared abort flag) and raises the gate flag; the
// CTA then waits for the TMA loads it issued and for its MMAs before freeing
// tensor memory.  A full queue also raises the flag.  With the flag raised
// the host runs the FP32 block after k_sng_reset has cleared the counts (the
// FP32 block rewrites every mask word).
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "dist_tile.cuh"
#include "tc_common.cuh"

#include <algorithm>

namespace sdb {
namespace {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4;
constexpr int EPI_WARPS = 8, NT = 64 + EPI_WARPS * 32;  // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;  // 16 KB + 32 KB
constexpr uint32_t kTmemCols = 2 * BN;  // two accumulators
constexpr uint32_t kIdesc = tc::idesc_bf16(BM, BN);
constexpr float kMargin = 0.009f;

__global__ void __launch_bounds__(NT, 1) k_sng_tc(const __grid_constant__ CUtensorMap tmX,
                                                 const __grid_constant__ CUtensorMap tmU, SngArgs a, int nk, int nbt,
                                                 int64_t tiles, uint64_t* __restrict__ queue, int64_t qcap,
                                                 unsigned long long* __restrict__ qcount, int32_t* __restrict__ gate) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ uint64_t fullBar[STAGES], emptyBar[STAGES], tfullBar[2], temptyBar[2], epiBar[2], doneBar, neverBar;
    __shared__ uint32_t tmemBase;
    __shared__ int colCount[2][BN];
    __shared__ volatile int abortFlag;
    __shared__ volatile long long loadsIssued, loadsUsed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t base = (tc::smem_u32(smraw) + 1023u) & ~1023u;  // 1024-aligned operand tiles

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(tc::smem_u32(&fullBar[s]), 1);
            tc::mbar_init(tc::smem_u32(&emptyBar[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(tc::smem_u32(&tfullBar[b]), 1);
            tc::mbar_init(tc::smem_u32(&temptyBar[b]), EPI_WARPS);
            tc::mbar_init(tc::smem_u32(&epiBar[b]), EPI_WARPS);
        }
        tc::mbar_init(tc::smem_u32(&doneBar), 1);
        tc::mbar_init(tc::smem_u32(&neverBar), 1);  // the stall test's barrier: nothing arrives on it
        abortFlag = 0;
        loadsIssued = 0;
        loadsUsed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (int i = tid; i < 2 * BN; i += NT) colCount[i / BN][i % BN] = 0;
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
        atomicExch(gate, 1);
    };

    if (warp == 0) {
        if (lane == 0) {  // TMA producer
            long long it = 0;
            for (int64_t t = blockIdx.x; t < tiles && !abortFlag; t += gridDim.x) {
                const int m0 = (int)(t / nbt) * BM, n0 = (int)(t % nbt) * BN;
                for (int kc = 0; kc < nk; ++kc, ++it) {
                    const int s = (int)(it % STAGES);
                    if (it >= STAGES && !tc::mbar_wait_or(tc::smem_u32(&emptyBar[s]),
                                                          (uint32_t)(((it / STAGES) - 1) & 1), &abortFlag)) {
                        stop();
                        break;
                    }
                    if (abortFlag) break;
                    const uint32_t sA = base + s * STAGE_BYTES, sB = sA + A_BYTES, bar = tc::smem_u32(&fullBar[s]);
                    tc::mbar_expect_tx(bar, STAGE_BYTES);
                    tc::tma_load_2d(sA, &tmX, kc * BK, m0, bar);
                    tc::tma_load_2d(sB, &tmU, kc * BK, n0, bar);
                    loadsIssued = it + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            long long it = 0;
            int i = 0;
            for (int64_t t = blockIdx.x; t < tiles && !abortFlag; t += gridDim.x, ++i) {
                const int buf = i & 1;
                if (i >= 2 && !tc::mbar_wait_or(tc::smem_u32(&temptyBar[buf]), (uint32_t)(((i >> 1) - 1) & 1),
                                                &abortFlag)) {
                    stop();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(buf * BN);
                // the stall test: a producer that never delivers, with loads in flight
                bool bad = i == 0 && a.stallSpins > 0 && !tc::stall_wait(tc::smem_u32(&neverBar), a.stallSpins);
                for (int kc = 0; kc < nk && !bad; ++kc, ++it) {
                    const int s = (int)(it % STAGES);
                    if (!tc::mbar_wait_or(tc::smem_u32(&fullBar[s]), (uint32_t)((it / STAGES) & 1), &abortFlag)) {
                        bad = true;
                        break;
                    }
                    loadsUsed = it + 1;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t sA = base + s * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k)
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
    } else {  // epilogue warps
        const int ew = warp - 2, quarter = warp & 3, half = ew >> 2;
        int i = 0;
        for (int64_t t = blockIdx.x; t < tiles && !abortFlag; t += gridDim.x, ++i) {
            const int buf = i & 1;
            const int m0 = (int)(t / nbt) * BM, n0 = (int)(t % nbt) * BN, bt = (int)(t % nbt);
            if (!tc::mbar_wait_or(tc::smem_u32(&tfullBar[buf]), (uint32_t)((i >> 1) & 1), &abortFlag)) {
                stop();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int row = m0 + quarter * 32 + lane;
            const bool rv = row < a.n;
            const int selfc = rv ? __ldg(a.colOf + row) : -1;  // the row's own column (if sampled)
            const float lo = a.eps - kMargin, hi = a.eps + kMargin;
            int cc[4] = {0, 0, 0, 0};  // column counts of lane + 32 s (s < 4) within the half
            int wsum = 0, nPass = 0;
#pragma unroll
            for (int wdi = 0; wdi < 2; ++wdi) {  // the half's two 64-column words
                const int cbase = n0 + half * 128 + wdi * 64;
                uint64_t pw = 0, uw = 0;
#pragma unroll
                for (int c16 = 0; c16 < 4; ++c16) {
                    float v[16];
                    tc::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) +
                                      (uint32_t)(buf * BN + half * 128 + wdi * 64 + c16 * 16),
                                  v);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float dist = 1.0f - v[j];
                        const bool p = dist <= lo;
                        pw |= (uint64_t)p << (c16 * 16 + j);
                        uw |= (uint64_t)(!p && dist <= hi) << (c16 * 16 + j);
                    }
                }
                // valid columns of the word, not the row's own point, real rows only
                const int nvalid = a.nU - cbase;
                uint64_t keep = nvalid >= 64 ? ~0ull : (nvalid > 0 ? (1ull << nvalid) - 1ull : 0ull);
                if (selfc >= cbase && selfc < cbase + 64) keep &= ~(1ull << (selfc - cbase));
                if (!rv) keep = 0;
                pw &= keep;
                uw &= keep;
                if (__any_sync(0xffffffffu, uw != 0)) {  // rare: pairs within the margin go to the queue
                    const int cnt = __popcll(uw);
                    if (cnt) {
                        unsigned long long at = atomicAdd(qcount, (unsigned long long)cnt);
                        for (uint64_t u = uw; u; u &= u - 1, ++at) {
                            const int c = cbase + __ffsll((long long)u) - 1;
                            if ((int64_t)at < qcap) queue[at] = ((uint64_t)(uint32_t)row << 32) | (uint32_t)c;
                            else atomicExch(gate, 2);
                        }
                    }
                }
                if (rv) {
                    const int wd = bt * 4 + half * 2 + wdi;
                    if (wd < a.nct) a.mask[(size_t)wd * a.n + row] = pw;
                }
                const int np = __popcll(pw);
                nPass += np;
                wsum += np;
                const uint64_t heavy = a.heavy != nullptr && cbase < a.nU ? __ldg(a.heavy + (cbase >> 6)) : 0ull;
                for (uint64_t hb = pw & heavy; hb; hb &= hb - 1)  // columns drawn more than once
                    wsum += __ldg(a.mult + cbase + __ffsll((long long)hb) - 1) - 1;
#pragma unroll
                for (int bit = 0; bit < 64; ++bit) {
                    const int pc = __popc(__ballot_sync(0xffffffffu, (pw >> bit) & 1ull));
                    if (lane == ((wdi * 64 + bit) & 31)) cc[(wdi * 64 + bit) >> 5] += pc;
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            if (wsum) atomicAdd(a.rowDeg + row, wsum);
#pragma unroll
            for (int s2 = 0; s2 < 4; ++s2)
                if (cc[s2]) atomicAdd(&colCount[buf][half * 128 + s2 * 32 + lane], cc[s2]);
            const int wp = warp_sum(nPass);
            if (lane == 0 && wp) atomicAdd(a.pairs, (unsigned long long)wp);
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&epiBar[buf]));
            if (ew == 0) {  // every epilogue warp is done with this tile: flush its column counts
                if (!tc::mbar_wait_or(tc::smem_u32(&epiBar[buf]), (uint32_t)((i >> 1) & 1), &abortFlag)) {
                    stop();
                    break;
                }
                for (int j = lane; j < BN; j += 32) {
                    const int cnt = colCount[buf][j];
                    if (cnt) {
                        atomicAdd(a.colCnt + n0 + j, cnt);
                        colCount[buf][j] = 0;
                    }
                }
                __syncwarp();
            }
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&temptyBar[buf]));  // the accumulator may be reused
        }
    }
    __syncthreads();
    if (tid == 0) {
        // a stopped CTA still has TMA loads in flight into its shared memory
        for (long long it = loadsUsed; it < loadsIssued; ++it)
            tc::mbar_wait(tc::smem_u32(&fullBar[it % STAGES]), (uint32_t)((it / STAGES) & 1));
        if (!tc::mbar_wait(tc::smem_u32(&doneBar), 0u)) atomicExch(gate, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// Exact re-decision of the queued (point, column) pairs: a warp takes 32
// entries, one per lane, with the plain path's sequential FP32 dot.
constexpr int RC_WARPS = 4;

__global__ void __launch_bounds__(RC_WARPS * 32) k_sng_recheck(SngArgs a, const uint64_t* __restrict__ queue,
                                                               const unsigned long long* __restrict__ qcount,
                                                               int64_t qcap, const int32_t* __restrict__ gate) {
    __shared__ float tile[RC_WARPS][64][33];  // rows 0..31: the pairs' points, 32..63: their sampled points
    __shared__ const float* rows[RC_WARPS][64];
    if (*gate) return;  // the screening failed: the FP32 block redoes the stage
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nq = (int64_t)min((unsigned long long)qcap, *qcount);
    const int64_t warpsTotal = (int64_t)gridDim.x * RC_WARPS;
    for (int64_t b0 = ((int64_t)blockIdx.x * RC_WARPS + w) * 32; b0 < nq; b0 += warpsTotal * 32) {
        const int64_t e = b0 + lane;
        const bool valid = e < nq;
        int p = 0, c = 0, q = 0;
        if (valid) {
            const uint64_t v = queue[e];
            p = (int)(v >> 32);
            c = (int)(uint32_t)v;
            q = __ldg(a.cols + c);
        }
        rows[w][lane] = a.Xt + (size_t)p * a.ld;
        rows[w][32 + lane] = a.Xt + (size_t)q * a.ld;
        __syncwarp();
        const float dist = dtile::warp_staged_cosine(rows[w], tile[w], a.ld);
        const bool pass = valid && p != q && dist <= a.eps;
        if (pass) {
            atomicOr(reinterpret_cast<unsigned long long*>(a.mask) + (size_t)(c >> 6) * a.n + p, 1ull << (c & 63));
            atomicAdd(a.rowDeg + p, a.mult != nullptr ? __ldg(a.mult + c) : 1);
            atomicAdd(a.colCnt + c, 1);
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        if (lane == 0 && pm) atomicAdd(a.pairs, (unsigned long long)__popc(pm));
        __syncwarp();
    }
}

// When the screening failed: clear what it counted (the FP32 block follows).
__global__ void k_sng_reset(SngArgs a, const int32_t* __restrict__ gate) {
    if (__ldg(gate) == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        a.rowDeg[i] = 0;
        if (i < a.nU) a.colCnt[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.pairs = 0;
}

// Ub[c] = bf16 of the sampled point's transformed row (zero padded to ldb).
__global__ void k_sng_gather_bf16(const float* __restrict__ Xt, int ld, const int32_t* __restrict__ cols, int nU,
                                  __nv_bfloat16* __restrict__ Ub, int ldb) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = (size_t)ldb / 8;
    if (q >= (size_t)nU * per) return;
    const int c = (int)(q / per), e0 = (int)(q % per) * 8;
    const float* x = Xt + (size_t)__ldg(cols + c) * ld;
    __align__(16) __nv_bfloat16 out[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = __float2bfloat16_rn(e0 + i < ld ? x[e0 + i] : 0.0f);
    *reinterpret_cast<uint4*>(Ub + (size_t)c * ldb + e0) = *reinterpret_cast<const uint4*>(out);
}

}  // namespace

int launch_sng_gather_bf16(const SngArgs& a, void* Ub, int ldb, cudaStream_t st) {
    if (a.nU <= 0) return 0;
    const size_t total = (size_t)a.nU * (ldb / 8);
    k_sng_gather_bf16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a.Xt, a.ld, a.cols, a.nU,
                                                                      static_cast<__nv_bfloat16*>(Ub), ldb);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_sng_tc(const SngArgs& a, const void* Xb, const void* Ub, int ldb, uint64_t* queue, int64_t qcap,
                  unsigned long long* qcount, int32_t* gate, cudaStream_t st) {
    if (a.nU <= 0) return 0;
    if (ldb % BK != 0 || (reinterpret_cast<uintptr_t>(Xb) & 15) || (reinterpret_cast<uintptr_t>(Ub) & 15)) return -1;
    CUtensorMap tmX, tmU;
    if (!tc::encode_bf16_2d(&tmX, Xb, a.n, ldb, BK, BM) || !tc::encode_bf16_2d(&tmU, Ub, a.nU, ldb, BK, BN))
        return -1;
    const size_t sm = (size_t)STAGES * STAGE_BYTES + 1024;
    if (cudaFuncSetAttribute(k_sng_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    const int nbt = (a.nU + BN - 1) / BN;
    const int64_t tiles = (int64_t)((a.n + BM - 1) / BM) * nbt;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sm_count());
    k_sng_tc<<<grid, NT, sm, st>>>(tmX, tmU, a, ldb / BK, nbt, tiles, queue, qcap, qcount, gate);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    k_sng_recheck<<<sm_count() * 8, RC_WARPS * 32, 0, st>>>(a, queue, qcount, qcap, gate);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    k_sng_reset<<<sm_count() * 4, 256, 0, st>>>(a, gate);
    return cudaPeekAtLastError() == cudaSuccess ? 3 : -1;
}

}  // namespace sdb
