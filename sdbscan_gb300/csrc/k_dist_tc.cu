// Stage 4, BF16 screening mode: candidate dot products on the tcgen05 tensor
// cores, with an exact FP32 re-decision of every pair near eps.
//
// Same grouped, gathered formulation as k_dist (tile = list l, 128 member rows,
// 64 candidate columns), but the operands are BF16 copies of the unit-norm
// rows and the products accumulate in FP32 in tensor memory:
//   - operands are staged by cp.async into shared memory in the 128-byte
//     swizzled K-major layout the MMA reads (8-row x 128-byte atoms, 16-byte
//     chunk c of row r stored at chunk c ^ (r & 7)), 3 stages of 64 dimensions
//     (73 KB, so three CTAs share an SM);
//   - one thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=64,
//     K=16) into a 128 x 64 FP32 accumulator in TMEM, and tcgen05.commit
//     arrives on the stage's mbarrier when the MMAs have read it;
//   - the epilogue reads the accumulator with tcgen05.ld (thread t = row t).
//
// Decision rule.  For unit vectors x, y and their BF16 roundings x', y'
// (relative error <= 2^-8 each), |x'.y' - x.y| <= (2^-7 + 2^-16) * sum|x_i y_i|
// <= 0.00783; FP32 accumulation of 784 exact products adds < 2^-10, and the
// FP32 reference's own rounding < 5e-5, 0.00886 in all.  A pair whose screened
// distance is farther than kMargin = 0.009 from eps is therefore on the same
// side of eps as the reference's FP32 distance; every other pair goes to a
// queue and is recomputed by k_recheck with the plain path's exact sequential
// FP32 dot.  The resulting masks are identical to the plain FP32 path's.
//
// Every wait on an mbarrier is bounded; on timeout the CTA records an error,
// stops issuing work, drains its own copies, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "common.cuh"
#include "dist_tile.cuh"
#include "tc_common.cuh"

namespace sdb {
namespace {

constexpr int TM = 128, TN = 64, TKB = 64;  // rows, candidate columns, bf16 per stage row (128 B)
constexpr int STAGES = 3, NT = 128;
constexpr int A_BYTES = TM * 128, B_BYTES = TN * 128, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr float kMargin = 0.009f;
constexpr uint32_t kTmemCols = 64;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}

using tc::mbar_init;
using tc::mbar_wait;
using tc::smem_desc;
using tc::smem_u32;
using tc::tmem_ld16;
using tc::mma_commit;

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = 64.
constexpr uint32_t kIdesc = tc::idesc_bf16(TM, TN);

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    tc::mma_bf16(dtmem, adesc, bdesc, kIdesc, accumulate);
}

// Swizzled byte offset of 16-byte chunk c (0..7) of row r in an operand tile.
__device__ __forceinline__ uint32_t sw128(int r, int c) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// SWEEP: store the screened distance of every pair and queue the pairs near
// any of the sweep's eps values (masks follow per eps from the distances);
// otherwise decide against eps and write the masks.
template <bool SWEEP>
__global__ void __launch_bounds__(NT, 3) k_dist_tc(DistArgs a, const __nv_bfloat16* __restrict__ Xb, int ldb,
                                                  uint64_t* __restrict__ queue, int64_t qcap,
                                                  unsigned long long* __restrict__ qcount, int32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ uint64_t bars[STAGES];
    __shared__ uint32_t tmemBase;
    // tile ids: the next tile's are loaded under this tile's epilogue, which
    // by then holds its own row's ids in registers (column ids by tile
    // parity); kept small so three CTAs still share an SM's shared memory
    __shared__ int rowPoints[TM], colPoints[2][TN], colCount[TN];
    __shared__ uint8_t rowSlots[TM];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t base = (smem_u32(smraw) + 1023u) & ~1023u;  // 1024-aligned operand tiles

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmemBase)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmemBase;
    uint32_t phaseBits = 0;  // bit s: parity of the next completion of stage s's barrier
    bool timedOut = false;
    const int nk = ldb / TKB;
    const int64_t total = *a.tileTotal;

    // The next tile's ids and first STAGES - 1 stages are loaded before the
    // current tile's epilogue (its MMAs are done by then), so the gathers
    // overlap the epilogue.
    auto load_meta = [&](int64_t tb, int b) {  // tb: launch index, mapped to a tile id
        const int64_t t = tile_at(a.tilePerm, tb);
        const int l = a.tileList[t];
        const int64_t ti = t - a.tileOff[l];
        const int mt = (int)(ti / a.nct), ct = (int)(ti % a.nct);
        const int64_t mbeg = a.listOff[l] + (int64_t)mt * TM, mend = a.listOff[l + 1];
        const int r = l % a.nproj, side = l / a.nproj;
        const int32_t* cand = a.topM + (size_t)r * 2 * a.m + side * a.m;
        for (int i = tid; i < TM; i += NT) {
            const int64_t q = mbeg + i;
            if (q < mend) {
                const int2 mb = a.members[q];
                rowPoints[i] = mb.x;
                rowSlots[i] = (uint8_t)mb.y;
            } else {
                rowPoints[i] = -1;
                rowSlots[i] = 0;
            }
        }
        for (int j = tid; j < TN; j += NT) {
            const int c = ct * TN + j;
            colPoints[b][j] = c < a.m ? cand[c] : -1;
        }
    };
    auto load_stage = [&](int b, int stage, int kc) {
        const uint32_t sA = base + stage * STAGE_BYTES, sB = sA + A_BYTES;
        const int k0 = kc * TKB;
#pragma unroll
        for (int it = 0; it < (TM * 8) / NT; ++it) {  // 8 per thread
            const int idx = tid + it * NT, row = idx >> 3, c = idx & 7;
            const int p = rowPoints[row];
            const bool ok = p >= 0;
            cp_async16(sA + sw128(row, c), ok ? Xb + (size_t)p * ldb + k0 + c * 8 : Xb, ok);
        }
#pragma unroll
        for (int it = 0; it < (TN * 8) / NT; ++it) {  // 4 per thread
            const int idx = tid + it * NT, row = idx >> 3, c = idx & 7;
            const int p = colPoints[b][row];
            const bool ok = p >= 0;
            cp_async16(sB + sw128(row, c), ok ? Xb + (size_t)p * ldb + k0 + c * 8 : Xb, ok);
        }
    };
    auto prologue = [&](int b) {
        for (int s = 0; s < STAGES - 1; ++s) {
            if (s < nk) load_stage(b, s, s);
            asm volatile("cp.async.commit_group;\n" ::);
        }
    };
    for (int j = tid; j < TN; j += NT) colCount[j] = 0;  // re-zeroed after each tile's use
    if ((int64_t)blockIdx.x < total) {
        load_meta(blockIdx.x, 0);
        __syncthreads();
        prologue(0);
    }

    int tb = 0;  // parity of the current tile's buffers
    for (int64_t t = blockIdx.x; t < total; t += gridDim.x, tb ^= 1) {
        const int64_t tileId = tile_at(a.tilePerm, t);
        const int ct = (int)((tileId - a.tileOff[a.tileList[tileId]]) % a.nct);
        const int* colPoint = colPoints[tb];
        for (int kc = 0; kc < nk; ++kc) {
            const int stage = kc % STAGES;
            asm volatile("cp.async.wait_group %0;\n" ::"n"(STAGES - 2));
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // cp.async data -> async proxy
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t sA = base + stage * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
                for (int k = 0; k < TKB / 16; ++k)
                    mma_bf16(tmem, smem_desc(sA + k * 32), smem_desc(sB + k * 32), (kc > 0 || k > 0) ? 1u : 0u);
                mma_commit(smem_u32(&bars[stage]));
            }
            const int nxt = kc + STAGES - 1;
            if (nxt < nk) {
                const int ns = nxt % STAGES;
                if (kc >= 1) {  // stage ns was read by the MMAs of chunk kc - 1
                    if (!mbar_wait(smem_u32(&bars[ns]), (phaseBits >> ns) & 1u)) timedOut = true;
                    phaseBits ^= 1u << ns;
                }
                load_stage(tb, ns, nxt);
            }
            asm volatile("cp.async.commit_group;\n" ::);
        }
        // chunks [0, nk - STAGES) were waited on inside the loop; wait for the rest
        for (int c = (nk > STAGES ? nk - STAGES : 0); c < nk; ++c) {
            const int s = c % STAGES;
            if (!mbar_wait(smem_u32(&bars[s]), (phaseBits >> s) & 1u)) timedOut = true;
            phaseBits ^= 1u << s;
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // epilogue: thread tid owns row tid
        const int row = tid;
        const int p = rowPoints[row];
        const int mySlot = rowSlots[row];
        const int64_t tn = t + gridDim.x;
        if (tn < total) {  // the next tile's gathers start now, under this tile's epilogue
            __syncthreads();  // every thread holds its row's ids
            load_meta(tn, tb ^ 1);
            __syncthreads();
            prologue(tb ^ 1);
        }
        uint64_t bits = 0;
        int nPass = 0;
        if constexpr (SWEEP) {
#pragma unroll 1
        for (int c16 = 0; c16 < TN / 16; ++c16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c16 * 16), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = c16 * 16 + j;
                const int q = colPoint[col];
                bool unsure = false;
                if (p >= 0 && q >= 0) {  // keep the screened distance, re-decide near any eps
                    const float dist = 1.0f - v[j];
                    a.dists[((size_t)p * 2 * a.k + mySlot) * a.m + ct * TN + col] = dist;
                    if (p != q)
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
                                        (uint32_t)(ct * TN + col);
                        else
                            atomicExch(err, 2);
                    }
                }
            }
        }
        } else {
        // The row's 64 decisions as bit words: pass (screened distance below
        // eps - margin), unsure (within the margin), near zero (the only place
        // the point itself can be among the candidates); then the columns
        // that do not exist, the row's own point and empty rows are masked out.
        uint64_t uw = 0, zw = 0;
        const float lo = a.eps - kMargin, hi = a.eps + kMargin;
#pragma unroll
        for (int c16 = 0; c16 < TN / 16; ++c16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c16 * 16), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float dist = 1.0f - v[j];
                const bool pass = dist <= lo;
                bits |= (uint64_t)pass << (c16 * 16 + j);
                uw |= (uint64_t)(!pass && dist <= hi) << (c16 * 16 + j);
                zw |= (uint64_t)(dist <= kMargin) << (c16 * 16 + j);
            }
        }
        const int nvalid = a.m - ct * TN;
        uint64_t keep = p < 0 ? 0ull : (nvalid >= 64 ? ~0ull : (1ull << nvalid) - 1ull);
        for (uint64_t z = zw & keep & (bits | uw); z; z &= z - 1) {  // rare: is the row's point a candidate?
            const int col = __ffsll((long long)z) - 1;
            if (colPoint[col] == p) keep &= ~(1ull << col);
        }
        bits &= keep;
        uw &= keep;
        if (__any_sync(0xffffffffu, uw != 0)) {  // pairs within the margin go to the queue
            const int cnt = __popcll(uw);
            if (cnt) {
                unsigned long long at = atomicAdd(qcount, (unsigned long long)cnt);
                for (uint64_t u = uw; u; u &= u - 1, ++at) {
                    const int col = __ffsll((long long)u) - 1;
                    if ((int64_t)at < qcap)
                        queue[at] = ((uint64_t)(uint32_t)p << 32) | ((uint32_t)mySlot << 16) |
                                    (uint32_t)(ct * TN + col);
                    else
                        atomicExch(err, 2);
                }
            }
        }
        nPass = __popcll(bits);
        int cc0 = 0, cc1 = 0;  // passes of columns lane and lane + 32
#pragma unroll
        for (int col = 0; col < TN; ++col) {
            const int pc = __popc(__ballot_sync(0xffffffffu, (bits >> col) & 1ull));
            if (lane == (col & 31)) {
                if (col < 32) cc0 += pc;
                else cc1 += pc;
            }
        }
        if (cc0) atomicAdd(&colCount[lane], cc0);
        if (cc1) atomicAdd(&colCount[lane + 32], cc1);
        }
        if (!SWEEP && p >= 0) a.masks[((size_t)p * 2 * a.k + mySlot) * a.W + ct] = bits;
        const int wp = warp_sum(nPass);
        if (lane == 0 && wp) atomicAdd(a.pairs, (unsigned long long)wp);
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        for (int j = tid; j < TN; j += NT)
            if (colCount[j]) {
                atomicAdd(a.inRaw + colPoint[j], colCount[j]);
                colCount[j] = 0;
            }
        // a timed-out wait anywhere in the CTA ends the CTA's work (uniformly)
        if (__syncthreads_or(timedOut ? 1 : 0)) {
            if (tid == 0) atomicExch(err, 1);
            break;
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// Exact re-decision of the queued pairs: a warp takes 32 queue entries, one
// per lane, and computes their distances with the plain path's sequential
// FP32 dot (dtile::warp_staged_cosine), so the decision equals k_dist's.
constexpr int RC_WARPS = 4;

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
        const float dist = dtile::warp_staged_cosine(rows[w], tile[w], a.ld);
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

int launch_dist_tc(const DistArgs& a, const void* Xb, int ldb, uint64_t* queue, int64_t qcap,
                   unsigned long long* qcount, int32_t* err, int grid, cudaStream_t st) {
    const size_t sm = (size_t)STAGES * STAGE_BYTES + 1024;
    auto kern = a.dists != nullptr ? k_dist_tc<true> : k_dist_tc<false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    kern<<<grid, NT, sm, st>>>(a, static_cast<const __nv_bfloat16*>(Xb), ldb, queue, qcap, qcount, err);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_screen_reset(const DistArgs& a, cudaStream_t st) {
    k_screen_reset<<<sm_count() * 4, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_recheck(const DistArgs& a, const uint64_t* queue, const unsigned long long* qcount, int64_t qcap,
                   cudaStream_t st) {
    k_recheck<<<sm_count() * 8, RC_WARPS * 32, 0, st>>>(a, queue, qcount, qcap);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int dist_tc_tile_rows() { return TM; }

}  // namespace sdb
