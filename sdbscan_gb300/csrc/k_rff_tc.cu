// Stage 1, BF16 mode for L1 / L2: the random-Fourier-feature embedding
// (src/sDbscan.cpp:53-68) as one GEMM on the tcgen05 tensor cores,
//   V = X R^T   (X: n x d points, R: h x d, h = ker / 2),   E = [cos V, sin V],
// with BF16 operands loaded by TMA and FP32 accumulation in tensor memory.
//
// Split BF16: each FP32 operand x is stored as hi = bf16(x), lo = bf16(x - hi)
// (x - hi is exact in FP32) and the accumulator takes hi.hi + hi.lo + lo.hi:
// three passes over K into the same tensor memory.  Each product then errs by
// at most ~3 * 2^-16 of |x||y| (the dropped lo.lo and the rounding of the lo
// parts) instead of 2^-7 for one BF16 pass, which keeps the cos / sin
// features within ~1e-4 of FP32 and the candidate lists of the plain path.
//
// Tile: 128 points x 256 rows of R, K in chunks of 64 (one 128-byte swizzle
// atom per row, the layout TMA's 128B swizzle writes and the MMA's smem
// descriptor reads); 97 KB of smem, so two CTAs share an SM and one's
// epilogue overlaps the other's loads.  Thread 0 keeps a STAGES-deep ring of TMA loads in
// flight (an mbarrier per stage counts the bytes in, a second one is
// committed by the MMAs that read the stage) and issues
// tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = 256, K = 16) into a
// 128 x 256 FP32 accumulator.  Then the eight warps read their points' rows of
// the accumulator with tcgen05.ld (two warps per 32-lane quarter, one half of
// the columns each) and write cos / sin to E.
//
// Every wait is bounded: on a timeout the CTA records an error, waits (again
// bounded) for the loads it issued, frees its tensor memory and returns; the
// host then runs the FP32 kernel instead (launch_rff with the flag as gate).
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "tc_common.cuh"

namespace sdb {
namespace {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 2, NT = 256;
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;  // 16 KB + 32 KB
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kIdesc = tc::idesc_bf16(BM, BN);

__global__ void __launch_bounds__(NT, 2) k_rff_tc(const __grid_constant__ CUtensorMap tmX,
                                                 const __grid_constant__ CUtensorMap tmR, int n, int h, int nk,
                                                 float* __restrict__ E, int32_t* __restrict__ err,
                                                 long long stallSpins) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __shared__ uint64_t fullBar[STAGES], freeBar[STAGES], doneBar, neverBar;
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (tc::smem_u32(smraw) + 1023u) & ~1023u;  // 1024-aligned operand tiles
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(tc::smem_u32(&fullBar[s]), 1);
            tc::mbar_init(tc::smem_u32(&freeBar[s]), 1);
        }
        tc::mbar_init(tc::smem_u32(&doneBar), 1);
        tc::mbar_init(tc::smem_u32(&neverBar), 1);  // the stall test's barrier: nothing arrives on it
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

    int failed = 0;
    if (tid == 0) {
        int issued[STAGES] = {}, landed[STAGES] = {};  // loads issued into / waited on per stage
        // chunk kc of pass kc / nk: pass 0 hi(X).hi(R), 1 hi(X).lo(R), 2 lo(X).hi(R)
        // (each matrix holds [hi | lo], nk chunks apiece)
        auto load = [&](int kc) {
            const int s = kc % STAGES, pass = kc / nk, kk = kc % nk;
            const uint32_t sA = base + s * STAGE_BYTES, sB = sA + A_BYTES, bar = tc::smem_u32(&fullBar[s]);
            tc::mbar_expect_tx(bar, STAGE_BYTES);
            tc::tma_load_2d(sA, &tmX, (pass == 2 ? nk + kk : kk) * BK, m0, bar);
            tc::tma_load_2d(sB, &tmR, (pass == 1 ? nk + kk : kk) * BK, n0, bar);
            ++issued[s];
        };
        const int nkAll = 3 * nk;
        for (int kc = 0; kc < nkAll && kc < STAGES; ++kc) load(kc);
        int committed = 0;
        // the stall test: a producer that never delivers, with loads in flight
        if (stallSpins > 0 && !tc::stall_wait(tc::smem_u32(&neverBar), stallSpins)) failed = 1;
        for (int kc = 0; kc < nkAll && !failed; ++kc) {
            const int s = kc % STAGES;
            if (!tc::mbar_wait(tc::smem_u32(&fullBar[s]), (uint32_t)(landed[s] & 1))) {
                failed = 1;
                break;
            }
            ++landed[s];
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sA = base + s * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
            for (int k = 0; k < BK / 16; ++k)
                tc::mma_bf16(tmem, tc::smem_desc(sA + k * 32), tc::smem_desc(sB + k * 32), kIdesc,
                             (kc > 0 || k > 0) ? 1u : 0u);
            tc::mma_commit(tc::smem_u32(&freeBar[s]));
            ++committed;
            const int nxt = kc + STAGES;
            if (nxt < nkAll) {  // stage s is refilled once the MMAs above have read it
                if (!tc::mbar_wait(tc::smem_u32(&freeBar[s]), (uint32_t)((kc / STAGES) & 1))) {
                    failed = 1;
                    break;
                }
                load(nxt);
            }
        }
        tc::mma_commit(tc::smem_u32(&doneBar));
        if (failed) {
            atomicExch(err, 1);
            for (int s = 0; s < STAGES; ++s)  // drain the loads still in flight
                while (landed[s] < issued[s]) {
                    tc::mbar_wait(tc::smem_u32(&fullBar[s]), (uint32_t)(landed[s] & 1));
                    ++landed[s];
                }
        }
        (void)committed;
    }
    // every thread waits for the accumulator (all MMAs committed above)
    const bool done = tc::mbar_wait(tc::smem_u32(&doneBar), 0u);
    failed = __syncthreads_or(failed || !done);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    if (!failed) {
        // warps w and w + 4 read tensor-memory lanes 32 (w % 4) .. + 31 (their
        // points), each for one half of the 256 columns
        const int lanes = (warp & 3) * 32, half = warp >> 2;
        const int row = m0 + lanes + (tid & 31);
        const bool vec = (h & 3) == 0;
#pragma unroll 1
        for (int c16 = half * (BN / 32); c16 < (half + 1) * (BN / 32); ++c16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)lanes << 16) + (uint32_t)(c16 * 16), v);
            if (row >= n) continue;
            float* ec = E + (size_t)row * 2 * h;
#pragma unroll
            for (int j = 0; j < 16; j += 4) {
                const int r = n0 + c16 * 16 + j;
                float sn[4], cs[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) sincosf(v[j + t], &sn[t], &cs[t]);
                if (vec && r + 3 < h) {
                    *reinterpret_cast<float4*>(ec + r) = make_float4(cs[0], cs[1], cs[2], cs[3]);
                    *reinterpret_cast<float4*>(ec + h + r) = make_float4(sn[0], sn[1], sn[2], sn[3]);
                } else {
                    for (int t = 0; t < 4; ++t)
                        if (r + t < h) {
                            ec[r + t] = cs[t];
                            ec[h + r + t] = sn[t];
                        }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

// Xs: n x 2 ldb BF16 points ([hi | lo] per row), Rs: h x 2 ldb BF16 rows of R
// likewise (ldb a multiple of 64, zero padded past d, 16-byte aligned);
// E: n x 2h FP32.
int launch_rff_tc(const void* Xs, const void* Rs, int n, int h, int ldb, float* E, int32_t* err, long long stallSpins,
                  cudaStream_t st) {
    if (ldb % BK != 0 || (reinterpret_cast<uintptr_t>(Xs) & 15) || (reinterpret_cast<uintptr_t>(Rs) & 15)) return -1;
    CUtensorMap tmX, tmR;
    if (!tc::encode_bf16_2d(&tmX, Xs, n, 2 * ldb, BK, BM) || !tc::encode_bf16_2d(&tmR, Rs, h, 2 * ldb, BK, BN))
        return -1;
    const size_t sm = (size_t)STAGES * STAGE_BYTES + 1024;
    if (cudaFuncSetAttribute(k_rff_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    dim3 grid((n + BM - 1) / BM, (h + BN - 1) / BN);
    k_rff_tc<<<grid, NT, sm, st>>>(tmX, tmR, n, h, ldb / BK, E, err, stallSpins);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
