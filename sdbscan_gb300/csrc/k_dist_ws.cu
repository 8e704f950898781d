// Stage 4, plain FP32: the candidate distances of rp_findCorePoints /
// rp_findCoreDist (src/sDbscan.cpp:243-359, :1323-1412; computeDist,
// src/Utilities.h:212-287) as a persistent, warp-specialised kernel.
//
// Same tiles, arithmetic and epilogue as k_dist (k_dist.cu): tile = (list l,
// 128 member rows, TX * CN candidate columns); every thread of the
// consumer warps owns 8 x CN pairs and runs one sequential fmaf chain per pair
// over ascending dimensions, so every distance is bit-identical to the CPU
// path's.  What changes is how the operands arrive:
//   - warp NCW (the last) is the producer: it gathers the tile's member rows
//     and candidate rows, 16 dimensions per stage, into a ring of NST stages
//     with cp.async, each lane's copies arriving on the stage's "full"
//     mbarrier (cp.async.mbarrier.arrive.noinc) when they land;
//   - the consumer warps wait on "full", compute, and arrive on the stage's
//     "empty" mbarrier; the producer refills a stage once every consumer warp
//     has released it.
// No CTA-wide barrier sits in the main loop, so a warp that is ahead keeps
// issuing FMAs while another still works on an older stage, and the producer
// runs into the next tile while the consumers finish the current one (tile
// metadata is double-buffered behind its own full / empty barriers).  The
// CTA is persistent and takes the launch order's tiles b, b + grid, ...,
// which keeps the tiles in flight in one window of point chunks (L2 reuse of
// the gathered rows).
//
// Every mbarrier wait is bounded.  A wait that runs out raises the error flag
// (the fit then fails with SDB_ERR_INTERNAL), every role stops at the next
// tile boundary, and the producer waits for its own copies before exiting.
#include "dist_tile.cuh"
#include "tc_common.cuh"

namespace sdb {
namespace {

using namespace dtile;

constexpr int WKT = 16, WLDK = WKT + 4;  // dimensions per stage; smem row stride (floats)

template <int TX, int CN, int NST> struct Ws {
    static constexpr int TNK = TX * CN;    // candidate columns computed
    static constexpr int NC = 16 * TX;      // consumer threads
    static constexpr int NCW = NC / 32;     // consumer warps
    static constexpr int NT = NC + 32;      // + the producer warp
    static constexpr int A_FL = TM * WLDK, B_FL = TNK * WLDK, STAGE_FL = A_FL + B_FL;
    static constexpr size_t SMEM = sizeof(float) * (size_t)NST * STAGE_FL;
    static_assert(NC % 32 == 0, "consumer threads in whole warps");
    static_assert(TNK <= 64, "one 64-bit mask word per tile row");
};

struct TileMeta {
    int rowPoint[TM];
    int rowSlot[TM];
    int colPoint[64];
    int ct;
};

__device__ __forceinline__ void cp_async_arrive_noinc(uint32_t bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(bar) : "memory");
}

// Named barrier 1 over the consumer threads only (the producer warp never
// takes part); the OR form returns the same value to every consumer.
__device__ __forceinline__ bool consumers_or(bool v, int n) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(n)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void consumers_sync(int n) { asm volatile("bar.sync 1, %0;\n" ::"r"(n) : "memory"); }

template <int DIST, int TX, int CN, int NST, int MINB>
__global__ void __launch_bounds__(Ws<TX, CN, NST>::NT, MINB) k_dist_ws(DistArgs a) {
    using C = Ws<TX, CN, NST>;
    constexpr int NC = C::NC, NCW = C::NCW, TNK = C::TNK;
    if (a.gate != nullptr && __ldg(a.gate) == 0) return;  // the BF16 screening succeeded
    extern __shared__ __align__(16) float sm[];
    __shared__ TileMeta meta[2];
    __shared__ uint64_t fullBar[NST], emptyBar[NST], metaFull[2], metaEmpty[2], neverBar;
    __shared__ unsigned smask[2 * TM];
    __shared__ int colCount[64];
    __shared__ int passTotal;
    __shared__ volatile int abortFlag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t total = *a.tileTotal;
    const int nk = (a.d + WKT - 1) / WKT;
    if (tid == 0) {
        for (int s = 0; s < NST; ++s) {
            tc::mbar_init(tc::smem_u32(&fullBar[s]), 32);   // one noinc arrival per producer lane
            tc::mbar_init(tc::smem_u32(&emptyBar[s]), NCW);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(tc::smem_u32(&metaFull[b]), 32);
            tc::mbar_init(tc::smem_u32(&metaEmpty[b]), NCW);
        }
        tc::mbar_init(tc::smem_u32(&neverBar), 1);  // the stall test's barrier: nothing arrives on it
        abortFlag = 0;
        passTotal = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (int i = tid; i < 2 * TM; i += C::NT) smask[i] = 0;
    for (int i = tid; i < 64; i += C::NT) colCount[i] = 0;
    __syncthreads();

    if (warp == NCW) {
        // ---------------- producer ----------------
        long long it = 0;
        int i = 0;
        for (int64_t b = blockIdx.x; b < total && !abortFlag; b += gridDim.x, ++i) {
            const int mb = i & 1;
            if (i >= 2 && !tc::mbar_wait_or(tc::smem_u32(&metaEmpty[mb]), (uint32_t)(((i >> 1) - 1) & 1),
                                            &abortFlag)) {
                abortFlag = 1;
                break;
            }
            TileMeta& M = meta[mb];
            const int64_t t = tile_at(a.tilePerm, b);
            const int l = a.tileList[t];
            const int64_t ti = t - a.tileOff[l];
            const int mt = (int)(ti / a.nct), ct = (int)(ti % a.nct);
            const int64_t mbeg = a.listOff[l] + (int64_t)mt * TM, mend = a.listOff[l + 1];
            const int r = l % a.nproj, side = l / a.nproj;
            const int32_t* cand = a.topM + (size_t)r * 2 * a.m + side * a.m;
#pragma unroll
            for (int u = 0; u < TM / 32; ++u) {
                const int row = lane + 32 * u;
                const int64_t q = mbeg + row;
                int p = -1, slot = 0;
                if (q < mend) {
                    const int2 mm = a.members[q];
                    p = mm.x;
                    slot = mm.y;
                }
                M.rowPoint[row] = p;
                M.rowSlot[row] = slot;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int j = lane + 32 * u;
                const int c = ct * TN + j;
                M.colPoint[j] = (j < TNK && c < a.m) ? cand[c] : -1;
            }
            if (lane == 0) M.ct = ct;
            __syncwarp();
            // copy u of this lane: 16-byte chunk lane % 4 of row 8 u + lane / 4,
            // so the four lanes of a row read its 64 contiguous bytes together
            const int c4 = lane & 3;
            const float* ra[TM / 8];
            const float* rb[(TNK + 7) / 8];
#pragma unroll
            for (int u = 0; u < TM / 8; ++u) {
                const int p = M.rowPoint[8 * u + (lane >> 2)];
                ra[u] = p >= 0 ? a.Xt + (size_t)p * a.ld + 4 * c4 : nullptr;
            }
#pragma unroll
            for (int u = 0; u < (TNK + 7) / 8; ++u) {
                const int row = 8 * u + (lane >> 2);
                const int q = row < TNK ? M.colPoint[row] : -1;
                rb[u] = q >= 0 ? a.Xt + (size_t)q * a.ld + 4 * c4 : nullptr;
            }
            tc::mbar_arrive(tc::smem_u32(&metaFull[mb]));  // release: the tile's ids are visible
            for (int kc = 0; kc < nk; ++kc, ++it) {
                const int s = (int)(it % NST);
                // the stall test: consumers that never release a stage, with copies in flight
                if (it == NST && a.stallSpins > 0 && !tc::stall_wait(tc::smem_u32(&neverBar), a.stallSpins)) {
                    abortFlag = 1;
                    break;
                }
                if (it >= NST && !tc::mbar_wait_or(tc::smem_u32(&emptyBar[s]), (uint32_t)(((it / NST) - 1) & 1),
                                                   &abortFlag)) {
                    abortFlag = 1;
                    break;
                }
                float* As = sm + (size_t)s * C::STAGE_FL;
                float* Bs = As + C::A_FL;
                const int k0 = kc * WKT;
                const bool inRow = k0 + 4 * c4 < a.ld;
#pragma unroll
                for (int u = 0; u < TM / 8; ++u) {
                    const bool ok = ra[u] != nullptr && inRow;
                    cp_async16(As + (8 * u + (lane >> 2)) * WLDK + 4 * c4, ok ? ra[u] + k0 : a.Xt, ok);
                }
#pragma unroll
                for (int u = 0; u < (TNK + 7) / 8; ++u) {
                    const int row = 8 * u + (lane >> 2);
                    if (row < TNK) {
                        const bool ok = rb[u] != nullptr && inRow;
                        cp_async16(Bs + row * WLDK + 4 * c4, ok ? rb[u] + k0 : a.Xt, ok);
                    }
                }
                cp_async_arrive_noinc(tc::smem_u32(&fullBar[s]));
            }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        if (abortFlag && lane == 0) atomicExch(a.waitErr, 1);
        return;
    }

    // ---------------- consumers ----------------
    const int ty = tid / TX, tx = tid % TX;
    long long it = 0;
    int i = 0;
    bool bad = false;
    for (int64_t b = blockIdx.x; b < total; b += gridDim.x, ++i) {
        const int mb = i & 1;
        if (!bad && !tc::mbar_wait_or(tc::smem_u32(&metaFull[mb]), (uint32_t)((i >> 1) & 1), &abortFlag)) bad = true;
        float acc[8][CN];
#pragma unroll
        for (int r8 = 0; r8 < 8; ++r8)
#pragma unroll
            for (int j = 0; j < CN; ++j) acc[r8][j] = 0.0f;
        for (int kc = 0; kc < nk; ++kc, ++it) {
            const int s = (int)(it % NST);
            if (!bad && !tc::mbar_wait_or(tc::smem_u32(&fullBar[s]), (uint32_t)((it / NST) & 1), &abortFlag))
                bad = true;
            if (!bad) {
                const float* as = sm + (size_t)s * C::STAGE_FL;
                const float* bs = as + C::A_FL;
#pragma unroll
                for (int kk = 0; kk < WKT; kk += 4) {
                    float4 av[8], bv[CN];
#pragma unroll
                    for (int r8 = 0; r8 < 8; ++r8)
                        av[r8] = *reinterpret_cast<const float4*>(as + (ty + 16 * r8) * WLDK + kk);
#pragma unroll
                    for (int j = 0; j < CN; ++j)
                        bv[j] = *reinterpret_cast<const float4*>(bs + (tx + TX * j) * WLDK + kk);
#pragma unroll
                    for (int r8 = 0; r8 < 8; ++r8)
#pragma unroll
                        for (int j = 0; j < CN; ++j) {
                            float c = acc[r8][j];
                            c = acc_step<DIST>(c, av[r8].x, bv[j].x);
                            c = acc_step<DIST>(c, av[r8].y, bv[j].y);
                            c = acc_step<DIST>(c, av[r8].z, bv[j].z);
                            c = acc_step<DIST>(c, av[r8].w, bv[j].w);
                            acc[r8][j] = c;
                        }
                }
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&emptyBar[s]));
        }
        // epilogue (the same decisions and outputs as k_dist)
        const TileMeta& M = meta[mb];
        const int ct = M.ct;
        int myPass = 0;
        int colPass[CN];
#pragma unroll
        for (int j = 0; j < CN; ++j) colPass[j] = 0;
        if (!bad) {
#pragma unroll
            for (int r8 = 0; r8 < 8; ++r8) {
                const int row = ty + 16 * r8;
                const int p = M.rowPoint[row];
                unsigned lo = 0, hi = 0;
#pragma unroll
                for (int j = 0; j < CN; ++j) {
                    const int col = tx + TX * j;
                    const int q = M.colPoint[col];
                    const float dist = finish<DIST>(acc[r8][j]);
                    const bool pass = p >= 0 && q >= 0 && p != q && dist <= a.eps;
                    if (pass) {
                        if (col < 32) lo |= 1u << col;
                        else hi |= 1u << (col - 32);
                        colPass[j] += 1;
                        ++myPass;
                    }
                    if (a.dists != nullptr && p >= 0 && q >= 0)
                        a.dists[((size_t)p * 2 * a.k + M.rowSlot[row]) * a.m + ct * TN + col] = dist;
                }
                if (lo) atomicOr(&smask[2 * row], lo);
                if (hi) atomicOr(&smask[2 * row + 1], hi);
            }
#pragma unroll
            for (int j = 0; j < CN; ++j)
                if (colPass[j]) atomicAdd(&colCount[tx + TX * j], colPass[j]);
            const int wp = warp_sum(myPass);
            if (lane == 0 && wp) atomicAdd(&passTotal, wp);
        }
        const bool stopNow = consumers_or(bad || abortFlag != 0, NC);
        for (int row = tid; row < TM; row += NC) {
            const int p = M.rowPoint[row];
            if (!stopNow && p >= 0) {
                const uint64_t w = ((uint64_t)smask[2 * row + 1] << 32) | smask[2 * row];
                a.masks[((size_t)p * 2 * a.k + M.rowSlot[row]) * a.W + ct] = w;
            }
            smask[2 * row] = 0;
            smask[2 * row + 1] = 0;
        }
        for (int j = tid; j < TNK; j += NC) {
            if (!stopNow && colCount[j]) atomicAdd(a.inRaw + M.colPoint[j], colCount[j]);
            colCount[j] = 0;
        }
        if (tid == 0) {
            if (!stopNow && passTotal) atomicAdd(a.pairs, (unsigned long long)passTotal);
            passTotal = 0;
        }
        consumers_sync(NC);  // the cleared counters before the next tile's atomics
        if (lane == 0) tc::mbar_arrive(tc::smem_u32(&metaEmpty[mb]));
        if (stopNow) {
            abortFlag = 1;
            if (tid == 0) atomicExch(a.waitErr, 1);
            break;
        }
    }
}

template <int DIST, int TX, int CN, int NST, int MINB> int launch_ws(const DistArgs& a, cudaStream_t st) {
    using C = Ws<TX, CN, NST>;
    auto kern = k_dist_ws<DIST, TX, CN, NST, MINB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM) != cudaSuccess)
        return -1;
    if (a.nTiles <= 0) return 0;
    const int64_t grid = std::min<int64_t>(a.nTiles, (int64_t)sm_count() * MINB);
    kern<<<(unsigned)grid, C::NT, C::SMEM, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace

// The warp-specialised shapes: 128 x 50 (m <= 50, five consumer warps) and
// 128 x 64 (any m, eight consumer warps).  variant 4 = 4 stages, 3 CTAs per
// SM; variant 5 = 6 stages, 2 CTAs per SM.
int launch_dist_ws(const DistArgs& a, int variant, cudaStream_t st) {
    if (a.waitErr == nullptr) return -1;
    const bool fits50 = a.m <= 50;
    switch (a.dist) {
#define SDB_WS(D)                                                                                  \
    case D:                                                                                        \
        if (fits50) return variant == 5 ? launch_ws<D, 10, 5, 6, 2>(a, st) : launch_ws<D, 10, 5, 4, 3>(a, st); \
        return variant == 5 ? launch_ws<D, 16, 4, 6, 1>(a, st) : launch_ws<D, 16, 4, 4, 2>(a, st);
        SDB_WS(DIST_COSINE)
        SDB_WS(DIST_L1)
        SDB_WS(DIST_L2)
        SDB_WS(DIST_CHI2)
        SDB_WS(DIST_JS)
#undef SDB_WS
    }
    return -1;
}

}  // namespace sdb
