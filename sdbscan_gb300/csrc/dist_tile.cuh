// The FP32 distance tile shared by the candidate-distance stage (k_dist) and
// the sampled-neighbourhood block of sngDbscan / sngOptics (k_sng_block):
// computeDist (src/Utilities.h:212-287) for TM member rows x TX * CN
// candidate columns.
//
// Rows and columns are points of the transformed data (row stride ld, zero
// padded), named by id in shared memory (-1 for an empty row or column).
// They are staged through shared memory with cp.async, TK dimensions per
// stage in STAGES stages; each of the 16 * TX threads owns an 8 x CN block of
// pairs and accumulates over dimensions in ascending order, one rounding
// sequence per pair identical to the oracle's, so every distance is
// bit-identical to the CPU path.
#pragma once

#include "common.cuh"

namespace sdb {
namespace dtile {

// Tile rows, dimensions per stage, smem row stride, stages, and the tile
// grid's candidate columns (and mask bits) per tile.
constexpr int TM = 128, TK = 32, LDS = TK + 4, STAGES = 2;
constexpr int TN = 64;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <int DIST> __device__ __forceinline__ float acc_step(float acc, float a, float b) {
    if (DIST == DIST_COSINE) {
        return __fmaf_rn(a, b, acc);
    } else if (DIST == DIST_L2) {
        const float t = __fsub_rn(a, b);
        return __fmaf_rn(t, t, acc);
    } else if (DIST == DIST_L1) {
        return __fadd_rn(acc, fabsf(__fsub_rn(a, b)));
    } else if (DIST == DIST_CHI2) {
        // Branch-free: every lane divides (1 / 1 where an entry is not
        // positive) and adds the term or +0; acc >= +0, so acc + 0 == acc and
        // the sum is bit-identical to skipping the term.
        const bool both = a > 0.0f && b > 0.0f;
        const float q = __fdiv_rn(both ? __fmul_rn(a, b) : 1.0f, both ? __fadd_rn(a, b) : 1.0f);
        return __fadd_rn(acc, both ? q : 0.0f);
    } else {  // JS with EPSILON = 1e-6 added to both (src/Utilities.h:248-266)
        const float x = __fadd_rn(a, 1e-6f), y = __fadd_rn(b, 1e-6f);
        const float l2 = 0.693147182464599609375f;  // (float)log(2.0)
        const float s = __fadd_rn(x, y);
        const float t1 = __fmul_rn(__fdiv_rn(logf(__fdiv_rn(s, x)), l2), x);
        const float t2 = __fmul_rn(__fdiv_rn(logf(__fdiv_rn(s, y)), l2), y);
        return __fadd_rn(acc, __fadd_rn(t1, t2));
    }
}

template <int DIST> __device__ __forceinline__ float finish(float acc) {
    if (DIST == DIST_COSINE) return __fsub_rn(1.0f, acc);           // 1 - x.y
    if (DIST == DIST_L2) return __fsqrt_rn(acc);                    // ||x - y||
    if (DIST == DIST_L1) return acc;                                 // sum |x - y|
    if (DIST == DIST_CHI2) return __fsub_rn(1.0f, __fmul_rn(2.0f, acc));  // == (float)(1.0 - 2.0*t), exact
    return __fsub_rn(1.0f, __fmul_rn(acc, 0.5f));                    // == (float)(1.0 - t/2.0), exact
}

// One pair on one thread, the same rounding sequence as the tile.
template <int DIST> __device__ __forceinline__ float pair_distance(const float* __restrict__ x,
                                                                   const float* __restrict__ y, int d) {
    float acc = 0.0f;
    for (int j = 0; j < d; ++j) acc = acc_step<DIST>(acc, __ldg(x + j), __ldg(y + j));
    return finish<DIST>(acc);
}

// Exact distances of 32 pairs, one per lane of the calling warp: rows[0..31]
// point at the lanes' first rows, rows[32..63] at their second rows
// (transformed data, stride ld, zero padded; rows in the warp's shared
// memory, written before the call and synchronised with __syncwarp).  Both
// rows of every pair are staged through tile (64 x 33 floats of the warp's
// shared memory) 32 dimensions at a time with coalesced loads, the next chunk
// prefetched into registers; each lane runs its pair's sequential chain in
// ascending dimension order (a zero-padded dimension leaves it unchanged),
// the plain path's arithmetic (acc_step, finish).
template <int DIST>
__device__ __forceinline__ float warp_staged(const float* const* rows, float (*tile)[33], int ld) {
    const int lane = threadIdx.x & 31;
    float stage[64];
#pragma unroll
    for (int r = 0; r < 64; ++r) stage[r] = lane < ld ? __ldg(rows[r] + lane) : 0.0f;
    float s = 0.0f;
    for (int c = 0; c < ld; c += 32) {
#pragma unroll
        for (int r = 0; r < 64; ++r) tile[r][lane] = stage[r];
        __syncwarp();
        const int cn = c + 32 + lane;
        if (c + 32 < ld) {
#pragma unroll
            for (int r = 0; r < 64; ++r) stage[r] = cn < ld ? __ldg(rows[r] + cn) : 0.0f;
        }
        const int tn = min(32, ld - c);
        if (tn == 32) {
#pragma unroll
            for (int t = 0; t < 32; ++t) s = acc_step<DIST>(s, tile[lane][t], tile[32 + lane][t]);
        } else {
            for (int t = 0; t < tn; ++t) s = acc_step<DIST>(s, tile[lane][t], tile[32 + lane][t]);
        }
        __syncwarp();
    }
    return finish<DIST>(s);
}
__device__ __forceinline__ float warp_staged_cosine(const float* const* rows, float (*tile)[33], int ld) {
    return warp_staged<DIST_COSINE>(rows, tile, ld);
}

// The thread's row group ty (0..15) and column group tx (0..TX-1).  A
// quarter-warp's eight 16-byte fragment loads are conflict-free when its
// column rows tx + TX j fall in eight different bank groups (row r's chunk
// sits in group (5 r + c) mod 8 for the row stride of 20 floats).  For TX = 10
// the plain tid % TX puts tx = 8, 9 next to 0, 1 in one quarter-warp (the same
// groups); instead, of every five quarter-warps four take tx = 0..7 of one row
// group each and the fifth takes tx = 8, 9 of all four.
template <int TX> __device__ __forceinline__ void tile_coords(int tid, int& ty, int& tx) {
    if constexpr (TX == 10) {
        const int qw = tid >> 3, l8 = tid & 7, g = qw / 5, qi = qw % 5;
        ty = 4 * g + (qi < 4 ? qi : (l8 >> 1));
        tx = qi < 4 ? l8 : 8 + (l8 & 1);
    } else {
        ty = tid / TX;
        tx = tid % TX;
    }
}

// acc[i][j] = accumulated distance terms of (row ty + 16 i, column tx + TX j)
// with (ty, tx) = tile_coords<TX>(tid).  KT dimensions per stage, NST stages:
// As / Bs are NST x TM x (KT + 4) and NST x (TX * CN) x (KT + 4) floats of
// shared memory (the +4 keeps the float4 fragment reads of consecutive rows
// in different bank groups).  Ends with every copy landed; the caller
// synchronises before reusing the buffers.
template <int DIST, int TX, int CN, int KT = TK, int NST = STAGES>
__device__ __forceinline__ void accumulate(const float* __restrict__ Xt, int ld, int d, const int* rowPoint,
                                           const int* colPoint, float* As, float* Bs, float (&acc)[8][CN]) {
    constexpr int NT = 16 * TX, TNK = TX * CN, LDK = KT + 4, CPR = KT / 4;  // CPR: 16-byte chunks per row
    const int tid = threadIdx.x;
    const int nk = (d + KT - 1) / KT;
    auto load_stage = [&](int stage, int kc) {
        float* as = As + stage * TM * LDK;
        float* bs = Bs + stage * TNK * LDK;
        const int k0 = kc * KT;
#pragma unroll
        for (int idx = tid; idx < TM * CPR; idx += NT) {
            const int row = idx / CPR, c4 = idx % CPR;
            const int p = rowPoint[row];
            const int col = k0 + c4 * 4;
            const bool ok = p >= 0 && col < ld;
            const float* src = ok ? Xt + (size_t)p * ld + col : Xt;
            cp_async16(as + row * LDK + c4 * 4, src, ok);
        }
#pragma unroll
        for (int idx = tid; idx < TNK * CPR; idx += NT) {
            const int row = idx / CPR, c4 = idx % CPR;
            const int p = colPoint[row];
            const int col = k0 + c4 * 4;
            const bool ok = p >= 0 && col < ld;
            const float* src = ok ? Xt + (size_t)p * ld + col : Xt;
            cp_async16(bs + row * LDK + c4 * 4, src, ok);
        }
    };

#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < CN; ++j) acc[i][j] = 0.0f;

    int ty, tx;
    tile_coords<TX>(tid, ty, tx);
#pragma unroll
    for (int s = 0; s < NST - 1; ++s) {
        if (s < nk) load_stage(s, s);
        cp_async_commit();
    }
    for (int kc = 0; kc < nk; ++kc) {
        cp_async_wait<NST - 2>();
        __syncthreads();
        const int nxt = kc + NST - 1;
        if (nxt < nk) load_stage(nxt % NST, nxt);
        cp_async_commit();
        const float* as = As + (kc % NST) * TM * LDK;
        const float* bs = Bs + (kc % NST) * TNK * LDK;
#pragma unroll
        for (int kk = 0; kk < KT; kk += 4) {
            float4 av[8], bv[CN];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = *reinterpret_cast<const float4*>(as + (ty + 16 * i) * LDK + kk);
#pragma unroll
            for (int j = 0; j < CN; ++j) bv[j] = *reinterpret_cast<const float4*>(bs + (tx + TX * j) * LDK + kk);
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < CN; ++j) {
                    float c = acc[i][j];
                    c = acc_step<DIST>(c, av[i].x, bv[j].x);
                    c = acc_step<DIST>(c, av[i].y, bv[j].y);
                    c = acc_step<DIST>(c, av[i].z, bv[j].z);
                    c = acc_step<DIST>(c, av[i].w, bv[j].w);
                    acc[i][j] = c;
                }
        }
    }
    cp_async_wait<0>();
}

}  // namespace dtile
}  // namespace sdb
