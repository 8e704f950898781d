// Stage 2: per random vector, the m largest ("close") and m smallest ("far")
// projections over all points — matrix_topM of rp_parIndex
// (src/sDbscan.cpp:151-208).
//
// Exact without a per-vector heap over n:
//  1. The projection kernel leaves, for every chunk of points, the maximum
//     and minimum projection onto each vector.  The m-th largest of the chunk
//     maxima is a value attained by m different points, so it is a lower
//     bound T on the true m-th largest value (k_thresholds).
//  2. One pass over the projections appends every (value, point) with value
//     >= T to the vector's candidate list (k_collect).  All of the top m are
//     in it.
//  3. An exact sort of each candidate list by (value desc, point asc) yields
//     the top m (k_select).  A list whose candidates overflow its buffer is
//     resolved by an exact radix select over the whole column (k_fallback).
// Ties: the reference's heap keeps, among equal values at the boundary, the
// ones its heap order dictates; this engine keeps the smallest point ids and
// counts such boundary ties.
#include "common.cuh"

#include <algorithm>

namespace sdb {
namespace {

// Block-wide bitonic sort (descending) of `len` (power of two) u64 keys in smem.
__device__ void block_sort_desc(uint64_t* s, int len) {
    for (int size = 2; size <= len; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (int i = threadIdx.x; i < len / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool desc = (lo & size) == 0;
                const uint64_t a = s[lo], b = s[hi];
                if ((a < b) == desc) {
                    s[lo] = b;
                    s[hi] = a;
                }
            }
        }
    }
    __syncthreads();
}

__host__ __device__ inline int pow2_ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// One CTA per list (r, side): T = m-th largest key among the G chunk extremes
// (0 when G < m), by a 4-pass 8-bit radix select over the keys staged in
// shared memory.
__global__ void k_thresholds(TopMArgs a) {
    extern __shared__ uint32_t keys[];
    __shared__ uint32_t hist[256];
    __shared__ uint32_t selPrefix, selMask, selRank;
    const int list = blockIdx.x;
    const int r = list % a.nproj, side = list / a.nproj;
    for (int g = threadIdx.x; g < a.G; g += blockDim.x) {
        const float x = side == 0 ? a.chunkMax[(size_t)g * a.nproj + r] : -a.chunkMin[(size_t)g * a.nproj + r];
        keys[g] = key_of(x);
    }
    if (threadIdx.x == 0) {
        selPrefix = 0;
        selMask = 0;
        selRank = (uint32_t)a.m;  // rank (1-based, from the top) still to find inside the prefix
    }
    if (a.G < a.m) {
        if (threadIdx.x == 0) (side == 0 ? a.thrMax : a.thrMin)[r] = __uint_as_float(0u);
        return;
    }
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        const uint32_t pre = selPrefix, msk = selMask;
        for (int g = threadIdx.x; g < a.G; g += blockDim.x) {
            const uint32_t k = keys[g];
            if ((k & msk) == pre) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t cum = 0, rank = selRank;
            for (int b = 255; b >= 0; --b) {
                if (cum + hist[b] >= rank) {
                    selRank = rank - cum;
                    selPrefix = pre | ((uint32_t)b << shift);
                    selMask = msk | (255u << shift);
                    break;
                }
                cum += hist[b];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) (side == 0 ? a.thrMax : a.thrMin)[r] = __uint_as_float(selPrefix);  // raw key bits
}

// A block takes kCollectRows consecutive points; a thread takes 4
// consecutive vectors of them (16-byte loads, all rows' loads issued before
// any compare, the vectors' thresholds loaded once).
constexpr int kCollectRows = 8;
__global__ void __launch_bounds__(256) k_collect(TopMArgs a) {
    const int per_row = a.nproj / 4;
    const int p0 = blockIdx.x * kCollectRows;
    for (int c4 = threadIdx.x; c4 < per_row; c4 += blockDim.x) {
        const int r0 = c4 * 4;
        float4 v4[kCollectRows];
#pragma unroll
        for (int i = 0; i < kCollectRows; ++i)
            v4[i] = p0 + i < a.n ? __ldcs(reinterpret_cast<const float4*>(a.P + (size_t)(p0 + i) * a.nproj) + c4)
                                 : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float4 tcv = __ldg(reinterpret_cast<const float4*>(a.thrMax) + c4);
        const float4 tfv = __ldg(reinterpret_cast<const float4*>(a.thrMin) + c4);
        const uint32_t tc[4] = {__float_as_uint(tcv.x), __float_as_uint(tcv.y), __float_as_uint(tcv.z),
                                __float_as_uint(tcv.w)};
        const uint32_t tf[4] = {__float_as_uint(tfv.x), __float_as_uint(tfv.y), __float_as_uint(tfv.z),
                                __float_as_uint(tfv.w)};
#pragma unroll
        for (int i = 0; i < kCollectRows; ++i) {
            const int p = p0 + i;
            if (p >= a.n) break;
            const float vv[4] = {v4[i].x, v4[i].y, v4[i].z, v4[i].w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int r = r0 + t;
                const uint32_t kc = key_of(vv[t]);
                const uint32_t kf = key_of(-vv[t]);
                if (kc >= tc[t]) {
                    const int slot = atomicAdd(a.candCount + r, 1);
                    if (slot < a.cap)
                        a.cand[(size_t)r * a.cap + slot] = ((uint64_t)kc << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
                }
                if (kf >= tf[t]) {
                    const int list = a.nproj + r;
                    const int slot = atomicAdd(a.candCount + list, 1);
                    if (slot < a.cap)
                        a.cand[(size_t)list * a.cap + slot] =
                            ((uint64_t)kf << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
                }
            }
        }
    }
}

// Generic (nproj % 4 != 0) variant: one thread per projection.
__global__ void k_collect1(TopMArgs a) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)a.n * a.nproj;
    if (q >= total) return;
    const int p = (int)(q / a.nproj);
    const int r = (int)(q % a.nproj);
    const float v = a.P[q];
    const uint32_t kc = key_of(v), kf = key_of(-v);
    if (kc >= __float_as_uint(a.thrMax[r])) {
        const int slot = atomicAdd(a.candCount + r, 1);
        if (slot < a.cap) a.cand[(size_t)r * a.cap + slot] = ((uint64_t)kc << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
    }
    if (kf >= __float_as_uint(a.thrMin[r])) {
        const int list = a.nproj + r;
        const int slot = atomicAdd(a.candCount + list, 1);
        if (slot < a.cap) a.cand[(size_t)list * a.cap + slot] = ((uint64_t)kf << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
    }
}

// One CTA per list: exact sort of the candidates, first m written to topM.
__global__ void k_select(TopMArgs a) {
    extern __shared__ uint64_t sk[];
    const int list = blockIdx.x;
    const int r = list % a.nproj, side = list / a.nproj;
    const int c = a.candCount[list];
    if (c > a.cap) return;  // resolved by k_fallback
    const int len = pow2_ceil(max(c, 2));
    for (int i = threadIdx.x; i < len; i += blockDim.x) sk[i] = i < c ? a.cand[(size_t)list * a.cap + i] : 0ull;
    block_sort_desc(sk, len);
    // c >= m always holds (the threshold is attained by >= m points); if it
    // ever did not, point 0 stands in and the fit reports an internal error.
    for (int i = threadIdx.x; i < a.m; i += blockDim.x)
        a.topM[(size_t)r * 2 * a.m + side * a.m + i] = i < c ? (int32_t)(0xffffffffu - (uint32_t)sk[i]) : 0;
    if (threadIdx.x == 0 && c < a.m) atomicExch(a.errFlag, 1);
    if (threadIdx.x == 0 && c > a.m && (sk[a.m - 1] >> 32) == (sk[a.m] >> 32)) atomicAdd(a.ties, 1ull);
}

// Exact radix select over a whole column, for lists whose candidate buffer
// overflowed (heavy ties, adversarial orderings).  One CTA per list; CTAs of
// lists that did not overflow return at once.
__global__ void k_fallback(TopMArgs a) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t prefix, prefixMask;
    __shared__ int need;  // how many of the remaining (prefix-matching) elements we still take
    __shared__ int above; // elements strictly above the final key
    __shared__ int taken;
    extern __shared__ uint64_t sk[];  // m (pow2) selected entries
    const int list = blockIdx.x;
    if (a.candCount[list] <= a.cap) return;
    const int r = list % a.nproj, side = list / a.nproj;
    auto keyAt = [&](int p) -> uint32_t {
        const float v = a.P[(size_t)p * a.nproj + r];
        return side == 0 ? key_of(v) : key_of(-v);
    };
    if (threadIdx.x == 0) {
        prefix = 0;
        prefixMask = 0;
        need = a.m;
        above = 0;
    }
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        for (int p = threadIdx.x; p < a.n; p += blockDim.x) {
            const uint32_t k = keyAt(p);
            if ((k & prefixMask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int b = 255; b >= 0; --b) {
                if (acc + (int)hist[b] >= need) {
                    prefix |= (uint32_t)b << shift;
                    prefixMask |= 255u << shift;
                    above += acc;
                    need -= acc;
                    break;
                }
                acc += hist[b];
            }
        }
        __syncthreads();
    }
    // prefix is now the exact m-th largest key K; `above` elements are > K and
    // `need` elements equal to K are taken, smallest point ids first.
    const uint32_t K = prefix;
    const int len = pow2_ceil(max(a.m, 2));
    for (int i = threadIdx.x; i < len; i += blockDim.x) sk[i] = 0;
    if (threadIdx.x == 0) taken = 0;
    __syncthreads();
    __shared__ int eqTaken;
    if (threadIdx.x == 0) eqTaken = 0;
    __syncthreads();
    // strictly greater: any order
    for (int p = threadIdx.x; p < a.n; p += blockDim.x) {
        const uint32_t k = keyAt(p);
        if (k > K) {
            const int s = atomicAdd(&taken, 1);
            sk[s] = ((uint64_t)k << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
        }
    }
    __syncthreads();
    // equal: in ascending point order, block-sequential chunks
    int eqTotal = 0;
    for (int base = 0; base < a.n; base += blockDim.x) {
        const int p = base + threadIdx.x;
        const bool eq = p < a.n && keyAt(p) == K;
        const int cnt = __syncthreads_count(eq);
        // rank within the chunk
        const unsigned bal = __ballot_sync(0xffffffffu, eq);
        __shared__ int warpCnt[32];
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) warpCnt[w] = __popc(bal);
        __syncthreads();
        int before = 0;
        for (int ww = 0; ww < w; ++ww) before += warpCnt[ww];
        before += __popc(bal & ((1u << (threadIdx.x & 31)) - 1u));
        const int rank = eqTaken + before;
        if (eq && rank < need) sk[above + rank] = ((uint64_t)K << 32) | (uint32_t)(0xffffffffu - (uint32_t)p);
        __syncthreads();
        if (threadIdx.x == 0) eqTaken += cnt;
        eqTotal += cnt;
        __syncthreads();
    }
    block_sort_desc(sk, len);
    for (int i = threadIdx.x; i < a.m; i += blockDim.x)
        a.topM[(size_t)r * 2 * a.m + side * a.m + i] = (int32_t)(0xffffffffu - (uint32_t)sk[i]);
    if (threadIdx.x == 0 && eqTotal > need) atomicAdd(a.ties, 1ull);
}

}  // namespace

int launch_topm_thresholds(const TopMArgs& a, cudaStream_t st) {
    const size_t sm = sizeof(uint32_t) * (size_t)a.G;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_thresholds, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_thresholds<<<2 * a.nproj, 256, sm, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_topm_collect(const TopMArgs& a, cudaStream_t st) {
    if (a.nproj % 4 == 0 && (reinterpret_cast<uintptr_t>(a.P) & 15) == 0 &&
        (reinterpret_cast<uintptr_t>(a.thrMax) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.thrMin) & 15) == 0) {
        const int threads = std::min(256, (a.nproj / 4 + 31) / 32 * 32);
        k_collect<<<(unsigned)((a.n + kCollectRows - 1) / kCollectRows), threads, 0, st>>>(a);
    } else {
        const size_t total = (size_t)a.n * a.nproj;
        k_collect1<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a);
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_topm_select(const TopMArgs& a, cudaStream_t st) {
    const size_t sm = sizeof(uint64_t) * pow2_ceil(a.cap);
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute(k_select, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    k_select<<<2 * a.nproj, 256, sm, st>>>(a);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    const size_t sm2 = sizeof(uint64_t) * pow2_ceil(a.m < 2 ? 2 : a.m);
    k_fallback<<<2 * a.nproj, 256, sm2, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

}  // namespace sdb
