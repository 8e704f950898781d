// Stage 1 of the fit: transformData + kernel embedding + the three rounds of
// random sign flips and Walsh-Hadamard transforms + per-point top-k.
//
// Reference: transformData (src/Utilities.h:289-335), the per-point loop of
// rp_parIndex (src/sDbscan.cpp:46-145) and the embeddings embedChi2 / embedJS
// (src/Utilities.h:132-208).
//
// Layout: one warp per point.  Lane l holds elements e = l + 32*j of the
// fhtDim-long rotation vector in register v[j].  Butterflies of stride < 32
// run across lanes (shfl_xor), strides >= 32 inside a lane.  The stages run in
// ascending stride order with (a + b, a - b) per butterfly, which is the exact
// sequence of roundings of the reference's fht_float, so the projections are
// bit-identical to the CPU path.
//
// Numerical contract of the transform (the oracle's and the shim's): the norm
// and the sum are sequential over ascending index, computed by one thread per
// point (k_colstats); the division is IEEE round-to-nearest.
#include "common.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace sdb {
namespace {

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src));
}
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src));
}

// One thread per point: Cosine norm (sequential fmaf of squares) or Chi2/JS
// column sum (sequential adds), plus the reference's input checks
// (src/Utilities.h:308-324) and a finiteness check.  The CTA's 256 rows are
// staged through shared memory 32 dimensions at a time (coalesced 128-byte
// row segments, transposed so each thread reads its own point's column
// without bank conflicts); each thread then runs its point's sequential chain.
constexpr int kCsPoints = 256, kCsDims = 32;

// Points [pBase, pEnd).
__global__ void __launch_bounds__(kCsPoints) k_colstats(const float* __restrict__ X, int ldx, int pBase, int n, int d,
                                                        int dist, float* __restrict__ scale, int32_t* __restrict__ err) {
    __shared__ float tile[kCsDims][kCsPoints + 1];
    const int p0 = pBase + blockIdx.x * kCsPoints;
    const int p = p0 + threadIdx.x;
    float s = 0.0f;
    bool neg = false, nonfinite = false;
    for (int c0 = 0; c0 < d; c0 += kCsDims) {
        __syncthreads();
        // 256 rows x 32 dims: each warp loads rows with lanes along the dims
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int row = w; row < kCsPoints; row += kCsPoints / 32) {
            const int pr = p0 + row, c = c0 + lane;
            tile[lane][row] = (pr < n && c < d) ? __ldcs(X + (size_t)pr * ldx + c) : 0.0f;
        }
        __syncthreads();
        const int cn = min(kCsDims, d - c0);
        if (dist == DIST_COSINE) {
            for (int i = 0; i < cn; ++i) {
                const float t = tile[i][threadIdx.x];
                nonfinite |= !isfinite(t);
                s = __fmaf_rn(t, t, s);
            }
        } else if (dist == DIST_CHI2 || dist == DIST_JS) {
            for (int i = 0; i < cn; ++i) {
                const float t = tile[i][threadIdx.x];
                nonfinite |= !isfinite(t);
                neg |= t < 0.0f;
                s = __fadd_rn(s, t);
            }
        } else {
            for (int i = 0; i < cn; ++i) nonfinite |= !isfinite(tile[i][threadIdx.x]);
        }
    }
    if (p >= n) return;
    if (dist == DIST_COSINE) {
        s = __fsqrt_rn(s);
        if (!(s > 0.0f)) atomicExch(err + 1, 1);
    } else if (dist == DIST_CHI2 || dist == DIST_JS) {
        if (neg) atomicExch(err + 0, 1);
        else if (!(s > 0.0f)) atomicExch(err + 1, 1);
    } else {
        s = 1.0f;
    }
    if (nonfinite) atomicExch(err + 2, 1);
    scale[p] = s;
}

// Element e of the Chi2 / JS embedding (src/Utilities.h:132-208) of a
// transformed row (row: d values): sqrt terms for e < d, then the cos / sin
// components; zero for e >= ker (the padding up to fhtDim).
__device__ float embed_chi2js(const ProjectArgs& a, const float* row, int e) {
    float t = 0.0f;
    if (e >= a.ker) return t;
    const float L = a.kerSam;
    if (e < a.d) {
        const float xv = row[e];
        if (xv > 0.0f) {
            if (a.dist == DIST_CHI2) t = __fsqrt_rn(__fmul_rn(xv, L));
            else t = (float)__dsqrt_rn(__ddiv_rn(__dmul_rn((double)__fmul_rn(xv, L), 2.0), a.ln4));
        }
        return t;
    }
    const int comps = ((a.ker / a.d) - 1) / 2;
    const int q = e - a.d;
    const int c = q / (2 * a.d) + 1;  // component index
    const int r = q % (2 * a.d);
    const int i = r % a.d;
    const bool isSin = r >= a.d;
    const float xv = row[i];
    if (c <= comps && xv > 0.0f) {
        float f;
        const double ch = a.compCosh[c - 1];  // cosh(PI*c*L), computed on the host
        if (a.dist == DIST_CHI2) {
            f = (float)__dsqrt_rn(__ddiv_rn(__dmul_rn(__dmul_rn(2.0, (double)xv), (double)L), ch));
        } else {
            const float cl = __fmul_rn((float)c, L);
            const float qq = __fadd_rn(1.0f, __fmul_rn(__fmul_rn(4.0f, cl), cl));
            f = (float)__ddiv_rn(2.0, __dmul_rn(__dmul_rn(a.ln4, (double)qq), ch));
            f = (float)__dsqrt_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, (double)xv), (double)L), (double)f));
        }
        const float ang = __fmul_rn(__fmul_rn((float)c, L), logf(xv));
        t = __fmul_rn(f, isSin ? sinf(ang) : cosf(ang));
    }
    return t;
}

// Warp bitonic sort of 32 u64 keys, one per lane, into descending lane order.
__device__ __forceinline__ uint64_t warp_sort_desc(uint64_t x) {
    const unsigned l = lane_id();
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const uint64_t o = shfl_xor_u64(x, stride);
            const bool up = ((l & size) == 0);          // descending blocks where bit `size` clear
            const bool lower = ((l & stride) == 0);
            const bool keep_max = (up == lower);
            x = keep_max ? (o > x ? o : x) : (o < x ? o : x);
        }
    }
    return x;
}

// 32-bit warp bitonic sort, one key per lane, descending in lane order.
__device__ __forceinline__ uint32_t warp_sort_desc_u32(uint32_t x) {
    const unsigned l = lane_id();
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const uint32_t o = __shfl_xor_sync(0xffffffffu, x, stride);
            const bool keep_max = ((l & size) == 0) == ((l & stride) == 0);
            x = keep_max ? max(o, x) : min(o, x);
        }
    }
    return x;
}

// Top-(k+1) of the warp's keys (key[j] for element l + 32 j, 0 for elements
// past nproj; every real key is > 0).  Writes the k winners in descending
// order to out[0..k) and returns whether the k-th and (k+1)-th values tie.
// Ties between equal values break toward the smaller vector index.
//   Fast path: T = the (k+1)-th largest lane maximum is attained by k+1
//   different elements, so every winner has key >= T; the (usually few)
//   candidates >= T are compacted and sorted in one warp sort.
//   Fallback (more than 32 candidates, e.g. many equal values): repeated
//   warp argmax.
template <int NJ>
__device__ bool warp_topk(const uint32_t (&key)[NJ], int nproj, int k, int32_t* out, uint64_t* sbuf) {
    const unsigned l = lane_id();
    const int want = k + 1 <= nproj ? k + 1 : k;
    if (want <= 32) {
        uint32_t lm = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) lm = max(lm, key[j]);
        const uint32_t T = __shfl_sync(0xffffffffu, warp_sort_desc_u32(lm), want - 1);
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) cnt += key[j] >= T ? 1 : 0;
        int incl = cnt;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, incl, s);
            if ((int)l >= s) incl += o;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total <= 32) {
            int pos = incl - cnt;
#pragma unroll
            for (int j = 0; j < NJ; ++j)
                if (key[j] >= T)
                    sbuf[pos++] = ((uint64_t)key[j] << 32) | (uint64_t)(0xffffffffu - (uint32_t)(l + 32 * j));
            __syncwarp();
            const uint64_t mine = (int)l < total ? sbuf[l] : 0ull;
            __syncwarp();
            const uint64_t s = warp_sort_desc(mine);
            if ((int)l < k) out[l] = (int32_t)(0xffffffffu - (uint32_t)s);
            const uint64_t a = __shfl_sync(0xffffffffu, s, k - 1);
            const uint64_t b = __shfl_sync(0xffffffffu, s, want - 1);
            return want > k && (uint32_t)(a >> 32) == (uint32_t)(b >> 32);
        }
    }
    uint64_t taken = 0;  // bit j: element l + 32 j already selected
    uint32_t prev = 0, last = 0;
    for (int it = 0; it < want; ++it) {
        uint64_t best = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            if (key[j] && !((taken >> j) & 1ull)) {
                const uint64_t pk = ((uint64_t)key[j] << 32) | (uint64_t)(0xffffffffu - (uint32_t)(l + 32 * j));
                best = pk > best ? pk : best;
            }
        }
        best = warp_max_u64(best);
        const int e = (int)(0xffffffffu - (uint32_t)best);
        if ((e & 31) == (int)l) taken |= 1ull << (e >> 5);
        if (it < k) {
            if (l == 0) out[it] = e;
            prev = (uint32_t)(best >> 32);
        } else {
            last = (uint32_t)(best >> 32);
        }
    }
    return want > k && prev == last;
}

template <int NJ, int EMB>
__global__ void __launch_bounds__(128, (NJ >= 64 ? 1 : 6)) k_project(ProjectArgs a, const float* __restrict__ scale) {
    extern __shared__ float smem[];
    const int warps = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const unsigned l = lane_id();
    const int FD = a.fhtDim;
    const int nsw = (3 * FD + 31) / 32;
    uint64_t* sbuf = reinterpret_cast<uint64_t*>(smem) + w * 32;     // per-warp top-k candidates
    uint32_t* sw = reinterpret_cast<uint32_t*>(smem + warps * 64);   // sign words
    const int rowLen = EMB == 2 ? ((a.d + 3) & ~3) + FD : 0;
    float* base = smem + warps * 64 + ((nsw + 3) & ~3);
    float* rowbuf = base + w * rowLen;                                // per-warp copy of the row (Chi2/JS)
    // per-warp running (max v, max -v) per vector, bf16x2 rounded toward -inf
    __nv_bfloat162* ext = reinterpret_cast<__nv_bfloat162*>(base + warps * rowLen) + (size_t)w * a.nproj;
    const int gEnd = a.chunkEnd > 0 ? a.chunkEnd : (a.n + a.chunk - 1) / a.chunk;
    int g = a.chunkBase + blockIdx.x;  // the block's current chunk of points
    // per-warp input row buffer: the next point's row is fetched with
    // cp.async as soon as the current one has been read, so it lands while
    // the current point's rotations and top-k run (one buffer instead of two
    // leaves room for six blocks per SM)
    const int xs = (a.d + 3) & ~3;
    float* xbuf = base + warps * rowLen + warps * a.nproj + (size_t)w * xs;
    // 16-byte copies need whole 16-byte rows: L1 / L2 pass the padded Xt
    // (ldx = ld, a multiple of 4) with any d, and d / 4 chunks would then
    // leave the row's last d % 4 elements unstaged
    const bool vec16 = (a.ldx & 3) == 0 && (a.d & 3) == 0 && (reinterpret_cast<uintptr_t>(a.X) & 15) == 0;
    auto fetch = [&](int pp) {
        if (pp < min(a.n, (g + 1) * a.chunk)) {
            const float* src = a.X + (size_t)pp * a.ldx;
            float* dst = xbuf;
            if (vec16) {
                for (int c = (int)l; c < a.d / 4; c += 32) cp_async16(dst + 4 * c, src + 4 * c);
            } else {
                for (int e = (int)l; e < a.d; e += 32) cp_async4(dst + e, src + e);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };
    for (int i = threadIdx.x; i < nsw; i += blockDim.x) sw[i] = a.signs[i];
    __syncthreads();
    // Lane l's sign bits for its elements e = l + 32 j, one 32-bit mask per
    // round (bit j): a set bit keeps the value, a clear bit negates it.
    uint64_t laneSigns[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        uint64_t msk = 0;
        for (int j = 0; j < NJ; ++j) {
            const int e = (int)l + 32 * j;
            if (e < FD) msk |= (uint64_t)((sw[(r * FD + e) >> 5] >> ((r * FD + e) & 31)) & 1u) << j;
        }
        laneSigns[r] = msk;
    }

    int localTies = 0;
    // the block's chunks, grid-stride
    for (; g < gEnd; g += gridDim.x) {
    // Per vector: (max v, max -v) over the warp's points, as bf16 rounded
    // toward -inf.  A rounded-down maximum is still a lower bound on a value
    // attained by a point of the chunk, which is all the top-m threshold needs.
    for (int e = (int)l; e < a.nproj; e += 32) ext[e] = __floats2bfloat162_rn(-INFINITY, -INFINITY);
    __syncwarp();
    const int p0 = g * a.chunk;
    const int p1 = min(a.n, p0 + a.chunk);
    fetch(p0 + w);
    for (int p = p0 + w; p < p1; p += warps) {
        const float sc = scale[p];
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncwarp();
        const float* x = xbuf;  // this point's input row, in shared memory
        // transformed row -> Xt (zero padded to ld)
        float v[NJ];
        if (EMB == 0) {
            // Cosine: the transformed row is the embedding; one division per
            // element, done in place on the warp's staged row by a rolled loop
            // (32 unrolled divisions made the body too large for the
            // instruction cache: 9.3 -> 8.2 ms at 1M x 784)
            if (a.do_transform) {
                float* xw = xbuf;
#pragma unroll 1
                for (int e = (int)l; e < a.d; e += 32) xw[e] = __fdiv_rn(xw[e], sc);
                __syncwarp();
            }
            // Xt row, zero padded to ld (a multiple of 4), 16 bytes per lane
            // from the staged row; the staged chunk holding element d - 1 is
            // the last one read, its elements past d are zeroed
            {
                const float4* x4 = reinterpret_cast<const float4*>(x);
                float4* xt4 = reinterpret_cast<float4*>(a.Xt + (size_t)p * a.ld);
#pragma unroll 1
                for (int c = (int)l; c < a.ld / 4; c += 32) {
                    float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (4 * c < a.d) {
                        t = x4[c];
                        if (4 * c + 1 >= a.d) t.y = 0.0f;
                        if (4 * c + 2 >= a.d) t.z = 0.0f;
                        if (4 * c + 3 >= a.d) t.w = 0.0f;
                    }
                    xt4[c] = t;
                }
            }
            // the tensor-core copy (BF16, zero padded to ldb), 8 values per lane store
            if (a.Xb) {
                uint4* xb8 = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.Xb) + (size_t)p * a.ldb);
#pragma unroll 1
                for (int c = (int)l; c < a.ldb / 8; c += 32) {
                    float f[8];
                    if (8 * c + 8 <= a.d) {
                        const float4 lo = reinterpret_cast<const float4*>(x)[2 * c];
                        const float4 hi = reinterpret_cast<const float4*>(x)[2 * c + 1];
                        f[0] = lo.x; f[1] = lo.y; f[2] = lo.z; f[3] = lo.w;
                        f[4] = hi.x; f[5] = hi.y; f[6] = hi.z; f[7] = hi.w;
                    } else {
#pragma unroll
                        for (int u = 0; u < 8; ++u) f[u] = 8 * c + u < a.d ? x[8 * c + u] : 0.0f;
                    }
                    uint4 o;
                    __nv_bfloat162 b;
                    b = __floats2bfloat162_rn(f[0], f[1]); o.x = *reinterpret_cast<uint32_t*>(&b);
                    b = __floats2bfloat162_rn(f[2], f[3]); o.y = *reinterpret_cast<uint32_t*>(&b);
                    b = __floats2bfloat162_rn(f[4], f[5]); o.z = *reinterpret_cast<uint32_t*>(&b);
                    b = __floats2bfloat162_rn(f[6], f[7]); o.w = *reinterpret_cast<uint32_t*>(&b);
                    xb8[c] = o;
                }
            }
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
                const int e = (int)l + 32 * j;
                v[j] = e < a.d ? x[e] : 0.0f;
            }
        }
        for (int i = (int)l; EMB != 0 && i < a.ld; i += 32) {
            float t = 0.0f;
            if (i < a.d) {
                t = x[i];
                if (a.do_transform && EMB != 1) t = __fdiv_rn(t, sc);
            }
            a.Xt[(size_t)p * a.ld + i] = t;
            if (EMB == 2 && i < a.d) rowbuf[i] = t;
        }
        __syncwarp();        // every lane is done with the staged row
        fetch(p + warps);    // the next point's row
        if (EMB == 2) {
            // Chi2 / JS embedding (src/Utilities.h:132-208) into the warp's row
            // buffer, lane-strided, then picked up per register below.
            __syncwarp();
            float* emb = rowbuf + ((a.d + 3) & ~3);
            for (int e = (int)l; e < FD; e += 32) emb[e] = embed_chi2js(a, rowbuf, e);
            __syncwarp();
        }
#pragma unroll
        for (int j = 0; j < NJ && EMB != 0; ++j) {
            const int e = (int)l + 32 * j;
            float t = 0.0f;
            if (EMB == 1) {
                if (e < a.ker) t = a.E[(size_t)p * a.ker + e];
            } else {
                if (e < FD) t = rowbuf[((a.d + 3) & ~3) + e];
            }
            v[j] = t;
        }
        if (EMB == 2) __syncwarp();
        // three rounds: random signs, then the Walsh-Hadamard transform
#pragma unroll 1
        for (int r = 0; r < 3; ++r) {
            const uint64_t sgn = ~laneSigns[r];  // bit j set: negate element j
#pragma unroll
            for (int j = 0; j < NJ; ++j)
                v[j] = __int_as_float(__float_as_int(v[j]) ^ (int)((uint32_t)((sgn >> j) & 1u) << 31));
            // (a rolled loop over the five cross-lane strides keeps the per-point
            // loop body small: the kernel's top stall is instruction fetch)
#pragma unroll 1
            for (int s = 1; s < 32 && s < FD; s <<= 1) {
                // lower element a: a + b; upper element b: a - b, i.e. fma(-1, b, a),
                // exactly the reference's rounding either way
                const float mul = (l & s) ? -1.0f : 1.0f;
#pragma unroll
                for (int j = 0; j < NJ; ++j) {
                    const float o = __shfl_xor_sync(0xffffffffu, v[j], s);
                    v[j] = __fmaf_rn(mul, v[j], o);
                }
            }
#pragma unroll
            for (int h = 1; h < NJ; h <<= 1) {
#pragma unroll
                for (int j = 0; j < NJ; ++j) {
                    if ((j & h) == 0) {
                        const float x0 = v[j], x1 = v[j + h];
                        v[j] = __fadd_rn(x0, x1);
                        v[j + h] = __fsub_rn(x0, x1);
                    }
                }
            }
        }
        // projections (the first nproj entries) and per-vector chunk extremes
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int e = (int)l + 32 * j;
            if (e < a.nproj) {
                a.P[(size_t)p * a.nproj + e] = v[j];
                __nv_bfloat162 b;
                b.x = __float2bfloat16_rd(v[j]);
                b.y = __float2bfloat16_rd(-v[j]);
                ext[e] = __hmax2(ext[e], b);
            }
        }
        // top-k on order-preserving keys; the far side's keys are the
        // complements (the order of -v), so one key array serves both sides
        uint32_t key[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) key[j] = ((int)l + 32 * j) < a.nproj ? key_of(v[j]) : 0u;
        int32_t* tk = a.topK + (size_t)p * 2 * a.k;
#pragma unroll 1
        for (int side = 0; side < 2; ++side) {
            localTies += warp_topk<NJ>(key, a.nproj, a.k, tk + side * a.k, sbuf) ? 1 : 0;
#pragma unroll
            for (int j = 0; j < NJ; ++j) key[j] = key[j] ? ~key[j] : 0u;
        }
        __syncwarp();
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // chunk extremes: reduce the warps' rows
    __syncthreads();
    const __nv_bfloat162* ext0 = reinterpret_cast<const __nv_bfloat162*>(base + warps * rowLen);
    for (int e = threadIdx.x; e < a.nproj; e += blockDim.x) {
        __nv_bfloat162 m2 = ext0[e];
        for (int ww = 1; ww < warps; ++ww) m2 = __hmax2(m2, ext0[(size_t)ww * a.nproj + e]);
        a.chunkMax[(size_t)g * a.nproj + e] = __bfloat162float(m2.x);
        a.chunkMin[(size_t)g * a.nproj + e] = -__bfloat162float(m2.y);
    }
    __syncthreads();  // the warps' extremes are re-initialised for the next chunk
    }  // chunks
    if (l == 0 && localTies) atomicAdd(a.ties, (unsigned long long)localTies);
}

// Stage 1 for fhtDim > 2048 (d or ker_n_features above 2048), where the
// rotation vector no longer fits a warp's registers: a CTA per point at a
// time, the vector in shared memory.  Same arithmetic as k_project: the
// transform, the embedding, three rounds of sign flips and FWHT stages in
// ascending stride order with (a + b, a - b) per butterfly (the pairs of a
// stage are independent, so their order does not change the bits), then the
// top-k of each side by repeated block-wide argmax (ties toward the smaller
// index, boundary ties counted) and the chunk extremes.
constexpr int kBigThreads = 256;

__device__ __forceinline__ uint64_t block_max_u64(uint64_t v, uint64_t* red) {
    v = warp_max_u64(v);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        uint64_t x = (int)threadIdx.x < kBigThreads / 32 ? red[threadIdx.x] : 0ull;
        x = warp_max_u64(x);
        if (threadIdx.x == 0) red[kBigThreads / 32] = x;
    }
    __syncthreads();
    const uint64_t r = red[kBigThreads / 32];
    __syncthreads();
    return r;
}

template <int EMB>
__global__ void __launch_bounds__(kBigThreads) k_project_smem(ProjectArgs a, const float* __restrict__ scale) {
    extern __shared__ float smem[];
    const int FD = a.fhtDim;
    const int ldr = (a.d + 3) & ~3;
    float* v = smem;                                          // FD
    float* row = v + FD;                                      // ldr: the transformed row
    __nv_bfloat162* ext = reinterpret_cast<__nv_bfloat162*>(row + ldr);  // nproj
    uint32_t* taken = reinterpret_cast<uint32_t*>(ext + a.nproj);        // nproj bits
    __shared__ uint64_t red[kBigThreads / 32 + 1];
    const int tid = threadIdx.x;
    const int gEnd = a.chunkEnd > 0 ? a.chunkEnd : (a.n + a.chunk - 1) / a.chunk;
    int localTies = 0;
    for (int g = a.chunkBase + blockIdx.x; g < gEnd; g += gridDim.x) {
        for (int e = tid; e < a.nproj; e += kBigThreads) ext[e] = __floats2bfloat162_rn(-INFINITY, -INFINITY);
        const int p0 = g * a.chunk, p1 = min(a.n, p0 + a.chunk);
        for (int p = p0; p < p1; ++p) {
            const float sc = scale[p];
            // transformed row -> Xt (zero padded to ld) and the embedding -> v
            for (int i = tid; i < a.ld; i += kBigThreads) {
                float t = 0.0f;
                if (i < a.d) {
                    t = __ldg(a.X + (size_t)p * a.ldx + i);
                    if (a.do_transform && EMB != 1) t = __fdiv_rn(t, sc);
                }
                a.Xt[(size_t)p * a.ld + i] = t;
                if (i < ldr) row[i] = t;
            }
            __syncthreads();
            for (int e = tid; e < FD; e += kBigThreads) {
                float t = 0.0f;
                if (EMB == 0) t = e < a.d ? row[e] : 0.0f;
                else if (EMB == 1) t = e < a.ker ? a.E[(size_t)p * a.ker + e] : 0.0f;
                else t = embed_chi2js(a, row, e);
                v[e] = t;
            }
            __syncthreads();
            for (int r = 0; r < 3; ++r) {
                for (int e = tid; e < FD; e += kBigThreads)  // a clear sign bit negates the element
                    if (!((a.signs[(r * FD + e) >> 5] >> ((r * FD + e) & 31)) & 1u)) v[e] = -v[e];
                __syncthreads();
                for (int st = 1; st < FD; st <<= 1) {
                    for (int b = tid; b < FD / 2; b += kBigThreads) {
                        const int i = (b / st) * 2 * st + (b % st);
                        const float x0 = v[i], x1 = v[i + st];
                        v[i] = __fadd_rn(x0, x1);
                        v[i + st] = __fsub_rn(x0, x1);
                    }
                    __syncthreads();
                }
            }
            for (int e = tid; e < a.nproj; e += kBigThreads) {
                const float x = v[e];
                a.P[(size_t)p * a.nproj + e] = x;
                __nv_bfloat162 b;
                b.x = __float2bfloat16_rd(x);
                b.y = __float2bfloat16_rd(-x);
                ext[e] = __hmax2(ext[e], b);
            }
            // top-k per side: (key, smaller index) maxima, k + 1 rounds for the tie test
            const int want = a.k + 1 <= a.nproj ? a.k + 1 : a.k;
            for (int side = 0; side < 2; ++side) {
                for (int e = tid; e < (a.nproj + 31) / 32; e += kBigThreads) taken[e] = 0u;
                __syncthreads();
                uint32_t kth = 0, last = 0;
                for (int it = 0; it < want; ++it) {
                    uint64_t best = 0;
                    for (int e = tid; e < a.nproj; e += kBigThreads) {
                        if ((taken[e >> 5] >> (e & 31)) & 1u) continue;
                        uint32_t key = key_of(v[e]);
                        if (side) key = ~key;
                        const uint64_t pk = ((uint64_t)key << 32) | (uint64_t)(0xffffffffu - (uint32_t)e);
                        best = pk > best ? pk : best;
                    }
                    best = block_max_u64(best, red);
                    const int e = (int)(0xffffffffu - (uint32_t)best);
                    if (tid == 0) {
                        taken[e >> 5] |= 1u << (e & 31);
                        if (it < a.k) a.topK[(size_t)p * 2 * a.k + side * a.k + it] = e;
                    }
                    if (it == a.k - 1) kth = (uint32_t)(best >> 32);
                    if (it == a.k) last = (uint32_t)(best >> 32);
                    __syncthreads();
                }
                if (want > a.k && kth == last && tid == 0) ++localTies;
            }
            __syncthreads();
        }
        for (int e = tid; e < a.nproj; e += kBigThreads) {
            a.chunkMax[(size_t)g * a.nproj + e] = __bfloat162float(ext[e].x);
            a.chunkMin[(size_t)g * a.nproj + e] = -__bfloat162float(ext[e].y);
        }
        __syncthreads();
    }
    if (tid == 0 && localTies) atomicAdd(a.ties, (unsigned long long)localTies);
}

template <int EMB>
int launch_project_smem(const ProjectArgs& a, const float* scale, cudaStream_t st) {
    const int G = (a.chunkEnd > 0 ? a.chunkEnd : (a.n + a.chunk - 1) / a.chunk) - a.chunkBase;
    if (G <= 0) return 0;
    const size_t sm = sizeof(float) * ((size_t)a.fhtDim + ((a.d + 3) & ~3)) + 4 * (size_t)a.nproj +
                      4 * (size_t)((a.nproj + 31) / 32);
    if (sm > 227 * 1024) return -1;
    if (cudaFuncSetAttribute(k_project_smem<EMB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess)
        return -1;
    k_project_smem<EMB><<<std::min(G, sm_count() * 2), kBigThreads, sm, st>>>(a, scale);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// transformData alone (src/Utilities.h:289-335) for the fits that use no
// projections (sngDbscan / sngOptics): Xt[p][e] = X[p][e] / scale[p] for
// Cosine (norm) and Chi2 / JS (sum), X[p][e] for L1 / L2, zero past d up to
// ld.  A warp per row, four elements per lane access (16-byte loads and
// stores when the rows are 16-byte aligned), rows grid-stride.
__global__ void k_transform_rows(const float* __restrict__ X, int ldx, int n, int d, int ld, int dist,
                                 const float* __restrict__ scale, float* __restrict__ Xt) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const bool divide = dist == DIST_COSINE || dist == DIST_CHI2 || dist == DIST_JS;
    const bool vec = (ldx & 3) == 0 && (d & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += warps) {
        const float sc = divide ? scale[p] : 1.0f;
        const float* x = X + (size_t)p * ldx;
        float* y = Xt + (size_t)p * ld;
        for (int e = lane * 4; e < ld; e += 128) {  // ld is a multiple of 4
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (vec && e + 3 < d) {
                v = __ldg(reinterpret_cast<const float4*>(x + e));
            } else {
                if (e < d) v.x = __ldg(x + e);
                if (e + 1 < d) v.y = __ldg(x + e + 1);
                if (e + 2 < d) v.z = __ldg(x + e + 2);
                if (e + 3 < d) v.w = __ldg(x + e + 3);
            }
            if (divide) {  // padding stays 0 (0 / sc = 0 for the sc > 0 the checks allow)
                v.x = e < d ? __fdiv_rn(v.x, sc) : 0.0f;
                v.y = e + 1 < d ? __fdiv_rn(v.y, sc) : 0.0f;
                v.z = e + 2 < d ? __fdiv_rn(v.z, sc) : 0.0f;
                v.w = e + 3 < d ? __fdiv_rn(v.w, sc) : 0.0f;
            }
            *reinterpret_cast<float4*>(y + e) = v;
        }
    }
}

template <int NJ, int EMB>
int launch_project_nje(const ProjectArgs& a, const float* scale, cudaStream_t st) {
    const int warps = 4;
    const int G = (a.chunkEnd > 0 ? a.chunkEnd : (a.n + a.chunk - 1) / a.chunk) - a.chunkBase;
    if (G <= 0) return 0;
    // one full wave of 6 blocks per SM; the blocks walk the launch's chunks grid-stride
    const int grid = std::min(G, project_wave_chunks());
    const int nsw = (3 * a.fhtDim + 31) / 32;
    const int rowLen = EMB == 2 ? ((a.d + 3) & ~3) + a.fhtDim : 0;
    const size_t xs = (size_t)((a.d + 3) & ~3);
    size_t sm = sizeof(float) * (warps * 64 + ((nsw + 3) & ~3) + (size_t)warps * rowLen + (size_t)warps * a.nproj +
                                 (size_t)warps * xs);
    if (sm > 227 * 1024) return -1;
    if (sm > 48 * 1024) {
        if (cudaFuncSetAttribute(k_project<NJ, EMB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
            cudaSuccess)
            return -1;
    }
    k_project<NJ, EMB><<<grid, warps * 32, sm, st>>>(a, scale);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <int NJ>
int launch_project_nj(const ProjectArgs& a, const float* scale, cudaStream_t st) {
    if (a.dist == DIST_COSINE) return launch_project_nje<NJ, 0>(a, scale, st);
    if (a.dist == DIST_L1 || a.dist == DIST_L2) return launch_project_nje<NJ, 1>(a, scale, st);
    return launch_project_nje<NJ, 2>(a, scale, st);
}

}  // namespace

int launch_project(const ProjectArgs& a, cudaStream_t st) {
    float* scale = a.scale;
    // the BF16 copy is written by the register kernels' Cosine path only
    if (a.Xb && (a.dist != DIST_COSINE || a.fhtDim > 2048 || a.ldb > a.fhtDim)) return -1;
    const int G = (a.n + a.chunk - 1) / a.chunk;
    const int pb = a.chunkBase * a.chunk, pe = std::min(a.n, (a.chunkEnd > 0 ? a.chunkEnd : G) * a.chunk);
    if (pe > pb)
        k_colstats<<<(pe - pb + kCsPoints - 1) / kCsPoints, kCsPoints, 0, st>>>(a.X, a.ldx, pb, pe, a.d, a.dist,
                                                                               scale, a.err);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    int r;
    switch (a.fhtDim) {
        case 16:
        case 32: r = launch_project_nj<1>(a, scale, st); break;
        case 64: r = launch_project_nj<2>(a, scale, st); break;
        case 128: r = launch_project_nj<4>(a, scale, st); break;
        case 256: r = launch_project_nj<8>(a, scale, st); break;
        case 512: r = launch_project_nj<16>(a, scale, st); break;
        case 1024: r = launch_project_nj<32>(a, scale, st); break;
        case 2048: r = launch_project_nj<64>(a, scale, st); break;
        default:
            if (a.fhtDim < 4096) return -1;
            if (a.dist == DIST_COSINE) r = launch_project_smem<0>(a, scale, st);
            else if (a.dist == DIST_L1 || a.dist == DIST_L2) r = launch_project_smem<1>(a, scale, st);
            else r = launch_project_smem<2>(a, scale, st);
    }
    return r < 0 ? -1 : r + 1;
}

int launch_transform(const ProjectArgs& a, cudaStream_t st) {
    if (a.n <= 0) return 0;
    k_colstats<<<(a.n + kCsPoints - 1) / kCsPoints, kCsPoints, 0, st>>>(a.X, a.ldx, 0, a.n, a.d, a.dist, a.scale,
                                                                        a.err);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    if (a.ld & 3) return -1;
    const int grid = (int)std::min<int64_t>(((int64_t)a.n + 7) / 8, (int64_t)sm_count() * 16);
    k_transform_rows<<<grid, 256, 0, st>>>(a.X, a.ldx, a.n, a.d, a.ld, a.dist, a.scale, a.Xt);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

}  // namespace sdb
