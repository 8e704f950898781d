// sDbscan-1NN noise labelling (clusterNoise = 1; labelNoise,
// src/sDbscan.cpp:648-807): every point the clustering left as noise takes the
// label of the sampled core point whose projections best match its top-k
// random vectors.
//
//  - Sampling (:683-699): all core points when #cores < samplingProb n, else
//    each with probability fProb = samplingProb n / #cores (float arithmetic
//    as in the reference).  The reference draws with the unseeded rand(); here
//    point p is taken iff fmix32(seed + 0x9E3779B9 (p + 1)) 2^-32 <= fProb
//    (MurmurHash3's 32-bit finaliser), the oracle's rule as well.
//  - A sampled core's projection vector is its row of P (the reference
//    recomputes it with the same embedding and rotations, :711-760): the rows
//    are gathered into a vector-major copy PcT (n_proj x S) so that a random
//    vector's values over all sampled cores are contiguous (L2-resident).
//  - Per noise point x (a warp, lanes over the sampled cores): the estimate
//    sum_k PcT[close_k][i] - PcT[far_k][i], accumulated in the reference's
//    order (:786-793), and the first maximum over ascending core index
//    (:798-806, strict >); x takes that core's label.
// clusterNoise = 2 reads neighbour lists that fit_sDbscan has already cleared
// for non-core points (:379-391), so it leaves the labels unchanged.
#include "common.cuh"

namespace sdb {
namespace {

__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__global__ void k_count_cores(const uint8_t* __restrict__ core, int n, int32_t* __restrict__ numCore) {
    int c = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) c += core[p] ? 1 : 0;
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(numCore, c);
}

__global__ void k_noise_flags(NoiseArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > a.n) return;
    if (p == a.n) {
        a.sampleFlag[p] = 0;
        a.noiseFlag[p] = 0;
        return;
    }
    const int numCore = *a.numCore;
    float fProb = 1.0f;
    if ((float)numCore >= a.samplingProb * (float)a.n) fProb = a.samplingProb * (float)a.n / (float)numCore;
    bool take = false;
    if (a.core[p]) {
        const double u = (double)fmix32(a.seed + 0x9E3779B9u * (uint32_t)(p + 1)) * (1.0 / 4294967296.0);
        take = fProb == 1.0f || u <= (double)fProb;
    }
    a.sampleFlag[p] = take ? 1 : 0;
    a.noiseFlag[p] = a.labels[p] == -1 ? 1 : 0;
}

// After the exclusive scans: compact sampled cores (capped at sMax) and noise points.
__global__ void k_noise_compact(NoiseArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int64_t s = a.sampleFlag[p];
    if (a.sampleFlag[p + 1] > s && s < a.sMax) a.cores[s] = p;
    const int64_t q = a.noiseFlag[p];
    if (a.noiseFlag[p + 1] > q) a.noise[q] = p;
}

// PcT[r][i] = P[cores[i]][r], 32 x 32 tiles through shared memory.
__global__ void k_core_proj_t(NoiseArgs a) {
    __shared__ float tile[32][33];
    const int S = (int)min((int64_t)a.sMax, a.sampleFlag[a.n]);
    const int i0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    if (i0 >= S) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    for (int yy = ty; yy < 32; yy += 8) {
        const int i = i0 + yy, r = r0 + tx;
        tile[yy][tx] = (i < S && r < a.nproj) ? __ldg(a.P + (size_t)a.cores[i] * a.nproj + r) : 0.0f;
    }
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {
        const int r = r0 + yy, i = i0 + tx;
        if (r < a.nproj && i < S) a.PcT[(size_t)r * a.sMax + i] = tile[tx][yy];
    }
}

__global__ void k_noise_1nn(NoiseArgs a) {
    const int S = (int)min((int64_t)a.sMax, a.sampleFlag[a.n]);
    const int64_t nNoise = a.noiseFlag[a.n];
    if (S == 0) return;  // no cluster to join
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = w0; w < nNoise; w += nw) {
        const int x = a.noise[w];
        const int32_t* tk = a.topK + (size_t)x * 2 * a.k;
        float best = -2147483648.0f;  // NEG_INF (Header.h:20)
        int bi = -1;
        for (int i = lane; i < S; i += 32) {
            float v = 0.0f;
            for (int j = 0; j < a.k; ++j) {
                v = __fadd_rn(v, __ldg(a.PcT + (size_t)__ldg(tk + j) * a.sMax + i));
                v = __fsub_rn(v, __ldg(a.PcT + (size_t)__ldg(tk + j + a.k) * a.sMax + i));
            }
            if (v > best) {
                best = v;
                bi = i;
            }
        }
        // first maximum over the whole warp: larger value, then smaller index
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi >= 0 && (bi < 0 || ov > best || (ov == best && oi < bi))) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0 && bi >= 0) a.labels[x] = a.labels[a.cores[bi]];
    }
}

}  // namespace

int launch_label_noise(const NoiseArgs& a, cudaStream_t st) {
    int launches = 0;
    if (cudaMemsetAsync(a.numCore, 0, sizeof(int32_t), st) != cudaSuccess) return -1;
    k_count_cores<<<sm_count() * 4, 256, 0, st>>>(a.core, a.n, a.numCore);
    k_noise_flags<<<(a.n + 1 + 255) / 256, 256, 0, st>>>(a);
    launches += 2;
    int r = launch_scan_i64(a.sampleFlag, a.sampleFlag, (size_t)a.n + 1, a.scanTmp, st);
    if (r < 0) return -1;
    launches += r;
    r = launch_scan_i64(a.noiseFlag, a.noiseFlag, (size_t)a.n + 1, a.scanTmp, st);
    if (r < 0) return -1;
    launches += r;
    k_noise_compact<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    dim3 tg((a.sMax + 31) / 32, (a.nproj + 31) / 32);
    k_core_proj_t<<<tg, 256, 0, st>>>(a);
    k_noise_1nn<<<sm_count() * 8, 256, 0, st>>>(a);
    launches += 3;
    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

}  // namespace sdb
