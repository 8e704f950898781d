// Random Fourier features for L1 / L2 (src/sDbscan.cpp:22-28, :59-64):
//   v = R x  (R: h x d, h = ker/2),   embed = [cos v, sin v].
// FP32 GEMM, one fmaf per dimension in ascending order per output (the
// order of the oracle's matrix-vector product).  R is passed transposed
// (h rows of d floats, row stride ld) so both operands stream row-wise.
#include "common.cuh"

namespace sdb {
namespace {

constexpr int TM = 128, TN = 64, TK = 32, LDS = TK + 4, STAGES = 3, NT = 256;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 16 : 0));
}

__global__ void __launch_bounds__(NT, 2)
    k_rff(const float* __restrict__ X, int ld, int n, int d, const float* __restrict__ Rt, int h, float* __restrict__ E,
          const int32_t* __restrict__ gate) {
    if (gate != nullptr && __ldg(gate) == 0) return;  // the tensor-core embedding succeeded
    extern __shared__ __align__(16) float sm[];
    float* As = sm;
    float* Bs = As + STAGES * TM * LDS;
    const int tid = threadIdx.x;
    const int p0 = blockIdx.x * TM, r0 = blockIdx.y * TN;
    const int nk = (d + TK - 1) / TK;
    auto load_stage = [&](int stage, int kc) {
        float* as = As + stage * TM * LDS;
        float* bs = Bs + stage * TN * LDS;
        const int k0 = kc * TK;
#pragma unroll
        for (int it = 0; it < 4; ++it) {
            const int idx = tid + it * NT, row = idx >> 3, c4 = idx & 7;
            const int p = p0 + row, col = k0 + c4 * 4;
            const bool ok = p < n && col < ld;
            cp_async16(as + row * LDS + c4 * 4, ok ? X + (size_t)p * ld + col : X, ok);
        }
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const int idx = tid + it * NT, row = idx >> 3, c4 = idx & 7;
            const int r = r0 + row, col = k0 + c4 * 4;
            const bool ok = r < h && col < ld;
            cp_async16(bs + row * LDS + c4 * 4, ok ? Rt + (size_t)r * ld + col : Rt, ok);
        }
    };
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    const int ty = tid >> 4, tx = tid & 15;
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nk) load_stage(s, s);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    for (int kc = 0; kc < nk; ++kc) {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(STAGES - 2));
        __syncthreads();
        const int nxt = kc + STAGES - 1;
        if (nxt < nk) load_stage(nxt % STAGES, nxt);
        asm volatile("cp.async.commit_group;\n" ::);
        const float* as = As + (kc % STAGES) * TM * LDS;
        const float* bs = Bs + (kc % STAGES) * TN * LDS;
#pragma unroll
        for (int kk = 0; kk < TK; kk += 4) {
            float4 av[8], bv[4];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = *reinterpret_cast<const float4*>(as + (ty + 16 * i) * LDS + kk);
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = *reinterpret_cast<const float4*>(bs + (tx + 16 * j) * LDS + kk);
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float c = acc[i][j];
                    c = __fmaf_rn(bv[j].x, av[i].x, c);
                    c = __fmaf_rn(bv[j].y, av[i].y, c);
                    c = __fmaf_rn(bv[j].z, av[i].z, c);
                    c = __fmaf_rn(bv[j].w, av[i].w, c);
                    acc[i][j] = c;
                }
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int p = p0 + ty + 16 * i;
        if (p >= n) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = r0 + tx + 16 * j;
            if (r >= h) continue;
            float s, c;
            sincosf(acc[i][j], &s, &c);
            E[(size_t)p * 2 * h + r] = c;
            E[(size_t)p * 2 * h + h + r] = s;
        }
    }
}

}  // namespace

int launch_rff(const float* Xt, int ld, int n, int d, const float* Rt, int h, float* E, cudaStream_t st,
               const int32_t* gate) {
    const size_t sm = sizeof(float) * STAGES * (TM + TN) * LDS;
    if (cudaFuncSetAttribute(k_rff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return -1;
    dim3 grid((n + TM - 1) / TM, (h + TN - 1) / TN);
    k_rff<<<grid, NT, sm, st>>>(Xt, ld, n, d, Rt, h, E, gate);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
