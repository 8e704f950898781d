// Allocation-free per-vector top-m selection: sdb_topm_noalloc.
//
// Some callers cannot call cudaMalloc while they run this step: a serving
// loop that owns all of the GPU's memory through its own pool (and so has
// nothing left for the driver to hand out), code that must not take the
// implicit device synchronisation an allocation can cause, or code issued
// while a CUDA stream is being captured, where allocation calls are not
// permitted.  For them this entry point does the top-m stage of a fit
// (src/sDbscan.cpp:151-208) on projections the caller already holds in device
// memory, writing the caller's output buffer, and takes every byte of scratch
// from one file-scope __device__ array, g_topmScratch, below.
//
// Limits (from the fixed scratch size): n_proj <= 1024, topM <= 64.  The
// array (about 12 MiB) is reserved on every GPU that loads this library, for
// as long as the library stays loaded.  All calls share it: two calls that
// overlap on the GPU (different streams, or different host threads) race and
// must not be issued.  Each call zeroes the counters it needs, so successive
// calls do not see the previous call's state.  The boundary-tie count and the
// internal-error flag that a fit reports are kept in the array but not
// returned by this entry point.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/sdbscan_gb300.h"
#include "common.cuh"

namespace {

constexpr int kMaxProj = 1024;
constexpr int kMaxTopM = 64;
constexpr int kCap = 512;       // candidates per list (>= 8 * kMaxTopM)
constexpr int kMaxChunks = 512; // chunk extremes per vector
constexpr int kLists = 2 * kMaxProj;

// Scratch layout, in bytes from the start of the array.
constexpr size_t kOffCand = 0;                                                    // kLists * kCap u64
constexpr size_t kOffChunkMax = kOffCand + sizeof(uint64_t) * kLists * kCap;      // kMaxChunks * kMaxProj f32
constexpr size_t kOffChunkMin = kOffChunkMax + sizeof(float) * kMaxChunks * kMaxProj;
constexpr size_t kOffThr = kOffChunkMin + sizeof(float) * kMaxChunks * kMaxProj;  // 2 * kMaxProj f32
constexpr size_t kOffCount = kOffThr + sizeof(float) * 2 * kMaxProj;              // kLists i32
constexpr size_t kOffFlags = kOffCount + sizeof(int32_t) * kLists;                // 4 i32 + 2 u64
constexpr size_t kScratchBytes = kOffFlags + 64;

__device__ __align__(256) unsigned char g_topmScratch[kScratchBytes];

// Per-device address of g_topmScratch, looked up once per device.
std::mutex g_setupMutex;
void* g_scratchPtr[64] = {};

// Column maxima / minima of the projections over `chunk` consecutive points:
// the chunk extremes the top-m thresholds are built from.
__global__ void k_chunk_extremes(const float* __restrict__ P, int n, int nproj, int chunk, float* __restrict__ cmax,
                                 float* __restrict__ cmin) {
    const int g = blockIdx.x;
    const int p0 = g * chunk, p1 = min(n, p0 + chunk);
    for (int r = threadIdx.x; r < nproj; r += blockDim.x) {
        float mx = -INFINITY, mn = INFINITY;
        for (int p = p0; p < p1; ++p) {
            const float v = __ldg(P + (size_t)p * nproj + r);
            mx = fmaxf(mx, v);
            mn = fminf(mn, v);
        }
        cmax[(size_t)g * nproj + r] = mx;
        cmin[(size_t)g * nproj + r] = mn;
    }
}

}  // namespace

extern "C" sdb_status sdb_topm_noalloc(const float* proj_device, int32_t n_points, int32_t n_proj, int32_t topM,
                                       int32_t* topM_device, void* stream) {
    if (!proj_device || !topM_device || n_points < 1 || n_proj < 1 || topM < 1) return SDB_ERR_ARG;
    if (n_proj > kMaxProj || topM > kMaxTopM || topM > n_points) return SDB_ERR_ARG;
    // rows of a multiple of 4 projections are read as float4: the base must be
    // 16-byte aligned (an offset view of a larger buffer may not be)
    if (n_proj % 4 == 0 && reinterpret_cast<uintptr_t>(proj_device) % 16 != 0) return SDB_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SDB_ERR_CUDA;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        if (!g_scratchPtr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_topmScratch) != cudaSuccess || p == nullptr) {
                cudaGetLastError();
                return SDB_ERR_CUDA;
            }
            g_scratchPtr[dev] = p;
        }
        base = static_cast<unsigned char*>(g_scratchPtr[dev]);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int chunk = (n_points + kMaxChunks - 1) / kMaxChunks;
    const int G = (n_points + chunk - 1) / chunk;

    sdb::TopMArgs a{};
    a.P = proj_device;
    a.n = n_points;
    a.nproj = n_proj;
    a.m = topM;
    a.chunkMax = reinterpret_cast<float*>(base + kOffChunkMax);
    a.chunkMin = reinterpret_cast<float*>(base + kOffChunkMin);
    a.G = G;
    a.thrMax = reinterpret_cast<float*>(base + kOffThr);
    a.thrMin = a.thrMax + n_proj;
    a.cand = reinterpret_cast<uint64_t*>(base + kOffCand);
    a.candCount = reinterpret_cast<int32_t*>(base + kOffCount);
    a.cap = kCap;
    a.topM = topM_device;
    a.errFlag = reinterpret_cast<int32_t*>(base + kOffFlags);
    a.ties = reinterpret_cast<unsigned long long*>(base + kOffFlags + 16);
    // counters and flags must start at zero on every call
    if (cudaMemsetAsync(base + kOffCount, 0, sizeof(int32_t) * 2 * n_proj, st) != cudaSuccess ||
        cudaMemsetAsync(base + kOffFlags, 0, 64, st) != cudaSuccess)
        return SDB_ERR_CUDA;
    k_chunk_extremes<<<G, 256, 0, st>>>(proj_device, n_points, n_proj, chunk, const_cast<float*>(a.chunkMax),
                                         const_cast<float*>(a.chunkMin));
    if (cudaPeekAtLastError() != cudaSuccess) return SDB_ERR_CUDA;
    if (sdb::launch_topm_thresholds(a, st) < 0 || sdb::launch_topm_collect(a, st) < 0 ||
        sdb::launch_topm_select(a, st) < 0)
        return SDB_ERR_CUDA;
    return SDB_OK;
}
