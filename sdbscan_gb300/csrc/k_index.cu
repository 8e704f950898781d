// Stage 3: the inverted index that turns the reference's per-point candidate
// loop (src/sDbscan.cpp:243-359) into a grouped, gathered GEMM.
//
// List l = side * D + r is the candidate list topM[r][side] (side 0 = close,
// 1 = far).  Its members are the (point, slot) pairs whose top-k list holds r
// on that side: point p meets the m candidates of list l exactly when
// topK[p][slot] == r (src/sDbscan.cpp:262-270, :317-323).  Members of a list
// share the same m candidate rows, so the distance kernel keeps those rows in
// shared memory and streams the members past them.
//
// Hub lists: for every point, the top-m lists that contain it.  A point in no
// list ("non-hub") can never be a candidate of anyone, so its neighbourhood
// is exactly its own candidates within eps.
#include "common.cuh"

#include <algorithm>

namespace sdb {
namespace {

__device__ __forceinline__ int list_of(const int32_t* topK, int p, int slot, int k, int nproj) {
    return topK[(size_t)p * 2 * k + slot] + (slot >= k ? nproj : 0);
}

// Members are placed in point-chunk order: CTA c handles the points of chunk
// c ([c chunkPts, (c + 1) chunkPts)).  k_index_count writes each chunk's
// per-list counts (list-major, chunkOff[l][c]) and the list totals;
// k_chunk_scan turns every list's row into offsets; k_index_scatter places
// the chunk's members from those offsets (order inside a chunk is free).
__global__ void k_index_count(IndexArgs a) {
    extern __shared__ int hist[];
    const int L = 2 * a.nproj, c = blockIdx.x;
    for (int i = threadIdx.x; i < L; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const int p0 = c * a.chunkPts, p1 = min(a.n, p0 + a.chunkPts);
    const size_t q1 = (size_t)p1 * 2 * a.k;
    for (size_t q = (size_t)p0 * 2 * a.k + threadIdx.x; q < q1; q += blockDim.x) {
        const int p = (int)(q / (2 * a.k)), slot = (int)(q % (2 * a.k));
        atomicAdd(&hist[list_of(a.topK, p, slot, a.k, a.nproj)], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        a.chunkOff[(size_t)i * a.nChunks + c] = hist[i];
        if (hist[i]) atomicAdd(reinterpret_cast<unsigned long long*>(a.listCount) + i, (unsigned long long)hist[i]);
    }
}

// Warp per list: exclusive scan of its chunk counts, in place.
__global__ void k_chunk_scan(IndexArgs a) {
    const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (l >= 2 * a.nproj) return;
    int32_t* row = a.chunkOff + (size_t)l * a.nChunks;
    int run = 0;
    for (int c0 = 0; c0 < a.nChunks; c0 += 32) {
        const int c = c0 + lane;
        const int v = c < a.nChunks ? row[c] : 0;
        int incl = v;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, incl, s);
            if (lane >= s) incl += o;
        }
        if (c < a.nChunks) row[c] = run + incl - v;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
}

__global__ void k_index_scatter(IndexArgs a) {
    extern __shared__ int cursor[];
    const int L = 2 * a.nproj, c = blockIdx.x;
    for (int i = threadIdx.x; i < L; i += blockDim.x)
        cursor[i] = (int)a.listOff[i] + a.chunkOff[(size_t)i * a.nChunks + c];
    __syncthreads();
    const int p0 = c * a.chunkPts, p1 = min(a.n, p0 + a.chunkPts);
    const size_t q1 = (size_t)p1 * 2 * a.k;
    for (size_t q = (size_t)p0 * 2 * a.k + threadIdx.x; q < q1; q += blockDim.x) {
        const int p = (int)(q / (2 * a.k)), slot = (int)(q % (2 * a.k));
        const int pos = atomicAdd(&cursor[list_of(a.topK, p, slot, a.k, a.nproj)], 1);
        a.members[pos] = make_int2(p, slot);
    }
}

// Tile order: counting sort of the tiles by the chunk of their first member.
__global__ void k_tile_keys(IndexArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.tileOff[2 * a.nproj]) return;
    const int l = a.tileList[t];
    const int mt = (int)((t - a.tileOff[l]) / a.nct);
    const int key = a.members[a.listOff[l] + (int64_t)mt * a.TM].x / a.chunkPts;
    a.tileKey[t] = key;
    atomicAdd(reinterpret_cast<unsigned long long*>(a.keyOff) + key, 1ull);
}

// The tensor-core distance kernel's order: tiles by (super-chunk of their
// first member, list), a super-chunk being superChunk consecutive point
// chunks.  The rows of a super-chunk stay in L2 while every list passes over
// them, and the few tiles a list has there run back to back, so its candidate
// rows are read once per super-chunk.
__global__ void k_tile_keys_list(IndexArgs a, int superChunk, int32_t* keys, int64_t* keyOff) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.tileOff[2 * a.nproj]) return;
    const int l = a.tileList[t];
    const int mt = (int)((t - a.tileOff[l]) / a.nct);
    const int sc = a.members[a.listOff[l] + (int64_t)mt * a.TM].x / a.chunkPts / superChunk;
    const int key = sc * 2 * a.nproj + l;
    keys[t] = key;
    atomicAdd(reinterpret_cast<unsigned long long*>(keyOff) + key, 1ull);
}

__global__ void k_tile_perm_keys(IndexArgs a, const int32_t* keys, int64_t* keyOff, int32_t* perm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.tileOff[2 * a.nproj]) return;
    const unsigned long long pos = atomicAdd(reinterpret_cast<unsigned long long*>(keyOff) + keys[t], 1ull);
    perm[pos] = (int32_t)t;
}

__global__ void k_tile_perm(IndexArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.tileOff[2 * a.nproj]) return;
    const unsigned long long pos =
        atomicAdd(reinterpret_cast<unsigned long long*>(a.keyOff) + a.tileKey[t], 1ull);
    a.tilePerm[pos] = (int32_t)t;
}

// tiles per list -> listCount reused as the tile count input of the scan
__global__ void k_tile_counts(IndexArgs a, int64_t* tiles) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= 2 * a.nproj) return;
    const int64_t members = a.listOff[l + 1] - a.listOff[l];
    tiles[l] = ((members + a.TM - 1) / a.TM) * a.nct;
}

__global__ void k_tile_fill(IndexArgs a) {
    const int l = blockIdx.x;
    const int64_t t0 = a.tileOff[l], t1 = a.tileOff[l + 1];
    for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) a.tileList[t] = l;
}

__global__ void k_hubs_count(IndexArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * a.nproj * a.m) return;
    atomicAdd(a.hubCount + a.topM[q], 1);
}

__global__ void k_hubs_scatter(IndexArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * a.nproj * a.m) return;
    const int r = q / (2 * a.m), side = (q % (2 * a.m)) / a.m;
    const int p = a.topM[q];
    const int pos = atomicAdd(a.hubCount + p, 1);
    a.hubLists[a.hubOff[p] + pos] = side * a.nproj + r;
}

__global__ void k_pad_copy(const float* __restrict__ X, int n, int d, float* __restrict__ Xt, int ld) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)n * ld) return;
    const int p = (int)(q / ld), c = (int)(q % ld);
    Xt[q] = c < d ? X[(size_t)p * d + c] : 0.0f;
}

__global__ void k_i32_to_i64(const int32_t* in, int64_t* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

// ---- exclusive scan of int64 (three phases, recursive on block sums) -------
constexpr int kScanBlock = 256, kScanItems = 4, kScanTile = kScanBlock * kScanItems;

__device__ int64_t block_exclusive(int64_t v, int64_t* total) {
    __shared__ int64_t wsum[kScanBlock / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        const int64_t o = __shfl_up_sync(0xffffffffu, x, s);
        if (lane >= s) x += o;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t y = lane < kScanBlock / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const int64_t o = __shfl_up_sync(0xffffffffu, y, s);
            if (lane >= s) y += o;
        }
        if (lane < kScanBlock / 32) wsum[lane] = y;
    }
    __syncthreads();
    const int64_t before = w ? wsum[w - 1] : 0;
    *total = wsum[kScanBlock / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void k_scan_tiles(const int64_t* in, int64_t* out, size_t n, int64_t* sums) {
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int64_t total;
    int64_t ex = block_exclusive(s, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int64_t* out, size_t n, const int64_t* offs) {
    const size_t i = (size_t)blockIdx.x * kScanTile + threadIdx.x;
    const int64_t o = offs[blockIdx.x];
    for (int t = 0; t < kScanItems; ++t) {
        const size_t j = i + (size_t)t * kScanBlock;
        if (j < n && j < (size_t)(blockIdx.x + 1) * kScanTile) out[j] += o;
    }
}

}  // namespace

size_t scan_tmp_elems(size_t n) {
    size_t tot = 0;
    while (n > 1) {
        const size_t nb = (n + kScanTile - 1) / kScanTile;
        tot += nb + 1;
        n = nb;
    }
    return tot + 2;
}

int launch_scan_i64(const int64_t* in, int64_t* out, size_t n, int64_t* tmp, cudaStream_t st) {
    if (n == 0) return 0;
    const size_t nb = (n + kScanTile - 1) / kScanTile;
    int launches = 0;
    k_scan_tiles<<<(unsigned)nb, kScanBlock, 0, st>>>(in, out, n, tmp);
    ++launches;
    if (nb > 1) {
        int r = launch_scan_i64(tmp, tmp, nb, tmp + nb + 1, st);
        if (r < 0) return -1;
        launches += r;
        k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(out, n, tmp);
        ++launches;
    }
    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

int launch_index_count(const IndexArgs& a, cudaStream_t st) {
    const size_t sm = sizeof(int) * 2 * a.nproj;
    k_index_count<<<a.nChunks, 1024, sm, st>>>(a);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    const int L = 2 * a.nproj;
    k_chunk_scan<<<(L * 32 + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

int launch_index_scatter(const IndexArgs& a, cudaStream_t st) {
    const size_t sm = sizeof(int) * 2 * a.nproj;
    k_index_scatter<<<a.nChunks, 1024, sm, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_tile_order(const IndexArgs& a, cudaStream_t st) {
    if (a.maxTiles <= 0) return 0;
    if (cudaMemsetAsync(a.keyOff, 0, sizeof(int64_t) * ((size_t)a.nChunks + 1), st) != cudaSuccess) return -1;
    const unsigned g = (unsigned)((a.maxTiles + 255) / 256);
    k_tile_keys<<<g, 256, 0, st>>>(a);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    const int r = launch_scan_i64(a.keyOff, a.keyOff, (size_t)a.nChunks + 1, a.scanTmp, st);
    if (r < 0) return -1;
    k_tile_perm<<<g, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? r + 2 : -1;
}

size_t tile_order_list_keys(const IndexArgs& a, int superChunk) {
    return (size_t)((a.nChunks + superChunk - 1) / superChunk) * 2 * a.nproj + 1;
}

int launch_tile_order_list(const IndexArgs& a, int superChunk, int32_t* keys, int64_t* keyOff, int32_t* perm,
                           cudaStream_t st) {
    if (a.maxTiles <= 0) return 0;
    const size_t nk = tile_order_list_keys(a, superChunk);
    if (cudaMemsetAsync(keyOff, 0, sizeof(int64_t) * nk, st) != cudaSuccess) return -1;
    const unsigned g = (unsigned)((a.maxTiles + 255) / 256);
    k_tile_keys_list<<<g, 256, 0, st>>>(a, superChunk, keys, keyOff);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    const int r = launch_scan_i64(keyOff, keyOff, nk, a.scanTmp, st);
    if (r < 0) return -1;
    k_tile_perm_keys<<<g, 256, 0, st>>>(a, keys, keyOff, perm);
    return cudaPeekAtLastError() == cudaSuccess ? r + 2 : -1;
}

// Computes tileOff (scan of per-list tile counts) into a.tileOff; tile counts
// are staged in a.listCount (free by then).
int launch_tile_offsets(const IndexArgs& a, cudaStream_t st) {
    const int L = 2 * a.nproj;
    k_tile_counts<<<(L + 255) / 256, 256, 0, st>>>(a, a.listCount);
    if (cudaPeekAtLastError() != cudaSuccess) return -1;
    int r = launch_scan_i64(a.listCount, a.tileOff, (size_t)L + 1, a.scanTmp, st);
    return r < 0 ? -1 : r + 1;
}

int launch_tiles(const IndexArgs& a, int64_t, cudaStream_t st) {
    k_tile_fill<<<2 * a.nproj, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_hubs_count(const IndexArgs& a, cudaStream_t st) {
    const int total = 2 * a.nproj * a.m;
    k_hubs_count<<<(total + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_hubs_scatter(const IndexArgs& a, cudaStream_t st) {
    const int total = 2 * a.nproj * a.m;
    k_hubs_scatter<<<(total + 255) / 256, 256, 0, st>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_pad_copy(const float* X, int n, int d, float* Xt, int ld, cudaStream_t st) {
    const size_t total = (size_t)n * ld;
    k_pad_copy<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(X, n, d, Xt, ld);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_i32_to_i64(const int32_t* in, int64_t* out, int n, cudaStream_t st) {
    k_i32_to_i64<<<(n + 255) / 256, 256, 0, st>>>(in, out, n);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

}  // namespace sdb
