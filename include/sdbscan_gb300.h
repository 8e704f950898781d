/*
 * sdbscan_gb300 — C ABI of the GB300 sDbscan / sOPTICS engine.
 *
 * A drop-in for the fit path of the reference's `sDbscan` class
 * (src/sDbscan.h:10-223, bound to Python in python/python_wrapper.cpp:14-65).
 * Each entry point below names the reference interface it replaces.  Plain C
 * types only: pointers, sizes, one parameter struct and status codes.
 *
 * Conventions
 *  - Data is d x n column-major float32 (one point per contiguous run of d
 *    floats), exactly as the reference takes it (README.md:39-41,
 *    src/Utilities.cpp:69-76).
 *  - Every output buffer is owned by the caller.
 *  - An engine owns its device buffers and one CUDA stream.  It is not
 *    thread-safe; use one engine per host thread.
 *  - Errors are returned as status codes, never by exiting; the message of
 *    the last failure is available from sdb_last_error().
 */
#ifndef SDBSCAN_GB300_H
#define SDBSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sdb_engine sdb_engine;

typedef enum {
    SDB_OK = 0,
    SDB_ERR_ARG = 1,        /* invalid argument or parameter combination          */
    SDB_ERR_CUDA = 2,       /* CUDA runtime error (message in sdb_last_error)      */
    SDB_ERR_NEGATIVE = 3,   /* Chi2/JS input has a negative value (src/Utilities.h:308-312) */
    SDB_ERR_ZERO_POINT = 4, /* a point with zero sum (Chi2/JS, :318-325) or zero norm (Cosine) */
    SDB_ERR_STATE = 5,      /* output requested before the matching fit            */
    SDB_ERR_NOMEM = 6,      /* device or host allocation failed                    */
    SDB_ERR_INTERNAL = 7    /* internal consistency check failed                   */
} sdb_status;

typedef enum { SDB_COSINE = 0, SDB_L1 = 1, SDB_L2 = 2, SDB_CHI2 = 3, SDB_JS = 4 } sdb_distance;

typedef enum {
    SDB_PREC_FP32 = 0,      /* plain FP32: results identical to the reference's CPU path */
    SDB_PREC_BF16 = 1       /* Cosine: BF16 tensor-core screening of the candidate
                               distances + exact FP32 re-decision near eps (labels
                               identical to FP32); L1/L2: the random-Fourier embedding
                               GEMM on the tensor cores in split BF16.  sOPTICS fits
                               and other distances run as FP32. */
} sdb_precision;

/* Parameters of sDbscan::set_params (src/sDbscan.h:79-108), same meaning and
 * order; `precision` is this engine's addition.  Fill with
 * sdb_params_default() to get the Python binding's defaults
 * (python/python_wrapper.cpp:17-24). */
typedef struct {
    int32_t n_proj;               /* numProj: number of random vectors D          */
    int32_t topK;                 /* k: close/far random vectors kept per point   */
    int32_t topM;                 /* m: close/far points kept per random vector   */
    int32_t distance;             /* sdb_distance                                 */
    int32_t ker_n_features;       /* kerDim (forced to n_features for Cosine)     */
    float ker_sigma;              /* kerSigma (L1/L2 random Fourier features)     */
    float ker_intervalSampling;   /* kerSam (Chi2/JS embeddings)                  */
    int32_t clusterNoise;         /* noiseClustering: 0, 1 (sDbscan-1NN), 2 (no-op) */
    float samplingProb;           /* prob: sDbscan-1NN core sampling; sng sample rate */
    int32_t verbose;              /* ver: print per-stage times                   */
    int32_t n_threads;            /* numThreads: accepted for API parity, unused  */
    int32_t random_seed;          /* randomSeed: < 0 means seeded from the clock  */
    int32_t precision;            /* sdb_precision                                */
} sdb_params;

/* Defaults of the Python binding (python/python_wrapper.cpp:17-24). */
void sdb_params_default(sdb_params* p);

/* sDbscan(int n, int d)  (src/sDbscan.h:74-77; python_wrapper.cpp:16).
 * device: CUDA device ordinal. */
sdb_status sdb_engine_create(int32_t n_points, int32_t n_features, int32_t device, sdb_engine** out);

/* ~sDbscan()  (src/sDbscan.h:165-168). */
void sdb_engine_destroy(sdb_engine* e);

/* set_params / set_kernel_params / set_topK / set_topM / set_threads /
 * set_clusterNoise  (src/sDbscan.h:79-124, :170-180).  Limits of this engine:
 * n_proj <= 2048, 9 <= max(n_proj, ker_n_features) <= 16384 (d <= 16384 for
 * Cosine), 1 <= topK <= 31 and topK <= n_proj, topM <= n_points, an even
 * ker_n_features for L1 / L2.  Chi2 and
 * JS need ker_n_features >= n_features, the reference's own precondition
 * (src/sDbscan.cpp:54; embedChi2 / embedJS write n_features slots of a
 * ker_n_features-long vector, src/Utilities.h:140-145, and overrun it
 * otherwise): SDB_ERR_ARG here. */
sdb_status sdb_set_params(sdb_engine* e, const sdb_params* p);

/* set_precision: SDB_PREC_FP32 or SDB_PREC_BF16 alone, without the index
 * parameter checks of sdb_set_params (for the sng fits).  No reference
 * counterpart (the reference computes in FP32 only). */
sdb_status sdb_set_precision(sdb_engine* e, int32_t precision);

/* Test and diagnostic limits (no reference counterpart; each 0 = off, the
 * default).  They let the failure paths run without a GPU fault:
 *   stall_spins      > 0: each tensor-core kernel (BF16 distance screening,
 *                    BF16 random-Fourier embedding, BF16 sngDbscan block) and
 *                    the persistent plain distance kernel waits once per launch
 *                    on a barrier that nothing completes, and gives up after
 *                    this many polls; the kernel then takes its failure path:
 *                    its roles stop, it waits for its own copies and MMAs, and
 *                    it raises its flag.  The BF16 stages then run their FP32
 *                    kernels (same results; sdb_get_counters out[5] counts
 *                    them); the persistent plain kernel (sdb_set_tile_variant
 *                    4, 5) fails the fit with SDB_ERR_INTERNAL.
 *   queue_cap        > 0: the BF16 re-decision queues hold at most this many
 *                    pairs; an overflow sends the stage to its FP32 kernel.
 *   device_bytes_cap > 0: the engine's device memory stays below this; a fit
 *                    that needs more returns SDB_ERR_NOMEM and the engine
 *                    stays usable.
 * Negative values return SDB_ERR_ARG. */
sdb_status sdb_set_debug_limits(sdb_engine* e, int64_t stall_spins, int64_t queue_cap, int64_t device_bytes_cap);

/* Tile shape of the plain FP32 distance kernel (a tuning control; no
 * reference counterpart): 0 = by topM and distance (default: for topM in
 * 41..50 shape 3 with Cosine, shape 2 otherwise; else 1), 1 = 128 x 64 tiles on 256 threads, 2 = 128 x 50 on 160 threads
 * (32 dimensions per stage, 2 stages), 3 = 128 x 50 with 16 dimensions per
 * stage in 4 stages (Cosine; shape 2 for the other distances), 4 and 5 = the
 * persistent warp-specialised kernel (a producer warp gathers the rows, the
 * other warps compute; 4 stages and 3 CTAs per SM, or 6 stages and 2).  The
 * 50-column shapes apply when topM <= 50 (else the 64-column ones).  Any shape
 * gives the same bits. */
sdb_status sdb_set_tile_variant(sdb_engine* e, int32_t variant);

/* fit_sDbscan(const Ref<const MatrixXf>& X, float eps, int minPts)
 * (src/sDbscan.h:183, src/sDbscan.cpp:830-890).  X_host: d x n column-major
 * host memory (pinned memory makes the upload faster).  Results stay in the
 * engine until read with sdb_get_*. */
sdb_status sdb_fit_sdbscan(sdb_engine* e, const float* X_host, float eps, int32_t minPts);

/* Same as sdb_fit_sdbscan with X already in device memory (d x n
 * column-major, device pointer of the engine's device).  No reference
 * counterpart: it is the same fit with the upload left out. */
sdb_status sdb_fit_sdbscan_device(sdb_engine* e, const float* X_device, float eps, int32_t minPts);

/* fit_sOptics(const Ref<const MatrixXf>& X, float eps, int minPts)
 * (src/sDbscan.h:197, src/sDbscan.cpp:1711-1769).  minPts >= 2. */
sdb_status sdb_fit_soptics(sdb_engine* e, const float* X_host, float eps, int32_t minPts);
sdb_status sdb_fit_soptics_device(sdb_engine* e, const float* X_device, float eps, int32_t minPts);

/* loadtxtData (src/Utilities.cpp:57-95), used by load_fit_sDbscan /
 * load_fit_sOptics (src/sDbscan.cpp:903-966, :1777-1837): reads n_points
 * lines of n_features whitespace-separated numbers into X_dxn (d x n
 * column-major, point n's values at X_dxn[n * d ...]), parsed like fscanf
 * "%f".  No engine and no GPU are involved.  Returns SDB_ERR_ARG when the
 * file is missing or holds fewer than n_points x n_features numbers (the
 * reference exits or keeps zeros). */
sdb_status sdb_load_txt(const char* path, int32_t n_points, int32_t n_features, float* X_dxn);

/* test_sDbscan(X, eps, rangeEps, n_tests, minPts)  (src/sDbscan.h:187,
 * src/sDbscan.cpp:980-1039): the index and the candidate distances are built
 * once, then core points and clusters for every eps in eps[0..n_eps).
 * labels: n_eps x n_points int32 (row i for eps[i]); n_clusters: n_eps.  The
 * reference derives its list as eps + i * rangeEps and writes each labelling
 * to a file; here the caller passes the list (any order, repeats allowed) and
 * gets the labellings back.  The eps values are processed in ascending order,
 * each adding only its new pairs; every labelling equals a separate
 * fit_sDbscan at that eps.  BF16 precision screens the distances once for all
 * eps values (up to 16; longer lists run FP32). */
sdb_status sdb_fit_sdbscan_sweep(sdb_engine* e, const float* X_host, const float* eps, int32_t n_eps, int32_t minPts,
                                 int32_t* labels, int32_t* n_clusters);

/* set_sngParams(dist, prob, noiseClustering, ver, filename, numThreads,
 * randomSeed)  (src/sDbscan.h:127-139): sets distance, samplingProb, verbose,
 * n_threads and random_seed, and clusterNoise = 2 when clusterNoise > 0; the
 * index parameters keep their values.  Enough for the sng fits below. */
sdb_status sdb_set_sng_params(sdb_engine* e, int32_t distance, float samplingProb, int32_t clusterNoise,
                              int32_t verbose, int32_t n_threads, int32_t random_seed);

/* How fit_sngDbscan draws its samples (no reference counterpart; the
 * reference's rule depends on the seed, src/sDbscan.cpp:437-440):
 *   0 (default) by the seed: random_seed >= 0 -> 1, random_seed < 0 -> 2;
 *   1 shared: every point draws the same sequence from random_seed, which is
 *     the reference's own behaviour for a fixed seed (identical labels);
 *   2 blocks: each block of 32 consecutive points draws its own S columns
 *     (draw j of block b from splitmix64 of the seed, b and j), so that every
 *     point has S forward and about S reverse draws, as when the reference's
 *     points seed their generators apart (random_seed < 0); the seed is
 *     random_seed, or the clock when < 0.  FP32 distances (BF16 precision
 *     does not apply).  samplingProb >= 1 is exact DBSCAN in every mode. */
sdb_status sdb_set_sng_sampling(sdb_engine* e, int32_t mode);

/* fit_sngDbscan(X, eps, minPts)  (src/sDbscan.h:190, src/sDbscan.cpp:1131-1179):
 * each point's neighbourhood from ceil(n samplingProb) random draws (both
 * directions of every draw within eps), core points with >= minPts - 1
 * neighbours counted with repeats, clusters as fit_sDbscan; samplingProb >= 1
 * is exact DBSCAN.  With random_seed >= 0 the labels equal the reference's
 * (every point's generator is seeded alike); with random_seed < 0 the sample
 * is drawn per block of points (sdb_set_sng_sampling).  Switches clusterNoise
 * to 0 (src/sDbscan.cpp:1157).
 * Results: sdb_get_labels, sdb_get_core (neighbourhood sizes with repeats). */
sdb_status sdb_fit_sngdbscan(sdb_engine* e, const float* X_host, float eps, int32_t minPts);
/* (With SDB_PREC_BF16 and Cosine the distance block is screened on the tensor
 * cores and every pair near eps re-decided in FP32: the same labels.) */
sdb_status sdb_fit_sngdbscan_device(sdb_engine* e, const float* X_device, float eps, int32_t minPts);

/* test_sngDbscan(X, eps, rangeEps, n_tests, minPts)  (src/sDbscan.h:193,
 * src/sDbscan.cpp:1192-1240): one transform and sample, then a clustering per
 * eps of eps[0..n_eps).  labels: n_eps x n_points int32; n_clusters: n_eps. */
sdb_status sdb_fit_sngdbscan_sweep(sdb_engine* e, const float* X_host, const float* eps, int32_t n_eps,
                                   int32_t minPts, int32_t* labels, int32_t* n_clusters);

/* fit_sngOptics(X, eps, minPts)  (src/sDbscan.h:200, src/sDbscan.cpp:1846-1880):
 * de-duplicated sampled neighbourhoods with distances, core distances
 * ((minPts-1)-th smallest), then the ordering and reachability of
 * fit_sOptics.  The reference seeds each point from std::random_device (not
 * reproducible); here all points share one seeded sequence of
 * ceil(samplingProb n) draws (random_seed, or the clock when < 0), each
 * skipping its own index.  minPts >= 2.  Results: sdb_get_optics,
 * sdb_get_core, sdb_get_core_dist. */
sdb_status sdb_fit_sngoptics(sdb_engine* e, const float* X_host, float eps, int32_t minPts);
sdb_status sdb_fit_sngoptics_device(sdb_engine* e, const float* X_device, float eps, int32_t minPts);

/* labels_ and n_clusters_  (src/sDbscan.h:67-68; python_wrapper.cpp:31-32).
 * labels: n_points int32. */
sdb_status sdb_get_labels(sdb_engine* e, int32_t* labels, int32_t* n_clusters);

/* ordering_ and reachability_  (src/sDbscan.h:71-72; python_wrapper.cpp:33-34).
 * ordering: n_points int32 (a permutation); reachability: n_points float,
 * indexed by point id, -2^31 for points never reached (src/sDbscan.cpp:1590). */
sdb_status sdb_get_optics(sdb_engine* e, int32_t* ordering, float* reachability);

/* clear()  (src/sDbscan.h:142-163): drops results; device buffers are kept
 * for the next fit. */
sdb_status sdb_clear(sdb_engine* e);

/* Intermediate state, for parity checks (protected members of the reference):
 *   matrix_topK  (src/sDbscan.h:50): n x 2k int32, point-major, row 0 = most extreme
 *   matrix_topM  (src/sDbscan.h:51): D x 2m int32, vector-major
 *   bit_CorePoints (src/sDbscan.h:56): n uint8
 *   |neighbourhood| per point (sizes of vec2D_Neighbors before the non-core
 *       lists are cleared, src/sDbscan.cpp:378-382): n int32
 *   vec_CoreDist (src/sDbscan.h:60): n float (sOPTICS fits only)
 *   projections (MATRIX_FHT, src/sDbscan.cpp:31, :91): n x D float, point-major */
sdb_status sdb_get_topk(sdb_engine* e, int32_t* topK);
sdb_status sdb_get_topm(sdb_engine* e, int32_t* topM);
sdb_status sdb_get_core(sdb_engine* e, uint8_t* core, int32_t* degree);
sdb_status sdb_get_core_dist(sdb_engine* e, float* core_dist);
sdb_status sdb_get_projections(sdb_engine* e, float* proj);

/* Counters of the last fit: ties at the top-k / top-m selection boundary
 * (where the reference's heap order decides), kernel launches, neighbour
 * pairs within eps. out[0]=topk ties, out[1]=topm ties, out[2]=launches,
 * out[3]=directed candidate pairs within eps (with duplicates),
 * out[4]=pairs re-decided in FP32 by the BF16 screening mode,
 * out[5]=BF16 screening stages redone on the plain path (engine lifetime),
 * out[6]=distinct sampled points and out[7]=extra draws of the last
 * sngDbscan / sngOptics fit. */
sdb_status sdb_get_counters(sdb_engine* e, int64_t* out, int32_t n_out);

/* Device time of each stage of the last fit in milliseconds (CUDA events):
 * ms[0]=upload, [1]=transform+projection+top-k, [2]=top-m, [3]=index,
 * [4]=distances, [5]=core, [6]=cluster/optics, [7]=download, [8]=total. */
sdb_status sdb_get_stage_ms(sdb_engine* e, float* ms, int32_t n_ms);

/* The CUDA stream the engine runs on (as a void*), for callers that want to
 * order their own work after a fit. */
void* sdb_engine_stream(sdb_engine* e);

/* Message of the last error on this engine ("" if none). */
const char* sdb_last_error(sdb_engine* e);

/* Many independent datasets, each with the same eps sweep, recorded once into
 * one CUDA graph and replayed with a single launch.  No reference counterpart
 * (the reference runs test_sDbscan per dataset, src/sDbscan.cpp:980-1039).
 * p->precision applies to every set (BF16: screened distances, labels equal
 * to FP32, where the autotuner finds the screening faster than the plain
 * tiles for that set).
 *   X_device[i]: d_i x n_i column-major data of set i, device memory, kept
 *                valid for the batch's lifetime
 * The batch plans every set once (sizing run; with topM <= 50 it also times
 * the three plain distance tile shapes per set and, with BF16 precision, the
 * tensor-core screening, and keeps the fastest, sdb_batch_tile_variant), then
 * times graphs with 4, 8, 16, 32 and 64
 * sets in flight and keeps the fastest (sdb_batch_lanes).
 * sdb_batch_run replays it; sdb_batch_labels reads set i's labelling for eps
 * index j. */
typedef struct sdb_batch sdb_batch;
sdb_status sdb_batch_create(int32_t n_sets, const int32_t* n_points, const int32_t* n_features,
                            const float* const* X_device, const sdb_params* p, const float* eps, int32_t n_eps,
                            int32_t minPts, int32_t device, sdb_batch** out);
sdb_status sdb_batch_run(sdb_batch* b, float* elapsed_ms);
sdb_status sdb_batch_labels(sdb_batch* b, int32_t set, int32_t eps_index, int32_t* labels, int32_t* n_clusters);
int32_t sdb_batch_lanes(sdb_batch* b);
/* The distance stage the autotuner kept for set i (topM <= 50): a plain tile
 * shape of sdb_set_tile_variant, 1..3, or 0 = the default (BF16 precision:
 * the tensor-core screening; FP32: the shape by topM); -1 for a bad index. */
int32_t sdb_batch_tile_variant(sdb_batch* b, int32_t set);
void sdb_batch_destroy(sdb_batch* b);
const char* sdb_batch_last_error(sdb_batch* b);

/* Per-vector top-m selection (the top-m stage of a fit) that allocates no
 * device memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc while they run -- a serving loop whose memory pool
 * already owns the GPU's memory, code that must avoid the implicit
 * synchronisation of an allocation, or work issued during stream capture.
 *   proj_device : n_points x n_proj projections, point-major, device memory
 *                 (the layout sdb_get_projections returns)
 *   topM_device : n_proj x 2*topM int32 output, device memory, same layout
 *                 and content as sdb_get_topm
 *   stream      : cudaStream_t to run on (NULL = legacy default stream)
 * Limits: n_proj <= 1024, topM <= 64, topM <= n_points; larger sizes return
 * SDB_ERR_ARG.  When n_proj is a multiple of 4 the rows are read as 16-byte
 * vectors, so proj_device must then be 16-byte aligned (SDB_ERR_ARG
 * otherwise; an offset view into a larger buffer may not be).
 * Scratch is one fixed __device__ array (about 12 MiB) held by every GPU that
 * loads this library until it is unloaded.  With CUDA's lazy module loading
 * (the default) the array is reserved on a device by the first call there,
 * which also looks up its device address: make that first call before the
 * caller's memory pool takes the device's memory, and before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.
 * The boundary-tie count and internal-error flag that a fit reports through
 * sdb_get_counters / SDB_ERR_INTERNAL are not reported by this call. */
sdb_status sdb_topm_noalloc(const float* proj_device, int32_t n_points, int32_t n_proj, int32_t topM,
                            int32_t* topM_device, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SDBSCAN_GB300_H */
