/*
 * cudaexactknn.h -- C ABI of the GB300 (sm_103a) exact k-nearest-neighbour engine.
 *
 * Plain pointers and sizes only; every function returns a knn_status code and never throws.
 * knn_last_error() gives a human-readable message for the calling thread's last failure.
 *
 * The entry points replace the GPU classes of the reference header library (namespace
 * KnnTrees of rezvoj/CudaExactKnn):
 *
 *   knn_bf_create    BruteForceGpu<Dims>::BruteForceGpu(devicePoints, n)      src/BruteForceGpu.cuh:63-68
 *   knn_kd_create    KdTreeGpu<Dims,AuxDims,CBlockSize>::KdTreeGpu(p,n,skips) src/KdTreeGpu.cuh:375-385
 *   knn_ball_create  BallTreeGpu<Dims,CBlockSize>::BallTreeGpu(p,n,skips)     src/BallTreeGpu.cuh:614-624
 *   knn_destroy      the three destructors                                     src/BruteForceGpu.cuh:70-72,
 *                                                                             src/KdTreeGpu.cuh:387-390,
 *                                                                             src/BallTreeGpu.cuh:626-629
 *   knn_query        batchKnn<K,BLOCK_SIZE,HEAP,SH_NN[,SH_STACK]>(Query&)      src/BruteForceGpu.cuh:74-83,
 *                                                                             src/KdTreeGpu.cuh:393-410,
 *                                                                             src/BallTreeGpu.cuh:631-648
 *                    with Query<Dims,K> = {points, count, maxDistance2,        src/KnnTrees.cuh:224-231
 *                                          rIndexes, rDistances}
 *   knn_status_string / knn_last_error   KnnTrees::CudaException's message     src/KnnTrees.cuh:20-23
 *
 * Semantics kept from the reference:
 *   - points are float32 [n][dims] row-major (Array<float,Dims>), device memory;
 *   - results are int32 [count][k] indices and float32 [count][k] squared distances;
 *   - a slot is filled by the k smallest keys (bits(dist2) << 32 | uint32(index)) with
 *     dist2 <= max_distance2; unfilled slots hold index -1 and distance max_distance2;
 *   - depthSkips: leaves of 2^skips points, skips clamped to log2Ceil(n)-1, and >= 1 for the
 *     ball tree; k-d split dimension = depth % aux_dims.
 * Differences, by design:
 *   - rows are always in ascending key order (the reference's heap tracking leaves heap order);
 *   - trees prune on bound > k-th distance with rigorous rounding margins, so every structure
 *     returns exactly brute force's answer, ties included;
 *   - work is enqueued on the caller's stream and the call returns without synchronising
 *     unless KNN_QF_SYNC is set (the reference synchronises the whole device per call);
 *   - a negative or NaN max_distance2, k == 0 or dims == 0 is KNN_ERR_INVALID_ARGUMENT.
 *
 * Supported sizes: 1 <= dims <= 128, 1 <= k <= 128, n < 2^31, count < 2^31.
 * Streams: an index owns one scratch workspace, so its queries run one after another on the
 * device.  A query issued on another stream than the index's previous query waits (an event on
 * the device, no host synchronisation) for that query to finish; different indexes on different
 * streams run concurrently.  Calls on one index come from one host thread at a time.
 */
#ifndef CUDAEXACTKNN_H
#define CUDAEXACTKNN_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define KNN_API __attribute__((visibility("default")))
#else
#define KNN_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct knn_index knn_index;

typedef enum knn_status {
    KNN_OK = 0,
    KNN_ERR_INVALID_ARGUMENT = 1,
    KNN_ERR_UNSUPPORTED = 2,   /* dims or k outside the supported range */
    KNN_ERR_CUDA = 3,          /* a CUDA runtime call failed (message in knn_last_error) */
    KNN_ERR_OUT_OF_MEMORY = 4,
    KNN_ERR_DEVICE_LIMIT = 5,  /* a kernel's bounds check fired; results are not valid */
    KNN_ERR_NOT_TRAINED = 6    /* KNN_QF_LEARNED_RADIUS without a trained radius model */
} knn_status;

typedef enum knn_structure {
    KNN_BRUTE_FORCE = 0,
    KNN_KD_TREE = 1,
    KNN_BALL_TREE = 2
} knn_structure;

/* Query flags. */
#define KNN_QF_SYNC 1u           /* synchronise the stream before returning */
#define KNN_QF_AUTOTUNE 2u       /* engine picks block size, tracking, storage and leaf size */
#define KNN_QF_LEARNED_RADIUS 4u /* seed each query's radius from the trained model; queries
                                    with fewer than k hits are re-run unbounded */
#define KNN_QF_BF16_FILTER 8u    /* any index, dims >= 16: 16-bit (FP16, or BF16 for values beyond
                                    FP16's range) tcgen05 filter with rigorous bounds + exact FP32
                                    rescore; the same answer as the plain search */
#define KNN_QF_KEEP_ORDER 16u    /* do not reorder queries for locality */
#define KNN_QF_TIMING 32u        /* record CUDA events around the query and each of its search kernels */
#define KNN_QF_FILTER_CODES 64u  /* KNN_QF_BF16_FILTER: keep the filter's running k-th bound as
                                    buffered 16-bit codes flushed in batches even where a heap per
                                    query fits (the heap, exact after every candidate, is the
                                    default where it fits: dims <= 32, or small k up to 64 dims) */
/* Test only: every tensor-core filter block gives up right after issuing its first point-tile
 * copy, as it does when one of its bounded waits runs out: it drains what it issued, frees its
 * tensor memory, flags the error, and leaves its queries (and the tiles it never took) to the
 * exhaustive search, so the answers are unchanged. */
#define KNN_QF_TEST_FILTER_GIVE_UP 0x40000000u

/*
 * Run-time form of batchKnn's template arguments (src/KdTreeGpu.cuh:392,
 * src/BruteForceGpu.cuh:74): BLOCK_SIZE, USE_HEAP_TRACKING, USE_TRACKING_SHMEM,
 * USE_STACK_SHMEM.  A zeroed struct (or NULL) means block 0 = engine default, sorted
 * insertion tracking in registers, stack in registers.
 */
typedef struct knn_query_opts {
    uint32_t block_size;
    uint32_t heap_tracking;
    uint32_t shmem_tracking;
    uint32_t shmem_stack;
    uint32_t flags;
    uint32_t leaf_scan;     /* trees: scan whole subtrees of at most this many points as one
                               leaf (0 = the tree's own leaves) */
    uint32_t traversal;     /* trees: 0 = one depth-first search per thread (the reference's
                               scheme), 1 = warp-coherent search (a warp's queries walk together);
                               k-d trees of at most 16 dims, k <= 32: 2 = warp-group search (a
                               warp's 32 queries walk the tree once against tight node boxes from
                               per-query radii -- the radius model's seeds, or each query's own
                               subtree -- and share out their (bucket, query) scans; leaf_scan =
                               points per bucket, 0 = 8); 3 = one search per thread bounded by
                               the same tight node boxes instead of splitting planes */
    uint32_t reserved;      /* KNN_QF_BF16_FILTER: candidates kept per query (0 = the engine's
                               default, min(4096, max(1024, 16 k))); for
                               knn_tuned_plan, the number of candidate plans timed */
} knn_query_opts;

/* Per-query statistics written by knn_query_stats (summed over the batch). */
typedef struct knn_query_counters {
    uint64_t nodes_visited;    /* internal nodes whose bound was evaluated */
    uint64_t leaves_visited;   /* leaves scanned */
    uint64_t points_scanned;   /* leaf slots whose distance was computed */
    uint64_t fallback_queries; /* queries the fast form handed to the plain search: learned-
                                  radius retries, warp-group and tensor-core filter fallbacks */
    uint64_t filter_give_ups;  /* tensor-core filter blocks whose bounded waits ran out (their
                                  queries are answered by the exhaustive search) */
    uint64_t reserved[3];
} knn_query_counters;

typedef struct knn_index_info {
    uint32_t structure;   /* knn_structure */
    uint32_t n;
    uint32_t dims;
    uint32_t aux_dims;    /* k-d split dimensions (k-d tree), else dims */
    uint32_t depth_skips; /* after clamping */
    uint32_t node_depth;  /* internal node levels */
    uint32_t leaf_slots;  /* 2^depth_skips */
    uint32_t node_count;  /* internal nodes, 2^node_depth - 1 */
    uint64_t device_bytes;
    float build_ms;       /* device time of the construction, CUDA events */
    uint32_t radius_model;/* 1 when a learned radius model is attached */
} knn_index_info;

/* Learned-radius training options; zeros select the defaults in brackets. */
typedef struct knn_train_opts {
    uint32_t steps;   /* Adam steps, cosine-decayed learning rate [3000] */
    uint32_t batch;   /* samples per step [1024] */
    float lr;         /* learning rate [3e-3] */
    float coverage;   /* fraction of training queries whose k-th distance must fall inside the
                         seeded radius; sets the calibrated margin [0.98] */
    uint32_t seed;    /* weight initialisation and shuffling [1] */
    uint32_t reserved[3];
} knn_train_opts;

typedef struct knn_train_report {
    float train_ms;          /* device time: exact targets + training + calibration */
    float final_batch_loss;  /* mean squared error on log k-th distance, last minibatch */
    float rmse;              /* over all samples */
    float margin;            /* added to the predicted log k-th distance */
    float coverage;          /* achieved on the samples */
    uint32_t samples;
    uint32_t steps;
    uint32_t reserved;
} knn_train_report;

/* ---- construction (points: device pointer, float32 [n][dims]; read during the call only) --- */
KNN_API int knn_bf_create(const float* d_points, uint32_t n, uint32_t dims, void* stream,
                  knn_index** out);
KNN_API int knn_kd_create(const float* d_points, uint32_t n, uint32_t dims, uint32_t aux_dims,
                  uint32_t depth_skips, uint32_t build_block, void* stream, knn_index** out);
KNN_API int knn_ball_create(const float* d_points, uint32_t n, uint32_t dims, uint32_t depth_skips,
                    uint32_t build_block, void* stream, knn_index** out);
KNN_API int knn_destroy(knn_index* index);
KNN_API int knn_index_get_info(const knn_index* index, knn_index_info* out);

/* ---- serialised indexes (no counterpart in the reference, whose trees live only in the class
 *      instance's device arrays: src/KdTreeGpu.cuh:293-294, src/BallTreeGpu.cuh:461-462) -------- */
/* Writes the index (its device arrays and any learned-radius model) to host memory.  With
 * host_buf NULL, only *size is set (the bytes needed).  Synchronises `stream`. */
KNN_API int knn_index_serialize(const knn_index* index, void* host_buf, size_t capacity, size_t* size,
                                void* stream);
/* Rebuilds an index on the current device from knn_index_serialize's bytes, without the
 * construction kernels.  Rejects (KNN_ERR_INVALID_ARGUMENT) a blob whose magic, version, shape,
 * array sizes or checksum do not match, before any device memory is used. */
KNN_API int knn_index_deserialize(const void* host_buf, size_t size, void* stream, knn_index** out);

/* ---- queries (device pointers; enqueued on `stream`, a cudaStream_t, NULL = legacy stream) -- */
KNN_API int knn_query(knn_index* index, const float* d_queries, uint32_t count, float max_distance2,
              uint32_t k, int32_t* d_indexes, float* d_distances, const knn_query_opts* opts,
              void* stream);

/* As knn_query, with one max_distance2 per query (device float32 [count]). */
KNN_API int knn_query_radii(knn_index* index, const float* d_queries, uint32_t count,
                    const float* d_max_distance2, uint32_t k, int32_t* d_indexes,
                    float* d_distances, const knn_query_opts* opts, void* stream);

/* As knn_query with HOST buffers, and synchronises: the queries are copied in on `stream`, the
 * search runs there, and the result rows go out in four pieces on four copy streams of the index
 * at once (one cudaMemcpyAsync each), so that several copy engines share the larger transfer.
 * Replaces the reference's copy, batchKnn and device-wide synchronisation
 * (src/KdTreeGpu.cuh:394-410, src/BruteForceGpu.cuh:75-83).  Pinned host memory gives
 * full-speed, asynchronous copies. */
KNN_API int knn_query_host(knn_index* index, const float* h_queries, uint32_t count,
                   float max_distance2, uint32_t k, int32_t* h_indexes, float* h_distances,
                   const knn_query_opts* opts, void* stream);

/* Runs the query with device counters enabled and returns the summed counters (synchronous). */
KNN_API int knn_query_stats(knn_index* index, const float* d_queries, uint32_t count,
                    float max_distance2, uint32_t k, int32_t* d_indexes, float* d_distances,
                    const knn_query_opts* opts, void* stream, knn_query_counters* out);

/* ---- batches of independent sets (the reference answers one set per batchKnn call, each ending in
 *      a device-wide sync: src/KdTreeGpu.cuh:393-410, src/BallTreeGpu.cuh:631-648) ---------------- */
typedef struct knn_batch knn_batch;
typedef struct knn_batch_item {
    knn_index* index;         /* k-d or ball tree */
    const float* d_queries;   /* [count][dims], device */
    uint32_t count;
    float max_distance2;
    uint32_t k;
    int32_t* d_indexes;       /* [count][k], device */
    float* d_distances;       /* [count][k], device */
} knn_batch_item;
/* Plans a batch: items grouped by (tree, dims, k) class, one persistent kernel per class over all
 * its sets, the classes captured as parallel branches of one CUDA graph.  flags: KNN_QF_AUTOTUNE
 * tunes each class on its largest set (runs queries, synchronously) and sends a class of dims >= 16
 * through the tensor-core filter when that times faster; KNN_QF_KEEP_ORDER skips the
 * locality sort.  The items' pointers are baked into the graph: refill the buffers, not the items. */
KNN_API int knn_batch_create(const knn_batch_item* items, uint32_t count, uint32_t flags, void* stream,
                             knn_batch** out);
/* Runs every item of the batch: one cudaGraphLaunch on `stream`. */
KNN_API int knn_batch_run(knn_batch* batch, void* stream);
/* Classes in the batch and kernel launches one knn_batch_run makes (kernel nodes of its graph). */
KNN_API int knn_batch_info(const knn_batch* batch, uint32_t* classes, uint32_t* kernels_per_run);
KNN_API int knn_batch_destroy(knn_batch* batch);

/* ---- learned radius (no counterpart in the reference; it seeds Query::maxDistance2,
 *      src/KnnTrees.cuh:228, per query) ---------------------------------------------------------
 * Trains the index's D->64->64->1 radius model on `count` sample queries (device float32
 * [count][dims]): exact k-th distances from the engine's own search are the targets; forward,
 * backward and Adam run on the GPU; the margin is calibrated to `coverage`.  Synchronous.
 * k must not exceed the index's point count (every k-th distance would be unbounded). */
KNN_API int knn_radius_model_train(knn_index* index, const float* d_samples, uint32_t count, uint32_t k,
                                   const knn_train_opts* opts, void* stream, knn_train_report* report);
/* Predicted natural log of the k-th squared distance per query (device float32 [count]). */
KNN_API int knn_radius_model_predict(knn_index* index, const float* d_queries, uint32_t count,
                                     float* d_log_kth, void* stream);
/* Parameter count of a model for `dims`, and host copies in and out (serialisation). */
KNN_API uint32_t knn_radius_model_size(uint32_t dims);
KNN_API int knn_radius_model_export(const knn_index* index, float* h_params, uint32_t capacity);
KNN_API int knn_radius_model_import(knn_index* index, const float* h_params, uint32_t count, uint32_t k);
/* Forward + backward of the model on a host batch (x [batch][dims], targets [batch]) with host
 * parameters; writes the loss and the gradient of every trainable parameter (gradient checks). */
KNN_API int knn_radius_model_gradients(const float* h_params, uint32_t dims, const float* h_x,
                                       const float* h_targets, uint32_t batch, float* h_grad, float* h_loss);

/* Device time (ms) of the index's last KNN_QF_TIMING query: the whole query, and the sum of the
 * spans of its search kernels (a learned-radius query: the seeded search and every retry search;
 * the tensor-core filter: its filter kernel) measured by CUDA events on the query's stream.
 * Waits for the query to finish. */
KNN_API int knn_last_query_timing(knn_index* index, float* total_ms, float* kernel_ms);

/* The plan KNN_QF_AUTOTUNE chose for this index and k (block size, tracking, storage, leaf
 * bucket, traversal), with the tuning sample's time in *ms and the number of candidates timed
 * in out->reserved.  Autotuning runs on the first KNN_QF_AUTOTUNE query per k class. */
KNN_API int knn_tuned_plan(const knn_index* index, uint32_t k, uint32_t learned_radius, knn_query_opts* out,
                           float* ms);

/* Brute-force query that allocates no device memory.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc (inside a stream capture, under an allocator that
 * forbids side allocations, in a loop that must not touch the allocator) and so cannot create an
 * index either.  Searches the caller's device points [n][dims] directly; its only scratch is a
 * 16 MiB array compiled into the library (held on every GPU that loads the library, until exit).
 * Limit: count * k <= 1,048,576, else KNN_ERR_UNSUPPORTED.  All calls on a device share that
 * array, so calls that overlap on the GPU race; the first call on each device looks up the
 * array's address and should come before any stream capture.  Same results as knn_query on a
 * brute-force index of the same points. */
KNN_API int knn_bf_query_noalloc(const float* d_points, uint32_t n, uint32_t dims, const float* d_queries,
                                 uint32_t count, float max_distance2, uint32_t k, int32_t* d_indexes,
                                 float* d_distances, void* stream);

/* Runs one 128 x 256 tile with K = dims through the tensor-core path (tcgen05.mma, BF16 in, FP32
 * accumulate) on fixed data and compares it with exact products of the BF16-rounded inputs:
 * worst relative error and the count of entries beyond the bound the filter assumes. */
KNN_API int knn_tc_selftest(uint32_t dims, float* max_rel_err, uint32_t* mismatches);

/* Number of kernels this library has launched since it was loaded (all indexes, all threads). */
KNN_API uint64_t knn_launch_count(void);

/* ---- errors ------------------------------------------------------------------------------ */
KNN_API const char* knn_status_string(int status);
KNN_API const char* knn_last_error(void);
KNN_API int knn_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CUDAEXACTKNN_H */
