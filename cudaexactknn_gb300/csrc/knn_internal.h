// Internal declarations of the engine: the index object behind the C ABI, its device memory
// layout, the scratch workspace, error plumbing and the per-structure entry points.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdint>
#include <initializer_list>
#include <new>
#include <vector>

#include "../../include/cudaexactknn.h"
#include "knn_common.cuh"

namespace knn {

// ---- errors -----------------------------------------------------------------------------------
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define KNN_TRY_CUDA(expr)                                                          \
    do {                                                                            \
        cudaError_t knn_e_ = (expr);                                                \
        if (knn_e_ != cudaSuccess) return ::knn::cuda_fail(knn_e_, #expr, __FILE__, __LINE__); \
    } while (0)

// Counts a kernel launch (or `n` of them) and checks the launch error.
void note_launches(uint32_t n);
#define KNN_LAUNCHED_N(n)                  \
    do {                                   \
        ::knn::note_launches(n);           \
        KNN_TRY_CUDA(cudaGetLastError());  \
    } while (0)
#define KNN_LAUNCHED() KNN_LAUNCHED_N(1)

#define KNN_TRY(expr)                   \
    do {                                \
        int knn_rc_ = (expr);           \
        if (knn_rc_ != KNN_OK) return knn_rc_; \
    } while (0)

// Names a host-side phase (construction, a query, the autotuner, training, a batch) for
// profilers as an NVTX range; without a profiler attached a push/pop pair is a pointer check.
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

// Runs f() and turns an exception from host code (a container's std::bad_alloc) into a status,
// so that nothing thrown crosses the C ABI.
template <class F>
int no_throw(F&& f) noexcept {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(KNN_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
        return fail(KNN_ERR_CUDA, "unexpected exception in host code");
    }
}

// ---- dimension padding ------------------------------------------------------------------------
// Kernels are compiled for padded dimension counts; padded coordinates are zero in both points
// and queries, so they add exactly 0 to every squared distance.
constexpr uint32_t kMaxDims = 128;
constexpr uint32_t kMaxK = 128;

inline uint32_t padded_dims(uint32_t d) {
    if (d <= 4) return d;
    if (d <= 8) return 8;
    if (d <= 16) return 16;
    if (d <= 32) return 32;
    if (d <= 64) return 64;
    return 128;
}

inline uint32_t round_up4(uint32_t v) { return (v + 3u) & ~3u; }

// Top-k capacity classes (run-time k <= KMAX).
inline uint32_t k_class(uint32_t k) {
    if (k <= 8) return 8;
    if (k <= 16) return 16;
    if (k <= 32) return 32;
    if (k <= 64) return 64;
    return 128;
}

// ---- device memory ------------------------------------------------------------------------------
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    int alloc(size_t n) {
        release();
        if (n == 0) return KNN_OK;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ptr = nullptr;
            return e == cudaErrorMemoryAllocation
                       ? fail(KNN_ERR_OUT_OF_MEMORY, "cudaMalloc of %zu bytes failed", n)
                       : cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
        }
        bytes = n;
        return KNN_OK;
    }
    // Grow-only: keeps the current allocation when it is large enough.
    int reserve(size_t n) { return n <= bytes ? KNN_OK : alloc(n); }
    template <class T>
    T* as() const { return static_cast<T*>(ptr); }
};

// Bump allocator over one device buffer (256-byte aligned carve-outs).
struct Carver {
    char* base;
    size_t off = 0;
    explicit Carver(void* b) : base(static_cast<char*>(b)) {}
    template <class T>
    T* take(size_t count) {
        off = (off + 255) & ~static_cast<size_t>(255);
        T* p = reinterpret_cast<T*>(base + off);
        off += count * sizeof(T);
        return p;
    }
};
inline size_t carve_bytes(std::initializer_list<size_t> sizes) {
    size_t off = 0;
    for (size_t s : sizes) off = ((off + 255) & ~static_cast<size_t>(255)) + s;
    return off + 256;
}

// ---- device-side counters (instrumented query runs) -------------------------------------------
struct DevCounters {
    unsigned long long nodes;
    unsigned long long leaves;
    unsigned long long points;
    unsigned long long fallback;
    int error;      // a kernel's bounds check fired
    int give_ups;   // tensor-core filter blocks that gave up (bounded waits ran out)
    int pad[6];
};

// ---- the index ----------------------------------------------------------------------------------
struct QueryPlan {
    uint32_t block = 0;      // threads per block
    bool heap = false;
    bool tc_codes = false;   // filter: k-th bound as buffered codes even where a heap fits
    bool sh_nn = false;
    bool sh_stack = false;
    bool reorder = true;
    bool timing = false;     // record events around the main search kernel
    bool warp = false;       // trees: warp-coherent traversal instead of one search per thread
    bool group = false;      // k-d tree: warp-group search from per-query radii (traversal 2)
    bool box = false;        // k-d tree: per-thread search over tight node boxes (traversal 3)
    uint32_t widen = 0;      // group search: learned seeds x exp(widen * margin / 2) (fewer retries)
    bool bf16 = false;       // brute force: BF16 tensor-core filter + FP32 rescoring
    uint32_t tc_cap = 0;     // candidates kept per query by the filter (0 = default)
    uint32_t leaf_scan = 0;  // 0 = tree leaves
    bool test_give_up = false;  // tensor-core filter blocks give up after their first copy (tests)
};

// Events bracketing a query and each of its search kernels (KNN_QF_TIMING).  A learned-radius
// query runs its seeded search and up to three retry searches: every one of them records a
// span, and the kernel time is the sum of the spans.
struct QueryTiming {
    static constexpr int kMaxSpans = 8;
    cudaEvent_t total0 = nullptr, total1 = nullptr;
    cudaEvent_t span[kMaxSpans][2] = {};
    int spans = 0;
    bool valid = false;
    ~QueryTiming() {
        for (cudaEvent_t e : {total0, total1})
            if (e) cudaEventDestroy(e);
        for (auto& p : span)
            for (cudaEvent_t e : p)
                if (e) cudaEventDestroy(e);
    }
    int ensure() {
        if (total0) return KNN_OK;
        KNN_TRY_CUDA(cudaEventCreate(&total0));
        KNN_TRY_CUDA(cudaEventCreate(&total1));
        for (auto& p : span)
            for (cudaEvent_t& e : p) KNN_TRY_CUDA(cudaEventCreate(&e));
        return KNN_OK;
    }
    // Opens / closes the span of one search kernel on stream s (spans past kMaxSpans are merged
    // into the last one).
    int begin(cudaStream_t s) {
        if (spans < kMaxSpans) KNN_TRY_CUDA(cudaEventRecord(span[spans][0], s));
        return KNN_OK;
    }
    int end(cudaStream_t s) {
        const int i = spans < kMaxSpans ? spans : kMaxSpans - 1;
        KNN_TRY_CUDA(cudaEventRecord(span[i][1], s));
        if (spans < kMaxSpans) ++spans;
        return KNN_OK;
    }
};

// Device-side ordering of the queries issued on one index: they share its workspaces, so a query
// issued on another stream than the previous one waits (on the device) for the previous one to
// finish.  Skipped while the stream is being captured into a graph.
struct StreamOrder {
    cudaEvent_t done = nullptr;
    cudaStream_t last = nullptr;
    bool used = false;
    ~StreamOrder() {
        if (done) cudaEventDestroy(done);
    }
    int before(cudaStream_t s) {
        if (!used || s == last) return KNN_OK;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        KNN_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs == cudaStreamCaptureStatusNone) KNN_TRY_CUDA(cudaStreamWaitEvent(s, done, 0));
        return KNN_OK;
    }
    int after(cudaStream_t s) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        KNN_TRY_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusNone) return KNN_OK;
        if (!done) KNN_TRY_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
        KNN_TRY_CUDA(cudaEventRecord(done, s));
        last = s;
        used = true;
        return KNN_OK;
    }
};

// A second stream of the index for work that can run beside the caller's stream within one
// query (the radius model's seeds beside the locality sort), joined back through events.
struct SideStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~SideStream() {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (stream) cudaStreamDestroy(stream);
    }
    int ensure() {
        if (stream) return KNN_OK;
        KNN_TRY_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        KNN_TRY_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        KNN_TRY_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
        return KNN_OK;
    }
};

// knn_query_host's copy streams: the result rows (by far the larger transfer) are copied out in
// kParts pieces on as many streams at once, so that several copy engines move them.
struct HostIo {
    static constexpr int kParts = 4;
    cudaStream_t part[kParts] = {};
    cudaEvent_t start = nullptr;
    cudaEvent_t done[kParts] = {};
    ~HostIo() {
        if (start) cudaEventDestroy(start);
        for (int i = 0; i < kParts; ++i) {
            if (done[i]) cudaEventDestroy(done[i]);
            if (part[i]) cudaStreamDestroy(part[i]);
        }
    }
    int ensure() {
        if (start) return KNN_OK;
        for (int i = 0; i < kParts; ++i) {
            KNN_TRY_CUDA(cudaStreamCreateWithFlags(&part[i], cudaStreamNonBlocking));
            KNN_TRY_CUDA(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming));
        }
        KNN_TRY_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
        return KNN_OK;
    }
};

}  // namespace knn

struct knn_index {
    int structure = KNN_BRUTE_FORCE;
    int device = 0;
    uint32_t n = 0, dims = 0, dp = 0, aux_dims = 0;
    uint32_t skips = 0, node_depth = 0, leaf_slots = 0, node_count = 0;

    // Brute force: points, padded to `point_stride` floats (a multiple of 4), zero padding.
    knn::DevBuf points;
    uint32_t point_stride = 0;

    // Tensor-core filter (bf_tc.cu), built on first use for any structure: the points grouped
    // into landmark cells, laid out cell by cell in tiles of 256 rows (each cell's last tile
    // padded), with
    //   img    16-bit operand image (FP16 scaled by 2^e, or BF16), 128-byte swizzle, per tile
    //   norm   squared norm of each scaled row (+inf on padding rows)
    //   pts    FP32 coordinates per padded row (stride ps, zero padded) for exact rescoring
    //   ids    index of each padded row in the caller's point array (0xFFFFFFFF on padding)
    //   pmax   per tile: upper bound on the scaled norm of its rows
    //   land   landmarks [cells][ps]; cell_start [cells + 1] first sorted point of each cell;
    //          cell_tile [cells + 1] first tile of each cell; cell_far [cells] float squared
    //          distance from each landmark to its farthest point
    //   limg, lnorm  the landmarks as a 16-bit operand image and their scaled norms (+inf on padding)
    //   cimg, cdata, cmax  the cell centres as a 16-bit operand image, per centre tile their
    //          norms and radii (scaled), and an upper bound on the centres' norms
    struct TensorCoreState {
        knn::DevBuf img, norm, pts, ids, pmax, land, cell_start, cell_tile, cell_far, limg, lnorm, cimg, cdata, cmax, ws;
        // Tree layout (low dims): per tree node its split dimension, value and leaf cell (-1 for
        // splits); per cell its centre and radius (scaled) and box [2][bd] (scaled minima, maxima).
        knn::DevBuf node_dim, node_val, node_leaf, ccentre, cradius, box;
        bool tree = false;
        uint32_t bd = 0;
        uint32_t cells = 0, ptiles = 0, ctiles = 0, ps = 0;
        bool f16 = true;
        float scale = 1.0f;   // power of two applied before rounding to FP16
        bool ready = false;   // built
        bool usable = false;  // built and every scaled norm finite
    } tc;

    // k-d tree: split value per internal node (implicit heap, children 2i+1, 2i+2).
    knn::DevBuf split;
    // k-d tree, warp-group search (built on first use): the tight bounding box of the points
    // under every node down to depth kd_box_depth (subtrees of at most 4 slots), per node
    // lo[q], hi[q] with q = max(4, padded dims) floats each; and the search's own scratch.
    knn::DevBuf kd_box;
    uint32_t kd_box_depth = 0, kd_box_stride = 0;
    knn::DevBuf group_ws;

    // Trees: leaf slots, 2^node_depth leaves x leaf_slots slots; a slot is `leaf_stride` floats:
    // coordinates (dp, zero padded) then the point index as int32 bits (-1 = empty slot).
    knn::DevBuf leaf;
    uint32_t leaf_stride = 0;
    uint32_t leaf_id_at = 0;

    // Ball tree: one ball per node of every level (root .. leaves), node i at
    // ball + i * ball_stride: centre (dp floats), then radius.
    knn::DevBuf ball;
    uint32_t ball_stride = 0;

    size_t device_bytes = 0;
    float build_ms = 0.0f;

    // Scratch for queries, grown on demand, reused across calls.
    knn::DevBuf workspace;
    knn::DevBuf staging;   // device copies of host queries/results (knn_query_host)
    knn::HostIo host_io;   // knn_query_host's copy streams
    knn::SideStream side;  // the radius model's stream within a learned-radius query
    knn::StreamOrder order_guard;
    knn::DevBuf counters;  // DevCounters
    knn::QueryTiming timing;

    // Learned radius model (weights on the device), see radius_model.cu.
    knn::DevBuf model;
    bool has_model = false;
    uint32_t model_k = 0;     // k the model was trained for
    float model_margin = 0.0f;  // the model's margin (log squared distance), kept on the host
    knn::DevBuf seed_ws;      // seeded radii, fallback list and count
    knn::DevBuf tune_ws;      // the autotuner's gathered sample (queries, radii)

    // Autotuned plans, one per k class (8, 16, 32, 64, 128) and learned-radius on/off.
    struct Tuned {
        bool valid = false;
        knn::QueryPlan plan;
        float ms = 0.0f;
        uint32_t candidates = 0;
    } tuned[5][2];
};

namespace knn {

// Stable LSD radix sort of (u32 key, u32 value) pairs over the low `key_bits` bits, 8 bits per
// pass.  Ping-pongs between (keys, vals) and (keys_alt, vals_alt); returns which pair holds
// the result via *in_alt.  `temp` must hold radix_sort_temp_bytes(n).
size_t radix_sort_temp_bytes(uint32_t n);
int radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt,
                     uint32_t n, int key_bits, void* temp, cudaStream_t s, bool* in_alt);

// dst[i] = rows idx[i'] of src ([*][dims] floats); dst_radii[i] = src_radii[idx[i']] when src_radii;
// i' = i, or with stride > 1 the i%32-th entry of the (i/32 * stride)-th run of 32 entries of idx
// (every stride-th group of 32; the caller keeps the last index below idx's length).
int gather_rows(const float* src, const float* src_radii, const uint32_t* idx, uint32_t count, uint32_t dims,
                uint32_t stride, float* dst, float* dst_radii, cudaStream_t s);

// Exclusive prefix sum of per-block counts: counts[rows][cols] row-major -> out, each row
// scanned independently (one thread block per row).
int scan_rows_exclusive(const uint32_t* counts, uint32_t* out, uint32_t rows, uint32_t cols,
                        cudaStream_t s);

// Structure entry points (bf.cu, kd.cu, ball.cu).
int bf_build(knn_index* ix, const float* d_points, cudaStream_t s);
int kd_build(knn_index* ix, const float* d_points, uint32_t build_block, cudaStream_t s);
int ball_build(knn_index* ix, const float* d_points, uint32_t build_block, cudaStream_t s);

struct QueryArgs {
    const float* queries;     // [count][dims] device
    uint32_t count;
    float max_d2;
    const float* radii;       // per-query max_distance2, or null
    uint32_t k;
    int32_t* out_idx;
    float* out_dist;
    DevCounters* counters;    // null unless instrumented
    const uint32_t* order = nullptr;      // explicit thread -> query list (no reordering)
    const uint32_t* count_dev = nullptr;  // device-side count bounding `order` (count is then an upper bound)
};

// Learned radius model (radius_model.cu).
size_t model_floats(uint32_t dims);
int model_gradients(const float* d_prm, uint32_t dims, const float* d_x, const float* d_t, const uint32_t* d_rows,
                    uint32_t batch, float* d_grad, float* d_loss_rows, DevBuf& scratch, cudaStream_t s);
int model_predict(const float* d_prm, uint32_t dims, const float* d_x, uint32_t count, float max_d2,
                  const float* user_radii, float* d_radii, float* d_raw, cudaStream_t s,
                  bool tensor_cores = false);
// Stable list (in `order`, or index order) of the queries that must be searched again, with
// their seeded radii grown by `grow` (capped by the caller's radius).
size_t retry_scratch_bytes(uint32_t count);
int model_retry_list(const uint32_t* order, const int32_t* out_idx, uint32_t count, uint32_t k, float* seeded,
                     float max_d2, const float* user_radii, float grow, uint32_t* list, uint32_t* list_count,
                     void* scratch, DevCounters* counters, cudaStream_t s);
int model_train(knn_index* ix, const float* d_samples, uint32_t count, uint32_t k, const knn_train_opts& o,
                cudaStream_t s, knn_train_report* rep);

int bf_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);
// The structure's own search, without the tensor-core filter (capi.cu).
int query_structure(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);
// Any index through the 16-bit tensor-core filter with tile skipping (bf_tc.cu).
bool tc_supported(uint32_t dims, uint32_t k);

int tc_prepare(knn_index* ix, cudaStream_t s);
int bf_tc_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);
int tc_selftest(uint32_t dims, float* max_rel_err, uint32_t* bad);
// Locality order of a query batch for the trees (kd_order / ball_order), in the index workspace.
// k-d: queries sorted by the node they reach after min(max_levels, 24, tree depth) descent steps.
int kd_order(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order, uint32_t max_levels = 24);
int ball_order(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order);
int kd_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);
// Warp-group k-d search from per-query seed radii (kd_kernels.cu); queries it cannot settle go to
// fb_list / fb_count and are answered by the per-thread search in the same call.
// The k-d node boxes the box and group searches read, built if missing (dims <= 16).
int kd_box_prepare(knn_index* ix, cudaStream_t s);
int kd_group_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, const uint32_t* order, float* seeds,
                   uint32_t* fb_list, uint32_t* fb_count, float seed_scale, cudaStream_t s);
int ball_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);

// Rows of unfilled results (index -1, distance = radius) for an empty point set.
int fill_empty_rows(const QueryArgs& a, cudaStream_t s);

int sm_count();

}  // namespace knn
