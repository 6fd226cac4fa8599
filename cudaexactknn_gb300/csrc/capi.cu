// C ABI of the engine (include/cudaexactknn.h): argument checks, tree shape rules, dispatch to
// the structure implementations, and per-thread error messages.  Nothing here throws across
// the ABI; every failure is a knn_status code plus knn_last_error().

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <cmath>
#include <new>
#include <vector>

#include "knn_internal.h"

namespace {

thread_local char g_last_error[512] = "";

}  // namespace

namespace knn {

namespace {
std::atomic<uint64_t> g_launches{0};
}

void note_launches(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    const char* base = std::strrchr(file, '/');
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", cudaGetErrorString(e), what,
                  base ? base + 1 : file, line);
    return e == cudaErrorMemoryAllocation ? KNN_ERR_OUT_OF_MEMORY : KNN_ERR_CUDA;
}

}  // namespace knn

using knn::fail;

namespace {

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

int check_points(const float* d_points, uint32_t n, uint32_t dims) {
    if (dims == 0) return fail(KNN_ERR_INVALID_ARGUMENT, "dims must be >= 1");
    if (dims > knn::kMaxDims) return fail(KNN_ERR_UNSUPPORTED, "dims %u > %u", dims, knn::kMaxDims);
    if (n > 0x7FFFFFFFu) return fail(KNN_ERR_UNSUPPORTED, "n %u >= 2^31", n);
    if (n > 0 && !d_points) return fail(KNN_ERR_INVALID_ARGUMENT, "points is null");
    return KNN_OK;
}

// Tree shape from n and depthSkips (src/KdTreeGpu.cuh:375-380, src/BallTreeGpu.cuh:614-619).
void tree_shape(knn_index* ix, uint32_t skips, bool ball) {
    const uint32_t l2 = knn::log2_ceil(ix->n);
    uint32_t s = ball ? (skips < 1 ? 1 : skips) : skips;
    if (s > l2 - 1) s = l2 - 1;
    ix->skips = s;
    ix->node_depth = l2 - s;
    ix->leaf_slots = 1u << s;
    ix->node_count = (1u << ix->node_depth) - 1;
}

template <class BuildFn>
int create_common(knn_index* ix, cudaStream_t s, BuildFn&& build) {
    const knn::Range range("knn create");
    cudaGetDevice(&ix->device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    int rc = ix->n ? knn::no_throw(build) : KNN_OK;
    if (rc == KNN_OK) {
        cudaEventRecord(e1, s);
        const cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = knn::cuda_fail(e, "construction", __FILE__, __LINE__);
        else cudaEventElapsedTime(&ix->build_ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == KNN_OK) rc = ix->counters.alloc(sizeof(knn::DevCounters));
    return rc;
}

int finish_create(knn_index* ix, int rc, knn_index** out) {
    if (rc != KNN_OK) {
        delete ix;
        *out = nullptr;
        return rc;
    }
    *out = ix;
    return KNN_OK;
}

int make_plan(const knn_index* ix, const knn_query_opts* o, knn::QueryPlan* p) {
    *p = knn::QueryPlan{};
    if (!o) return KNN_OK;
    if (o->block_size) {
        if (o->block_size > 256)
            return fail(KNN_ERR_INVALID_ARGUMENT, "block_size %u: at most 256", o->block_size);
        p->block = o->block_size;
    }
    p->heap = o->heap_tracking != 0;
    p->sh_nn = o->shmem_tracking != 0;
    p->sh_stack = o->shmem_stack != 0;
    p->reorder = (o->flags & KNN_QF_KEEP_ORDER) == 0;
    p->timing = (o->flags & KNN_QF_TIMING) != 0;
    p->bf16 = (o->flags & KNN_QF_BF16_FILTER) != 0;
    p->tc_codes = (o->flags & KNN_QF_FILTER_CODES) != 0;
    p->test_give_up = (o->flags & KNN_QF_TEST_FILTER_GIVE_UP) != 0;
    p->tc_cap = o->reserved;
    p->leaf_scan = o->leaf_scan;
    if (o->traversal > 3) return fail(KNN_ERR_INVALID_ARGUMENT, "traversal %u: 0 to 3", o->traversal);
    p->warp = o->traversal == 1;
    p->group = o->traversal == 2 && ix->structure == KNN_KD_TREE;
    p->box = o->traversal == 3 && ix->structure == KNN_KD_TREE;
    (void)ix;
    return KNN_OK;
}

// The tensor-core filter where the plan asks for it and its tile fits (k <= 100 at dims > 64),
// else the structure's own search.
int dispatch(knn_index* ix, const knn::QueryArgs& a, const knn::QueryPlan& plan, cudaStream_t s) {
    if (ix->n == 0) return knn::fill_empty_rows(a, s);
    if (plan.bf16 && knn::tc_supported(ix->dims, a.k)) return knn::bf_tc_query(ix, a, plan, s);
    return knn::query_structure(ix, a, plan, s);
}

// Learned radius: seed each query's radius from the model and search.  Queries that found fewer
// than k points inside a seed below the caller's radius are searched again with the radius
// grown 16x (squared distance), twice, and then with the caller's radius, which makes every
// answer exact.  Retry lists keep the locality order of the batch.  (Growing each query by the
// density it saw, (1.5 k / c)^(2/D), was tried on the mixture workload and was slower: queries
// that miss by a little take one more round, and each round is a launch over a scattered list.)
constexpr int kSeedRounds = 3;
constexpr float kSeedGrowth = 16.0f;

int seeded_query(knn_index* ix, const knn::QueryArgs& a, const knn::QueryPlan& plan, cudaStream_t s) {
    // The tensor-core filter tightens each query's bound from its own cell's points before it
    // skips tiles; a seed would only add retries, so it runs unseeded.
    if (plan.bf16) return dispatch(ix, a, plan, s);
    const knn::Range range("learned-radius search");
    const size_t n = a.count;
    KNN_TRY(ix->seed_ws.reserve(knn::carve_bytes({n * 4, n * 4, 256, knn::retry_scratch_bytes(a.count)})));
    knn::Carver c(ix->seed_ws.ptr);
    float* radii = c.take<float>(n);
    uint32_t* list = c.take<uint32_t>(n);
    uint32_t* list_count = c.take<uint32_t>(1);
    void* scratch = c.take<uint8_t>(knn::retry_scratch_bytes(a.count));
    // The seeds and the locality order depend on the queries alone: the model runs on the index's
    // second stream while the order is sorted on the caller's, and the search waits for both.
    KNN_TRY(ix->side.ensure());
    KNN_TRY_CUDA(cudaEventRecord(ix->side.fork, s));
    KNN_TRY_CUDA(cudaStreamWaitEvent(ix->side.stream, ix->side.fork, 0));
    KNN_TRY(knn::model_predict(ix->model.as<float>(), ix->dims, a.queries, a.count, a.max_d2, a.radii, radii,
                               nullptr, ix->side.stream, true));
    KNN_TRY_CUDA(cudaEventRecord(ix->side.join, ix->side.stream));
    const uint32_t* order = nullptr;
    if (plan.reorder && a.count >= 4096) {
        // (The group search takes its warps' queries from the order; 16 levels group them as well
        // as 24 at two radix passes instead of three.)
        if (ix->structure == KNN_KD_TREE) KNN_TRY(knn::kd_order(ix, a, s, &order, plan.group ? 16u : 24u));
        if (ix->structure == KNN_BALL_TREE) KNN_TRY(knn::ball_order(ix, a, s, &order));
    }
    KNN_TRY_CUDA(cudaStreamWaitEvent(s, ix->side.join, 0));
    // The warp-group k-d search settles or hands on every query itself (no retry rounds).
    // Its seeds may be widened by a factor exp(widen * margin / 2) that the autotuner picks: a
    // miss costs the warp another walk, a wider seed only a few more candidates per query.
    if (plan.group && ix->structure == KNN_KD_TREE)
        return knn::kd_group_query(ix, a, plan, order, radii, list, list_count,
                                   std::exp(0.5f * static_cast<float>(plan.widen) * ix->model_margin), s);
    knn::QueryArgs seeded = a;
    seeded.radii = radii;
    seeded.order = order;
    KNN_TRY(dispatch(ix, seeded, plan, s));
    for (int round = 0; round < kSeedRounds; ++round) {
        const float grow = round + 1 < kSeedRounds ? kSeedGrowth : INFINITY;
        KNN_TRY(knn::model_retry_list(order, a.out_idx, a.count, a.k, radii, a.max_d2, a.radii, grow, list,
                                      list_count, scratch, round == 0 ? a.counters : nullptr, s));
        knn::QueryArgs again = a;
        again.radii = radii;
        again.order = list;
        again.count_dev = list_count;
        KNN_TRY(dispatch(ix, again, plan, s));
    }
    return KNN_OK;
}

int k_slot(uint32_t k) {
    switch (knn::k_class(k)) {
        case 8: return 0;
        case 16: return 1;
        case 32: return 2;
        case 64: return 3;
        default: return 4;
    }
}

// Picks the fastest plan for this index and k by timing candidates on up to 32768 of the
// caller's queries (8192 for brute force; CUDA events, best of two runs after a warm-up), in
// three stages: traversal (thread or warp) x leaf bucket size, or the tensor-core filter; then
// block size; then tracker/stack storage.  Results are exact for every candidate.
int autotune(knn_index* ix, const knn::QueryArgs& a, bool learned, cudaStream_t s, knn::QueryPlan* out,
             float* best_ms, uint32_t* tried, bool allow_tc = true) {
    const knn::Range range("autotune");
    knn::QueryArgs t = a;
    // Brute force costs n distances per query; a smaller sample keeps tuning short.  k-d trees
    // take up to 131,072 queries: the warp-group search needs enough warps to fill the GPU before
    // its time per query means what it will mean on a large batch.
    t.count = std::min<uint32_t>(a.count, ix->structure == KNN_BRUTE_FORCE ? 8192u
                                          : ix->structure == KNN_KD_TREE ? 131072u : 32768u);
    t.counters = nullptr;
    cudaEvent_t e0, e1;
    KNN_TRY_CUDA(cudaEventCreate(&e0));
    KNN_TRY_CUDA(cudaEventCreate(&e1));
    int rc = KNN_OK;
    uint32_t n_tried = 0;
    // Sample size from a first run of the default plan on 1,024 queries: about 8 ms of search per
    // candidate run (at least 1,024 queries), so that slow workloads (trees in 32 dimensions that
    // visit most of their nodes) tune in seconds.
    if (t.count > 1024) {
        knn::QueryArgs probe = t;
        probe.count = 1024;
        knn::QueryPlan base;
        base.block = 128;
        float ms = 0.0f;
        int prc = cudaEventRecord(e0, s) == cudaSuccess ? KNN_OK : KNN_ERR_CUDA;
        if (prc == KNN_OK) prc = learned ? seeded_query(ix, probe, base, s) : dispatch(ix, probe, base, s);
        if (prc == KNN_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                              cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            prc = knn::fail(KNN_ERR_CUDA, "autotune: timing the sample");
        if (prc != KNN_OK) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return prc;
        }
        const double per_query = std::max(1e-6, static_cast<double>(ms) / 1024.0);
        const uint32_t fit = static_cast<uint32_t>(std::min(1e9, 8.0 / per_query));
        t.count = std::max(1024u, std::min(t.count, fit & ~127u));
    }
    // k-d trees: the batch's first queries are a sparser set than the batch (fewer queries per
    // region of space), which misjudges the warp-group search, whose cost depends on how close a
    // warp's queries are.  The sample is instead every s-th run of 32 queries of the batch's
    // locality order (s = count / sample), gathered into scratch: each run is a warp's group as
    // the real pass has it, and the runs cover the batch's whole extent.  Its rows are written to
    // the first rows of the caller's result buffers, which the real pass then overwrites.
    if (ix->structure == KNN_KD_TREE && a.count > t.count && !a.order && !a.count_dev) do {
        const uint32_t* order = nullptr;
        if ((rc = knn::kd_order(ix, a, s, &order)) != KNN_OK) break;
        if (order) {
            t.count &= ~31u;
            const uint32_t stride = a.count / t.count;  // >= 1; the last run ends below a.count
            const size_t m = t.count;
            if ((rc = ix->tune_ws.reserve(knn::carve_bytes({m * ix->dims * 4, m * 4}))) != KNN_OK) break;
            knn::Carver c(ix->tune_ws.ptr);
            float* sq = c.take<float>(m * ix->dims);
            float* sr = c.take<float>(m);
            rc = knn::gather_rows(a.queries, a.radii, order, t.count, ix->dims, stride, sq, sr, s);
            t.queries = sq;
            t.radii = a.radii ? sr : nullptr;
        }
    } while (false);
    if (rc != KNN_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
    }
    knn::QueryPlan best;
    best.block = 128;
    float best_t = 1e30f;
    auto time_plan = [&](const knn::QueryPlan& p, float* ms) -> int {
        float best_rep = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            KNN_TRY_CUDA(cudaEventRecord(e0, s));
            KNN_TRY(learned ? seeded_query(ix, t, p, s) : dispatch(ix, t, p, s));
            KNN_TRY_CUDA(cudaEventRecord(e1, s));
            KNN_TRY_CUDA(cudaEventSynchronize(e1));
            float v = 0.0f;
            KNN_TRY_CUDA(cudaEventElapsedTime(&v, e0, e1));
            if (rep > 0) best_rep = std::min(best_rep, v);  // the first run warms caches and workspaces
            // A candidate whose first run already takes 4x the best plan's time cannot win: its
            // warm runs are skipped (in 32-dimensional trees a run can take seconds).
            if (rep == 0 && v > 4.0f * best_t) {
                best_rep = v;
                break;
            }
        }
        *ms = best_rep;
        ++n_tried;
        return KNN_OK;
    };
    auto consider = [&](const knn::QueryPlan& p) -> int {
        float v = 0.0f;
        const int r = time_plan(p, &v);
        if (r == KNN_ERR_INVALID_ARGUMENT) return KNN_OK;  // a launch shape that does not fit: skip
        if (r != KNN_OK) return r;
        if (v < best_t) {
            best_t = v;
            best = p;
        }
        return KNN_OK;
    };
    do {
        // The tensor-core filter, for dims >= 16 (the form it is built for), on any structure.
        const bool try_tc = allow_tc && ix->dims >= 16 && knn::tc_supported(ix->dims, a.k);
        if (learned && ix->structure == KNN_KD_TREE && ix->dp <= 16 && a.k <= 32) {
            // The warp-group search, seeded by the radius model (seeds from each query's own
            // subtree are too loose to pay).
            for (uint32_t leaf : {8u, 16u, 32u}) {
                for (uint32_t widen : {0u, 1u, 2u}) {
                    knn::QueryPlan p;
                    p.block = 128;
                    p.group = true;
                    p.leaf_scan = leaf;
                    p.widen = widen;
                    if ((rc = consider(p)) != KNN_OK) break;
                }
                if (rc != KNN_OK) break;
            }
            if (rc != KNN_OK) break;
        }
        if (ix->structure != KNN_BRUTE_FORCE && try_tc) {
            // First, so that slow tree candidates are cut short against its time.
            knn::QueryPlan p;
            p.block = 128;
            p.bf16 = true;
            if ((rc = consider(p)) != KNN_OK) break;
        }
        if (ix->structure == KNN_KD_TREE && ix->dp <= 16) {
            // The per-thread search over tight node boxes, by bucket size.
            for (uint32_t leaf : {8u, 16u, 32u}) {
                knn::QueryPlan p;
                p.block = 128;
                p.box = true;
                p.leaf_scan = leaf;
                if ((rc = consider(p)) != KNN_OK) break;
            }
            if (rc != KNN_OK) break;
        }
        if (ix->structure != KNN_BRUTE_FORCE) {
            for (bool warp : {false, true}) {
                for (uint32_t leaf : {0u, 4u, 8u, 16u, 32u, 64u}) {
                    if (leaf && leaf <= ix->leaf_slots) continue;
                    knn::QueryPlan p = best;
                    p.bf16 = false;
                    p.group = p.box = false;
                    p.widen = 0;
                    p.warp = warp;
                    p.leaf_scan = leaf;
                    if ((rc = consider(p)) != KNN_OK) break;
                }
                if (rc != KNN_OK) break;
            }
            if (rc != KNN_OK) break;
        } else {
            if ((rc = consider(best)) != KNN_OK) break;
            if (try_tc) {
                knn::QueryPlan p = best;
                p.bf16 = true;
                if ((rc = consider(p)) != KNN_OK) break;
            }
        }
        const knn::QueryPlan stage2 = best;
        for (uint32_t block : {32u, 64u, 256u}) {
            if (stage2.bf16 || stage2.group || stage2.box) break;  // kernels of fixed shape
            knn::QueryPlan p = stage2;
            p.block = block;
            if ((rc = consider(p)) != KNN_OK) break;
        }
        if (rc != KNN_OK) break;
        const knn::QueryPlan stage3 = best;
        for (int v = 1; v < 8 && !stage3.bf16 && !stage3.group && !stage3.box; ++v) {
            knn::QueryPlan p = stage3;
            p.heap = v & 1;
            p.sh_nn = (v >> 1) & 1;
            p.sh_stack = (v >> 2) & 1;
            if (ix->structure == KNN_BRUTE_FORCE && p.sh_stack) continue;
            if ((rc = consider(p)) != KNN_OK) break;
        }
    } while (false);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != KNN_OK) return rc;
    best.timing = false;
    *out = best;
    *best_ms = best_t;
    *tried = n_tried;
    return KNN_OK;
}

}  // namespace

namespace knn {
// The structure's own search (no tensor-core filter).
int query_structure(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, cudaStream_t s) {
    if (ix->n == 0) return fill_empty_rows(a, s);
    switch (ix->structure) {
        case KNN_BRUTE_FORCE: return bf_query(ix, a, plan, s);
        case KNN_KD_TREE: return kd_query(ix, a, plan, s);
        case KNN_BALL_TREE: return ball_query(ix, a, plan, s);
        default: return fail(KNN_ERR_INVALID_ARGUMENT, "unknown structure");
    }
}

// The autotuner's plan for one query batch on one index, among the structure's own searches
// (used by batches, whose persistent kernels run those).
int tune_plan(knn_index* ix, const QueryArgs& a, cudaStream_t s, QueryPlan* out) {
    float ms = 0.0f;
    uint32_t tried = 0;
    return autotune(ix, a, false, s, out, &ms, &tried, false);
}
}  // namespace knn

namespace {

int run_query_checked(knn_index* ix, const knn::QueryArgs& a, const knn_query_opts* opts, cudaStream_t s) {
    if (!ix) return fail(KNN_ERR_INVALID_ARGUMENT, "index is null");
    if (a.k == 0) return fail(KNN_ERR_INVALID_ARGUMENT, "k must be >= 1");
    if (a.k > knn::kMaxK) return fail(KNN_ERR_UNSUPPORTED, "k %u > %u", a.k, knn::kMaxK);
    if (!a.radii && !(a.max_d2 >= 0.0f)) return fail(KNN_ERR_INVALID_ARGUMENT, "max_distance2 must be >= 0 (got %g)", a.max_d2);
    if (a.count > 0x7FFFFFFFu) return fail(KNN_ERR_UNSUPPORTED, "count %u >= 2^31", a.count);
    if (a.count == 0) return KNN_OK;
    if (!a.queries || !a.out_idx || !a.out_dist) return fail(KNN_ERR_INVALID_ARGUMENT, "null query or result pointer");
    const uint32_t flags = opts ? opts->flags : 0;
    if (flags & KNN_QF_LEARNED_RADIUS) {
        if (!ix->has_model) return fail(KNN_ERR_NOT_TRAINED, "no radius model attached to this index");
    }
    knn::QueryPlan plan;
    KNN_TRY(make_plan(ix, opts, &plan));
    const bool learned = (flags & KNN_QF_LEARNED_RADIUS) != 0;
    if ((flags & KNN_QF_AUTOTUNE) && ix->n > 0) {
        auto& slot = ix->tuned[k_slot(a.k)][learned ? 1 : 0];
        if (!slot.valid) {
            KNN_TRY(autotune(ix, a, learned, s, &slot.plan, &slot.ms, &slot.candidates));
            slot.valid = true;
        }
        const bool timing = plan.timing, give_up = plan.test_give_up;
        plan = slot.plan;
        plan.timing = timing;
        plan.test_give_up = give_up;
        plan.reorder = plan.reorder && (flags & KNN_QF_KEEP_ORDER) == 0;
    }
    if (plan.timing) {
        KNN_TRY(ix->timing.ensure());
        ix->timing.valid = false;
        ix->timing.spans = 0;
        KNN_TRY_CUDA(cudaEventRecord(ix->timing.total0, s));
    }
    const int rc = learned && ix->n > 0 ? seeded_query(ix, a, plan, s) : dispatch(ix, a, plan, s);
    if (rc != KNN_OK) return rc;
    if (plan.timing) {
        KNN_TRY_CUDA(cudaEventRecord(ix->timing.total1, s));
        ix->timing.valid = true;
    }
    if (flags & KNN_QF_SYNC) KNN_TRY_CUDA(cudaStreamSynchronize(s));
    return KNN_OK;
}

// Every query entry point: the tensor-core filter builds its layout on first use with host
// containers, the autotuner keeps plans in the index.
int run_query(knn_index* ix, const knn::QueryArgs& a, const knn_query_opts* opts, cudaStream_t s) {
    const knn::Range range("knn query");
    return knn::no_throw([&] {
        if (ix) KNN_TRY(ix->order_guard.before(s));
        KNN_TRY(run_query_checked(ix, a, opts, s));
        return ix ? ix->order_guard.after(s) : KNN_OK;
    });
}

}  // namespace

extern "C" {

int knn_bf_create(const float* d_points, uint32_t n, uint32_t dims, void* stream, knn_index** out) {
    if (!out) return fail(KNN_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    KNN_TRY(check_points(d_points, n, dims));
    auto* ix = new (std::nothrow) knn_index();
    if (!ix) return fail(KNN_ERR_OUT_OF_MEMORY, "host allocation failed");
    ix->structure = KNN_BRUTE_FORCE;
    ix->n = n;
    ix->dims = dims;
    ix->dp = knn::padded_dims(dims);
    ix->aux_dims = dims;
    cudaStream_t s = as_stream(stream);
    const int rc = create_common(ix, s, [&] { return knn::bf_build(ix, d_points, s); });
    return finish_create(ix, rc, out);
}

int knn_kd_create(const float* d_points, uint32_t n, uint32_t dims, uint32_t aux_dims, uint32_t depth_skips,
                  uint32_t build_block, void* stream, knn_index** out) {
    if (!out) return fail(KNN_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    KNN_TRY(check_points(d_points, n, dims));
    if (aux_dims == 0 || aux_dims > dims)
        return fail(KNN_ERR_INVALID_ARGUMENT, "aux_dims %u must be in [1, dims=%u]", aux_dims, dims);
    auto* ix = new (std::nothrow) knn_index();
    if (!ix) return fail(KNN_ERR_OUT_OF_MEMORY, "host allocation failed");
    ix->structure = KNN_KD_TREE;
    ix->n = n;
    ix->dims = dims;
    ix->dp = knn::padded_dims(dims);
    ix->aux_dims = aux_dims;
    if (n) tree_shape(ix, depth_skips, false);
    cudaStream_t s = as_stream(stream);
    const int rc = create_common(ix, s, [&] { return knn::kd_build(ix, d_points, build_block, s); });
    return finish_create(ix, rc, out);
}

int knn_ball_create(const float* d_points, uint32_t n, uint32_t dims, uint32_t depth_skips, uint32_t build_block,
                    void* stream, knn_index** out) {
    if (!out) return fail(KNN_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    KNN_TRY(check_points(d_points, n, dims));
    auto* ix = new (std::nothrow) knn_index();
    if (!ix) return fail(KNN_ERR_OUT_OF_MEMORY, "host allocation failed");
    ix->structure = KNN_BALL_TREE;
    ix->n = n;
    ix->dims = dims;
    ix->dp = knn::padded_dims(dims);
    ix->aux_dims = dims;
    if (n) tree_shape(ix, depth_skips, true);
    cudaStream_t s = as_stream(stream);
    const int rc = create_common(ix, s, [&] { return knn::ball_build(ix, d_points, build_block, s); });
    return finish_create(ix, rc, out);
}

int knn_destroy(knn_index* index) {
    if (!index) return KNN_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    const int dev = index->device;
    if (prev != dev) cudaSetDevice(dev);
    delete index;
    if (prev != dev) cudaSetDevice(prev);
    return KNN_OK;
}

int knn_index_get_info(const knn_index* ix, knn_index_info* out) {
    if (!ix || !out) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    out->structure = static_cast<uint32_t>(ix->structure);
    out->n = ix->n;
    out->dims = ix->dims;
    out->aux_dims = ix->aux_dims;
    out->depth_skips = ix->skips;
    out->node_depth = ix->node_depth;
    out->leaf_slots = ix->leaf_slots;
    out->node_count = ix->node_count;
    out->device_bytes = ix->device_bytes;
    out->build_ms = ix->build_ms;
    out->radius_model = ix->has_model ? 1u : 0u;
    return KNN_OK;
}

int knn_query(knn_index* index, const float* d_queries, uint32_t count, float max_distance2, uint32_t k,
              int32_t* d_indexes, float* d_distances, const knn_query_opts* opts, void* stream) {
    knn::QueryArgs a{d_queries, count, max_distance2, nullptr, k, d_indexes, d_distances, nullptr};
    return run_query(index, a, opts, as_stream(stream));
}

int knn_query_radii(knn_index* index, const float* d_queries, uint32_t count, const float* d_max_distance2,
                    uint32_t k, int32_t* d_indexes, float* d_distances, const knn_query_opts* opts, void* stream) {
    if (!d_max_distance2) return fail(KNN_ERR_INVALID_ARGUMENT, "radii is null");
    knn::QueryArgs a{d_queries, count, 0.0f, d_max_distance2, k, d_indexes, d_distances, nullptr};
    return run_query(index, a, opts, as_stream(stream));
}

int knn_query_host(knn_index* index, const float* h_queries, uint32_t count, float max_distance2, uint32_t k,
                   int32_t* h_indexes, float* h_distances, const knn_query_opts* opts, void* stream) {
    if (!index) return fail(KNN_ERR_INVALID_ARGUMENT, "index is null");
    if (count == 0) return KNN_OK;
    if (!h_queries || !h_indexes || !h_distances) return fail(KNN_ERR_INVALID_ARGUMENT, "null host pointer");
    if (k == 0 || k > knn::kMaxK) return fail(k == 0 ? KNN_ERR_INVALID_ARGUMENT : KNN_ERR_UNSUPPORTED, "k %u", k);
    cudaStream_t s = as_stream(stream);
    const size_t qrow = static_cast<size_t>(index->dims) * sizeof(float);
    const size_t rrow = static_cast<size_t>(k) * sizeof(int32_t);
    const size_t qb = count * qrow, rb = count * rrow;
    KNN_TRY(index->staging.reserve(knn::carve_bytes({qb, rb, rb})));
    knn::Carver c(index->staging.ptr);
    float* dq = c.take<float>(static_cast<size_t>(count) * index->dims);
    int32_t* di = c.take<int32_t>(static_cast<size_t>(count) * k);
    float* dd = c.take<float>(static_cast<size_t>(count) * k);
    KNN_TRY_CUDA(cudaMemcpyAsync(dq, h_queries, qb, cudaMemcpyHostToDevice, s));
    knn::QueryArgs a{dq, count, max_distance2, nullptr, k, di, dd, nullptr};
    KNN_TRY(run_query(index, a, opts, s));
    // The rows go out in pieces on the index's copy streams at once (several copy engines), each
    // piece after the search; the caller's stream then waits for every piece.
    knn::HostIo& io = index->host_io;
    KNN_TRY(io.ensure());
    KNN_TRY_CUDA(cudaEventRecord(io.start, s));
    constexpr int P = knn::HostIo::kParts;
    const uint32_t per = (count + P / 2 - 1) / (P / 2);  // rows per piece: two pieces per array
    for (int i = 0; i < P; ++i) {
        const uint32_t first = (i / 2) * per;
        if (first >= count) continue;
        const size_t rows = std::min<uint32_t>(per, count - first);
        KNN_TRY_CUDA(cudaStreamWaitEvent(io.part[i], io.start, 0));
        const size_t off = static_cast<size_t>(first) * k;
        if (i % 2 == 0)
            KNN_TRY_CUDA(cudaMemcpyAsync(h_indexes + off, di + off, rows * rrow, cudaMemcpyDeviceToHost, io.part[i]));
        else
            KNN_TRY_CUDA(cudaMemcpyAsync(h_distances + off, dd + off, rows * rrow, cudaMemcpyDeviceToHost, io.part[i]));
        KNN_TRY_CUDA(cudaEventRecord(io.done[i], io.part[i]));
        KNN_TRY_CUDA(cudaStreamWaitEvent(s, io.done[i], 0));
    }
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    return KNN_OK;
}

int knn_query_stats(knn_index* index, const float* d_queries, uint32_t count, float max_distance2, uint32_t k,
                    int32_t* d_indexes, float* d_distances, const knn_query_opts* opts, void* stream,
                    knn_query_counters* out) {
    if (!index || !out) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t s = as_stream(stream);
    auto* dc = index->counters.as<knn::DevCounters>();
    KNN_TRY_CUDA(cudaMemsetAsync(dc, 0, sizeof(knn::DevCounters), s));
    knn::QueryArgs a{d_queries, count, max_distance2, nullptr, k, d_indexes, d_distances, dc};
    KNN_TRY(run_query(index, a, opts, s));
    knn::DevCounters hc{};
    KNN_TRY_CUDA(cudaMemcpyAsync(&hc, dc, sizeof(hc), cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    std::memset(out, 0, sizeof(*out));
    out->nodes_visited = hc.nodes;
    out->leaves_visited = hc.leaves;
    out->points_scanned = hc.points;
    out->fallback_queries = hc.fallback;
    out->filter_give_ups = static_cast<uint64_t>(hc.give_ups);
    if (hc.error) return fail(KNN_ERR_DEVICE_LIMIT, "a query kernel's stack bound check fired");
    return KNN_OK;
}

int knn_last_query_timing(knn_index* index, float* total_ms, float* kernel_ms) {
    if (!index || !total_ms || !kernel_ms) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (!index->timing.valid) return fail(KNN_ERR_INVALID_ARGUMENT, "no timed query on this index");
    KNN_TRY_CUDA(cudaEventSynchronize(index->timing.total1));
    KNN_TRY_CUDA(cudaEventElapsedTime(total_ms, index->timing.total0, index->timing.total1));
    float sum = 0.0f;
    for (int i = 0; i < index->timing.spans; ++i) {
        float v = 0.0f;
        KNN_TRY_CUDA(cudaEventElapsedTime(&v, index->timing.span[i][0], index->timing.span[i][1]));
        sum += v;
    }
    *kernel_ms = sum;
    return KNN_OK;
}

int knn_tuned_plan(const knn_index* index, uint32_t k, uint32_t learned_radius, knn_query_opts* out, float* ms) {
    if (!index || !out) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (k == 0 || k > knn::kMaxK) return fail(KNN_ERR_INVALID_ARGUMENT, "k %u", k);
    const auto& slot = index->tuned[k_slot(k)][learned_radius ? 1 : 0];
    if (!slot.valid) return fail(KNN_ERR_INVALID_ARGUMENT, "no tuned plan for k %u yet", k);
    std::memset(out, 0, sizeof(*out));
    out->block_size = slot.plan.block;
    out->heap_tracking = slot.plan.heap;
    out->shmem_tracking = slot.plan.sh_nn;
    out->shmem_stack = slot.plan.sh_stack;
    out->leaf_scan = slot.plan.leaf_scan;
    out->traversal = slot.plan.group ? 2u : slot.plan.box ? 3u : (slot.plan.warp ? 1u : 0u);
    out->flags = slot.plan.bf16 ? KNN_QF_BF16_FILTER : 0u;
    out->reserved = slot.candidates;
    if (ms) *ms = slot.ms;
    return KNN_OK;
}

int knn_tc_selftest(uint32_t dims, float* max_rel_err, uint32_t* mismatches) {
    if (!max_rel_err || !mismatches) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (dims == 0 || dims > 128) return fail(KNN_ERR_UNSUPPORTED, "dims %u", dims);
    return knn::no_throw([&] { return knn::tc_selftest(dims, max_rel_err, mismatches); });
}

uint64_t knn_launch_count(void) { return knn::g_launches.load(); }

int knn_radius_model_train(knn_index* index, const float* d_samples, uint32_t count, uint32_t k,
                           const knn_train_opts* opts, void* stream, knn_train_report* report) {
    if (!index || !d_samples) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (index->n == 0) return fail(KNN_ERR_INVALID_ARGUMENT, "empty point set");
    if (count < 16) return fail(KNN_ERR_INVALID_ARGUMENT, "need at least 16 samples (got %u)", count);
    if (k == 0 || k > knn::kMaxK) return fail(k ? KNN_ERR_UNSUPPORTED : KNN_ERR_INVALID_ARGUMENT, "k %u", k);
    // With fewer than k points every sample's k-th distance is unbounded: no target to learn.
    if (k > index->n) return fail(KNN_ERR_INVALID_ARGUMENT, "k %u exceeds the %u points of the index", k, index->n);
    knn_train_opts o{};
    if (opts) o = *opts;
    if (!o.steps) o.steps = 3000;
    if (!o.batch) o.batch = 1024;
    if (!(o.lr > 0.0f)) o.lr = 3e-3f;
    if (!(o.coverage > 0.0f && o.coverage < 1.0f)) o.coverage = 0.98f;
    if (!o.seed) o.seed = 1;
    const knn::Range range("radius model training");
    return knn::no_throw([&] { return knn::model_train(index, d_samples, count, k, o, as_stream(stream), report); });
}

int knn_radius_model_predict(knn_index* index, const float* d_queries, uint32_t count, float* d_log_kth,
                             void* stream) {
    if (!index || !d_log_kth || (count && !d_queries)) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (!index->has_model) return fail(KNN_ERR_NOT_TRAINED, "no radius model attached to this index");
    if (!count) return KNN_OK;
    return knn::model_predict(index->model.as<float>(), index->dims, d_queries, count, INFINITY, nullptr, nullptr,
                              d_log_kth, as_stream(stream));
}

uint32_t knn_radius_model_size(uint32_t dims) {
    return dims && dims <= knn::kMaxDims ? static_cast<uint32_t>(knn::model_floats(dims)) : 0u;
}

int knn_radius_model_export(const knn_index* index, float* h_params, uint32_t capacity) {
    if (!index || !h_params) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (!index->has_model) return fail(KNN_ERR_NOT_TRAINED, "no radius model attached to this index");
    const size_t n = knn::model_floats(index->dims);
    if (capacity < n) return fail(KNN_ERR_INVALID_ARGUMENT, "capacity %u < %zu", capacity, n);
    KNN_TRY_CUDA(cudaMemcpy(h_params, index->model.ptr, n * 4, cudaMemcpyDeviceToHost));
    return KNN_OK;
}

int knn_radius_model_import(knn_index* index, const float* h_params, uint32_t count, uint32_t k) {
    if (!index || !h_params) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    const size_t n = knn::model_floats(index->dims);
    if (count != n) return fail(KNN_ERR_INVALID_ARGUMENT, "model for dims %u has %zu floats, got %u", index->dims, n, count);
    KNN_TRY(index->model.alloc(n * 4));
    KNN_TRY_CUDA(cudaMemcpy(index->model.ptr, h_params, n * 4, cudaMemcpyHostToDevice));
    index->has_model = true;
    index->model_k = k;
    index->model_margin = h_params[n - 1];  // the margin is the model's last parameter
    return KNN_OK;
}

int knn_radius_model_gradients(const float* h_params, uint32_t dims, const float* h_x, const float* h_targets,
                               uint32_t batch, float* h_grad, float* h_loss) {
    if (!h_params || !h_x || !h_targets || !h_grad || !h_loss || !batch)
        return fail(KNN_ERR_INVALID_ARGUMENT, "null argument or empty batch");
    if (!dims || dims > knn::kMaxDims) return fail(KNN_ERR_UNSUPPORTED, "dims %u", dims);
    const size_t np = knn::model_floats(dims);
    knn::DevBuf buf, scratch;
    KNN_TRY(buf.alloc(knn::carve_bytes({np * 4, np * 4, static_cast<size_t>(batch) * dims * 4,
                                        static_cast<size_t>(batch) * 4, static_cast<size_t>(batch) * 4})));
    knn::Carver c(buf.ptr);
    float* prm = c.take<float>(np);
    float* grad = c.take<float>(np);
    float* x = c.take<float>(static_cast<size_t>(batch) * dims);
    float* t = c.take<float>(batch);
    float* loss = c.take<float>(batch);
    KNN_TRY_CUDA(cudaMemcpy(prm, h_params, np * 4, cudaMemcpyHostToDevice));
    KNN_TRY_CUDA(cudaMemcpy(x, h_x, static_cast<size_t>(batch) * dims * 4, cudaMemcpyHostToDevice));
    KNN_TRY_CUDA(cudaMemcpy(t, h_targets, static_cast<size_t>(batch) * 4, cudaMemcpyHostToDevice));
    KNN_TRY(knn::model_gradients(prm, dims, x, t, nullptr, batch, grad, loss, scratch, nullptr));
    const size_t trainable = np - dims * 32 - 2 * dims - 1;  // fixed projection, scaling, margin follow
    KNN_TRY_CUDA(cudaMemcpy(h_grad, grad, trainable * 4, cudaMemcpyDeviceToHost));
    return knn::no_throw([&]() -> int {
        std::vector<float> lr(batch);
        KNN_TRY_CUDA(cudaMemcpy(lr.data(), loss, static_cast<size_t>(batch) * 4, cudaMemcpyDeviceToHost));
        double total = 0;
        for (float v : lr) total += v;
        *h_loss = static_cast<float>(total);
        return KNN_OK;
    });
}

const char* knn_status_string(int status) {
    switch (status) {
        case KNN_OK: return "ok";
        case KNN_ERR_INVALID_ARGUMENT: return "invalid argument";
        case KNN_ERR_UNSUPPORTED: return "unsupported size";
        case KNN_ERR_CUDA: return "CUDA error";
        case KNN_ERR_OUT_OF_MEMORY: return "out of device memory";
        case KNN_ERR_DEVICE_LIMIT: return "device bounds check fired";
        case KNN_ERR_NOT_TRAINED: return "no radius model";
        default: return "unknown status";
    }
}

const char* knn_last_error(void) { return g_last_error; }

int knn_version(void) { return 10000; }

}  // extern "C"
