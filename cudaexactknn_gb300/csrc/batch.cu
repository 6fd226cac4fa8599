// Batches of independent point sets and query batches (uneven n, dims and k) in one CUDA-graph
// launch.  The reference answers one (structure, query) pair per batchKnn call and synchronises
// the device after each (src/KdTreeGpu.cuh:393-410, src/BallTreeGpu.cuh:631-648); a caller with
// many small sets pays a launch and a device-wide sync per set.
//
// Here the items are grouped into classes of equal (tree, padded dims, k capacity).  Each class
// runs as one persistent kernel whose blocks take work blocks (blockDim queries of one set) from a
// shared counter, so small and large sets share the GPU within a single launch; the queries of a
// class are first sorted together by (set, leaf they descend to) for locality.  The classes are
// the parallel branches of one captured CUDA graph, replayed with one cudaGraphLaunch per run.
// Plans (leaf bucket size, block size, per-thread or warp-coherent traversal) come from the
// autotuner, run on each class's largest set; with autotuning, a class of dims >= 16 whose largest
// set answers faster through the tensor-core filter runs its items through the filter instead, one
// after another on a branch of their own.

#include <algorithm>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <tuple>
#include <vector>

#include "knn_internal.h"

namespace knn {

template <uint32_t DP>
int kd_batch_launch(const void*, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t*, uint32_t*,
                    uint32_t*, bool, cudaStream_t);
template <uint32_t DP>
int ball_batch_launch(const void*, uint32_t, uint32_t, uint32_t, uint32_t, bool, uint32_t, uint32_t*, uint32_t*,
                      uint32_t*, bool, cudaStream_t);
size_t kd_batch_set_bytes();
size_t ball_batch_set_bytes();
void kd_batch_set_fill(void*, const knn_index*, const QueryArgs&, const QueryPlan&, const uint32_t*, uint32_t,
                       uint32_t, uint32_t);
void ball_batch_set_fill(void*, const knn_index*, const QueryArgs&, const QueryPlan&, const uint32_t*, uint32_t,
                         uint32_t, uint32_t);
int tune_plan(knn_index* ix, const QueryArgs& a, cudaStream_t s, QueryPlan* out);
int query_structure(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s);

namespace {

// mode: 0 per-thread search, 1 warp-coherent, 2 box search (k-d only).
int batch_launch(int structure, uint32_t dp, const void* sets, uint32_t nsets, uint32_t total_queries,
                 uint32_t total_blocks, uint32_t kmax, uint32_t mode, uint32_t block, uint32_t* counter, uint32_t* keys,
                 uint32_t* vals, bool key_pass, cudaStream_t s) {
#define KNN_BL(D_)                                                                                                  \
    case D_:                                                                                                        \
        return structure == KNN_KD_TREE                                                                             \
                   ? kd_batch_launch<D_>(sets, nsets, total_queries, total_blocks, kmax, mode, block, counter, keys, \
                                         vals, key_pass, s)                                                         \
                   : ball_batch_launch<D_>(sets, nsets, total_queries, total_blocks, kmax, mode == 1, block, counter, \
                                           keys, vals, key_pass, s);
    switch (dp) {
        KNN_BL(1) KNN_BL(2) KNN_BL(3) KNN_BL(4) KNN_BL(8) KNN_BL(16) KNN_BL(32) KNN_BL(64) KNN_BL(128)
        default: return fail(KNN_ERR_UNSUPPORTED, "dims");
    }
#undef KNN_BL
}

}  // namespace
}  // namespace knn

struct knn_batch {
    struct Class {
        int structure = 0;
        uint32_t dp = 0, kmax = 0;
        knn::QueryPlan plan;
        std::vector<uint32_t> items;
        uint32_t total_queries = 0, total_blocks = 0;
        bool sort = false;
        uint32_t key_bits = 0;
        knn::DevBuf sets, scratch;
        uint32_t *counter = nullptr, *keys = nullptr, *vals = nullptr, *keys_alt = nullptr, *vals_alt = nullptr;
        void* sort_temp = nullptr;
        const uint32_t* order = nullptr;
        bool tc = false;  // items run one by one through the tensor-core filter instead
    };
    std::vector<knn_batch_item> items;
    std::deque<Class> classes;  // stable addresses (the device buffers are not movable)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    ~knn_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto s : streams) cudaStreamDestroy(s);
        for (auto e : events) cudaEventDestroy(e);
    }
};

namespace {

using knn::fail;

uint32_t class_mode(const knn_batch::Class& c) { return c.plan.box ? 2u : c.plan.warp ? 1u : 0u; }

// Enqueues one class: locality sort (key pass + radix sort) then the persistent search kernel.
int enqueue_class(knn_batch::Class& c, cudaStream_t s) {
    if (c.sort) {
        KNN_TRY(knn::batch_launch(c.structure, c.dp, c.sets.ptr, static_cast<uint32_t>(c.items.size()), c.total_queries,
                                  c.total_blocks, c.kmax, class_mode(c), c.plan.block, c.counter, c.keys, c.vals, true, s));
        bool in_alt = false;
        KNN_TRY(knn::radix_sort_pairs(c.keys, c.vals, c.keys_alt, c.vals_alt, c.total_queries,
                                      static_cast<int>(c.key_bits), c.sort_temp, s, &in_alt));
        if (c.order != (in_alt ? c.vals_alt : c.vals)) return fail(KNN_ERR_INVALID_ARGUMENT, "batch order buffer moved");
    }
    KNN_TRY_CUDA(cudaMemsetAsync(c.counter, 0, sizeof(uint32_t), s));
    return knn::batch_launch(c.structure, c.dp, c.sets.ptr, static_cast<uint32_t>(c.items.size()), c.total_queries,
                             c.total_blocks, c.kmax, class_mode(c), c.plan.block, c.counter, c.keys, c.vals, false, s);
}

knn::QueryArgs item_args(const knn_batch_item& it) {
    return knn::QueryArgs{it.d_queries, it.count, it.max_distance2, nullptr, it.k, it.d_indexes, it.d_distances, nullptr};
}

// Best of two timed runs of one query on `s` (the run before them warms caches and workspaces).
template <class F>
int time_query(F&& run, cudaStream_t s, float* ms) {
    cudaEvent_t e0, e1;
    KNN_TRY_CUDA(cudaEventCreate(&e0));
    KNN_TRY_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int rc = KNN_OK;
    for (int rep = 0; rep < 3 && rc == KNN_OK; ++rep) {
        cudaEventRecord(e0, s);
        rc = run();
        cudaEventRecord(e1, s);
        if (rc == KNN_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(KNN_ERR_CUDA, "event");
        float v = 0.0f;
        if (rc == KNN_OK && rep > 0 && cudaEventElapsedTime(&v, e0, e1) == cudaSuccess) best = std::min(best, v);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return rc;
}

int check_item(const knn_batch_item& it) {
    if (!it.index) return fail(KNN_ERR_INVALID_ARGUMENT, "batch item without index");
    if (it.index->structure != KNN_KD_TREE && it.index->structure != KNN_BALL_TREE)
        return fail(KNN_ERR_UNSUPPORTED, "batches take k-d and ball tree indexes");
    if (it.k == 0 || it.k > knn::kMaxK) return fail(it.k ? KNN_ERR_UNSUPPORTED : KNN_ERR_INVALID_ARGUMENT, "k %u", it.k);
    if (!(it.max_distance2 >= 0.0f)) return fail(KNN_ERR_INVALID_ARGUMENT, "max_distance2 must be >= 0");
    if (it.count && (!it.d_queries || !it.d_indexes || !it.d_distances)) return fail(KNN_ERR_INVALID_ARGUMENT, "null pointer");
    if (it.index->n == 0) return fail(KNN_ERR_UNSUPPORTED, "batch item with an empty point set");
    return KNN_OK;
}

}  // namespace

namespace {

int batch_create(const knn_batch_item* items, uint32_t count, uint32_t flags, void* stream, knn_batch** out) {
    const knn::Range range("knn batch create");
    if (out) *out = nullptr;
    if (!out || (count && !items)) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t i = 0; i < count; ++i) KNN_TRY(check_item(items[i]));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::unique_ptr<knn_batch> b(new knn_batch());
    b->items.assign(items, items + count);
    std::map<std::tuple<int, uint32_t, uint32_t>, uint32_t> class_of;
    for (uint32_t i = 0; i < count; ++i) {
        const auto& it = items[i];
        if (it.count == 0) continue;
        const auto key = std::make_tuple(it.index->structure, it.index->dp, knn::k_class(it.k));
        auto f = class_of.find(key);
        if (f == class_of.end()) {
            class_of[key] = static_cast<uint32_t>(b->classes.size());
            b->classes.emplace_back();
            auto& c = b->classes.back();
            c.structure = it.index->structure;
            c.dp = it.index->dp;
            c.kmax = knn::k_class(it.k);
            f = class_of.find(key);
        }
        b->classes[f->second].items.push_back(i);
    }
    int rc = KNN_OK;
    for (auto& c : b->classes) {
        // Plan: the autotuned plan of the class's largest set, or per-thread search with the
        // tree's own leaves.
        uint32_t largest = c.items[0];
        for (uint32_t i : c.items)
            if (items[i].count > items[largest].count) largest = i;
        c.plan.block = 128;
        if (flags & KNN_QF_AUTOTUNE) {
            const auto& it = items[largest];
            const knn::QueryArgs a = item_args(it);
            // dims >= 16: the tensor-core filter instead of the class's tree search when it is
            // faster per query on the class's largest set.  Both are first timed on a sample (the
            // filter on 8,192 queries, the tree's default search on 1,024: a whole set of
            // 32-dimensional uniform points takes seconds per tree search); a filter four times
            // faster than that settles it, otherwise the tree is autotuned and compared again.
            bool tc_ok = it.index->dims >= 16;
            for (uint32_t i : c.items) tc_ok = tc_ok && knn::tc_supported(items[i].index->dims, items[i].k);
            float tc_per_q = 0.0f;
            if (tc_ok) {
                knn::QueryPlan tp;
                tp.bf16 = true;
                knn::QueryArgs at = a, ad = a;
                at.count = std::min<uint32_t>(a.count, 8192u);
                ad.count = std::min<uint32_t>(a.count, 1024u);
                float t_tc = 0.0f, t_tree = 0.0f;
                if ((rc = time_query([&] { return knn::bf_tc_query(it.index, at, tp, s); }, s, &t_tc)) != KNN_OK) break;
                if ((rc = time_query([&] { return knn::query_structure(it.index, ad, c.plan, s); }, s, &t_tree)) != KNN_OK)
                    break;
                tc_per_q = t_tc / at.count;
                c.tc = 4.0f * tc_per_q < t_tree / ad.count;
            }
            if (!c.tc) {
                if ((rc = knn::tune_plan(it.index, a, s, &c.plan)) != KNN_OK) break;
                c.plan.heap = c.plan.sh_nn = c.plan.sh_stack = false;  // the batch kernels keep tracker and stack in registers
                if (tc_ok) {
                    knn::QueryArgs at = a;
                    at.count = std::min<uint32_t>(a.count, 8192u);
                    float t_tree = 0.0f;
                    if ((rc = time_query([&] { return knn::query_structure(it.index, at, c.plan, s); }, s, &t_tree)) !=
                        KNN_OK)
                        break;
                    c.tc = tc_per_q < t_tree / at.count;
                }
            }
        }
        if (c.tc) {
            // Prepare each index's filter layout and workspace now (capture cannot allocate).
            knn::QueryPlan tp;
            tp.bf16 = true;
            for (uint32_t i : c.items)
                if ((rc = knn::bf_tc_query(items[i].index, item_args(items[i]), tp, s)) != KNN_OK) break;
            if (rc != KNN_OK) break;
            if (cudaStreamSynchronize(s) != cudaSuccess) {
                rc = fail(KNN_ERR_CUDA, "stream synchronize");
                break;
            }
            continue;
        }
        if (c.plan.box) {
            // The box search reads each index's node boxes: build them now (capture cannot allocate).
            for (uint32_t i : c.items)
                if ((rc = knn::kd_box_prepare(items[i].index, s)) != KNN_OK) break;
            if (rc != KNN_OK) break;
        }
        const uint32_t block = c.plan.block;
        uint32_t first_block = 0;
        for (uint32_t i : c.items) {
            c.total_queries += items[i].count;
            first_block += knn::ceil_div(items[i].count, block);
        }
        c.total_blocks = first_block;
        c.sort = (flags & KNN_QF_KEEP_ORDER) == 0;
        uint32_t set_bits = 0;
        while ((1u << set_bits) < c.items.size()) ++set_bits;
        c.key_bits = 24 + set_bits;
        if (c.key_bits > 32) {
            rc = fail(KNN_ERR_UNSUPPORTED, "more than 256 sets in one class");
            break;
        }
        const size_t nq = c.total_queries;
        if ((rc = c.scratch.alloc(knn::carve_bytes({4, nq * 4, nq * 4, nq * 4, nq * 4,
                                                    knn::radix_sort_temp_bytes(c.total_queries)}))) != KNN_OK)
            break;
        knn::Carver cv(c.scratch.ptr);
        c.counter = cv.take<uint32_t>(1);
        c.keys = cv.take<uint32_t>(nq);
        c.vals = cv.take<uint32_t>(nq);
        c.keys_alt = cv.take<uint32_t>(nq);
        c.vals_alt = cv.take<uint32_t>(nq);
        c.sort_temp = cv.take<uint8_t>(knn::radix_sort_temp_bytes(c.total_queries));
        // The sort's result buffer depends only on the pass count (8 bits per pass).
        const uint32_t passes = (c.key_bits + 7) / 8;
        c.order = c.sort ? ((passes % 2) ? c.vals_alt : c.vals) : nullptr;
        const size_t set_bytes = c.structure == KNN_KD_TREE ? knn::kd_batch_set_bytes() : knn::ball_batch_set_bytes();
        std::vector<uint8_t> host(set_bytes * c.items.size());
        first_block = 0;
        uint32_t qoff = 0;
        for (size_t j = 0; j < c.items.size(); ++j) {
            const auto& it = items[c.items[j]];
            knn::QueryArgs a{it.d_queries, it.count, it.max_distance2, nullptr, it.k, it.d_indexes, it.d_distances, nullptr};
            const uint32_t* order = c.order ? c.order + qoff : nullptr;
            if (c.structure == KNN_KD_TREE)
                knn::kd_batch_set_fill(host.data() + j * set_bytes, it.index, a, c.plan, order, qoff, first_block, qoff);
            else
                knn::ball_batch_set_fill(host.data() + j * set_bytes, it.index, a, c.plan, order, qoff, first_block, qoff);
            first_block += knn::ceil_div(it.count, block);
            qoff += it.count;
        }
        if ((rc = c.sets.alloc(host.size())) != KNN_OK) break;
        const cudaError_t e = cudaMemcpy(c.sets.ptr, host.data(), host.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            rc = knn::cuda_fail(e, "cudaMemcpy(batch sets)", __FILE__, __LINE__);
            break;
        }
    }
    if (rc == KNN_OK && !b->classes.empty()) {
        // Capture: the classes as parallel branches forked from and joined into a capture stream.
        cudaStream_t cap = nullptr;
        rc = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess ? KNN_OK
                                                                                   : fail(KNN_ERR_CUDA, "stream create");
        if (rc == KNN_OK) {
            b->streams.push_back(cap);
            for (size_t i = 0; i <= b->classes.size() && rc == KNN_OK; ++i) {  // one stream per class, one for the filter
                cudaStream_t cs = nullptr;
                cudaEvent_t ev = nullptr;
                if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
                    rc = fail(KNN_ERR_CUDA, "stream/event create");
                b->streams.push_back(cs);
                b->events.push_back(ev);
            }
            cudaEvent_t fork = nullptr;
            if (rc == KNN_OK && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess)
                rc = fail(KNN_ERR_CUDA, "event create");
            if (fork) b->events.push_back(fork);
            if (rc == KNN_OK && cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                rc = fail(KNN_ERR_CUDA, "graph capture could not start");
            if (rc == KNN_OK) {
                int erc = cudaEventRecord(fork, cap) == cudaSuccess ? KNN_OK : fail(KNN_ERR_CUDA, "record");
                // Filter classes share one branch, item after item: items of one index share its
                // filter workspace.
                const size_t nc = b->classes.size();
                cudaStream_t tcs = b->streams[1 + nc];

                if (erc == KNN_OK && cudaStreamWaitEvent(tcs, fork, 0) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "fork");
                for (size_t i = 0; i < nc && erc == KNN_OK; ++i) {
                    auto& c = b->classes[i];
                    if (c.tc) {
                        knn::QueryPlan tp;
                        tp.bf16 = true;
                        for (uint32_t j : c.items)
                            if (erc == KNN_OK) erc = knn::bf_tc_query(items[j].index, item_args(items[j]), tp, tcs);

                        continue;
                    }
                    cudaStream_t cs = b->streams[1 + i];
                    if (cudaStreamWaitEvent(cs, fork, 0) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "fork");
                    if (erc == KNN_OK) erc = enqueue_class(c, cs);
                    if (erc == KNN_OK && cudaEventRecord(b->events[i], cs) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "join record");
                    if (erc == KNN_OK && cudaStreamWaitEvent(cap, b->events[i], 0) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "join");
                }
                if (erc == KNN_OK && cudaEventRecord(b->events[nc], tcs) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "join record");
                if (erc == KNN_OK && cudaStreamWaitEvent(cap, b->events[nc], 0) != cudaSuccess) erc = fail(KNN_ERR_CUDA, "join");

                cudaGraph_t g = nullptr;
                const cudaError_t ee = cudaStreamEndCapture(cap, &g);
                if (erc == KNN_OK && ee != cudaSuccess) erc = knn::cuda_fail(ee, "cudaStreamEndCapture", __FILE__, __LINE__);
                b->graph = g;
                if (erc == KNN_OK) {
                    const cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
                    if (ie != cudaSuccess) erc = knn::cuda_fail(ie, "cudaGraphInstantiate", __FILE__, __LINE__);
                }
                rc = erc;
            }
        }
    }
    if (rc != KNN_OK) return rc;
    *out = b.release();
    return KNN_OK;
}

}  // namespace

extern "C" {

// The plan's containers allocate host memory; an allocation failure there is a status, not an
// exception thrown across the C ABI.
int knn_batch_create(const knn_batch_item* items, uint32_t count, uint32_t flags, void* stream, knn_batch** out) {
    return knn::no_throw([&] { return batch_create(items, count, flags, stream, out); });
}

int knn_batch_run(knn_batch* batch, void* stream) {
    if (!batch) return fail(KNN_ERR_INVALID_ARGUMENT, "batch is null");
    if (!batch->exec) return KNN_OK;  // nothing to run (every item had zero queries)
    const knn::Range range("knn batch run");
    KNN_TRY_CUDA(cudaGraphLaunch(batch->exec, static_cast<cudaStream_t>(stream)));
    knn::note_launches(1);
    return KNN_OK;
}

int knn_batch_info(const knn_batch* batch, uint32_t* classes, uint32_t* kernels_per_run) {
    if (!batch || !classes || !kernels_per_run) return fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    *classes = static_cast<uint32_t>(batch->classes.size());
    size_t nodes = 0;
    uint32_t kernels = 0;
    if (batch->graph) {
        KNN_TRY_CUDA(cudaGraphGetNodes(batch->graph, nullptr, &nodes));
        std::vector<cudaGraphNode_t> list(nodes);
        if (nodes) KNN_TRY_CUDA(cudaGraphGetNodes(batch->graph, list.data(), &nodes));
        for (auto n : list) {
            cudaGraphNodeType t;
            KNN_TRY_CUDA(cudaGraphNodeGetType(n, &t));
            kernels += t == cudaGraphNodeTypeKernel;
        }
    }
    *kernels_per_run = kernels;
    return KNN_OK;
}

int knn_batch_destroy(knn_batch* batch) {
    delete batch;
    return KNN_OK;
}

}  // extern "C"
