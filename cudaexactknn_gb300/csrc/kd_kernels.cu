// k-d tree query kernels, one translation unit per padded dimension count (KNN_DP).
//
// Replaces KdTreeKernels::knnDevice and its four storage variants (src/KdTreeGpu.cuh:37-184).
// Same depth-first search: descend to the closer child, push the farther child with the squared
// distance to its splitting plane, scan leaves, pop.  Differences:
//   * queries are reordered so that neighbouring threads descend to neighbouring leaves (sorted
//     by the leaf each query reaches), which keeps a warp's node and leaf loads together;
//   * the plane bound fl((q[dim]-split)^2) never exceeds the float distance of any point
//     beyond the plane (float subtraction and rounding are monotone and every term of the
//     fused sum is non-negative), and nodes are pruned only when bound > k-th distance, so no
//     point whose key could enter the top-k is skipped, ties included;
//   * k-th key cached in a register; tracker/stack storage chosen by the plan.

#include <algorithm>
#include <cstring>

#include "tree_query.cuh"

#ifndef KNN_DP
#error "compile with -DKNN_DP=<padded dims>"
#endif

namespace knn {

struct KdParams {
    const float* split;
    const float* leaf;
    uint32_t leaf_stride;
    uint32_t node_count;
    uint32_t node_depth;
    uint32_t stop_depth;  // descend to this depth, then scan the subtree's slots
    uint32_t leaf_slots;
    uint32_t aux;
    const float* queries;
    uint32_t dims;
    uint32_t nq;
    const uint32_t* order;  // thread -> query, or null
    const uint32_t* count_dev;
    uint32_t order_base;  // subtracted from order entries (batched orders hold batch-wide ids)  // when set, *count_dev threads are live (nq is an upper bound)
    float max_d2;
    const float* radii;
    uint32_t k;
    int32_t* out_idx;
    float* out_dist;
    DevCounters* counters;
};

// One thread's search: query slot t of the batch (its query is p.order[t] - p.order_base, or t).
template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__device__ __forceinline__ void kd_search_thread(const KdParams& p, uint32_t t, unsigned char* smem) {
    uint64_t* sh_nn = reinterpret_cast<uint64_t*>(smem);
    uint32_t* sh_st = reinterpret_cast<uint32_t*>(smem + tracker_smem_bytes(SHNN, KMAX, blockDim.x));

    const uint32_t qi = p.order ? p.order[t] - p.order_base : t;
    float q[DP];
    load_query<DP>(p.queries, p.dims, qi, q);
    const float r2 = p.radii ? p.radii[qi] : p.max_d2;

    Tracker<KMAX, HEAP, SHNN> tr;
    tr.init(p.k, r2, sh_nn + threadIdx.x, blockDim.x);
    Stack<SHST> st;
    st.init(sh_st, blockDim.x);
    st.push(0, 0.0f);
    LocalCounters lc;
    bool overflow = false;

    while (st.top) {
        uint32_t node;
        float bound;
        st.pop(&node, &bound);
        if (bound > tr.radius()) continue;
        uint32_t depth = heap_depth(node);
        while (depth < p.stop_depth) {
            const uint32_t dim = depth % p.aux;
            const float diff = __fsub_rn(pick<DP>(q, dim), __ldg(p.split + node));
            const uint32_t l = 2 * node + 1;
            const uint32_t close_child = diff < 0.0f ? l : l + 1;
            const uint32_t far_child = diff < 0.0f ? l + 1 : l;
            const float b = __fmul_rn(diff, diff);
            if (b <= tr.radius()) overflow |= !st.push(far_child, b);
            node = close_child;
            ++depth;
            ++lc.nodes;
        }
        const SlotRange r = subtree_slots(node, depth, p.node_depth, p.node_count, p.leaf_slots);
        const float* slot = p.leaf + r.first * p.leaf_stride;
        ++lc.leaves;
        for (uint32_t s = 0; s < r.count; ++s, slot += p.leaf_stride) {
            int32_t id;
            const float d2 = slot_dist<DP>(q, slot, &id);
            if (id < 0) continue;  // padding of a partly filled leaf
            ++lc.points;
            tr.offer(make_key(d2, id));
        }
    }
    tr.emit(p.k, p.out_idx + static_cast<size_t>(qi) * p.k, p.out_dist + static_cast<size_t>(qi) * p.k);
    if (p.counters) {
        lc.flush(p.counters);
        if (overflow) atomicExch(&p.counters->error, 1);
    }
}

template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__global__ void __launch_bounds__(256) kd_knn_kernel(const KdParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (p.count_dev ? *p.count_dev : p.nq)) return;  // no block-wide barriers below
    kd_search_thread<DP, KMAX, HEAP, SHNN, SHST>(p, t, smem);
}

// Warp-coherent variant: the 32 queries of a warp (neighbours after the leaf-order sort) walk the
// tree together.  Each node's split is one broadcast load; the warp descends first into the
// child most of its still-interested lanes are closer to; every lane keeps its own lower bound
// for each stacked subtree, max(bound inherited from the parent, its squared distance to the
// plane), and a subtree is skipped only when no lane's bound is within that lane's radius.
// Leaf buckets are scanned by all lanes against the same slots (broadcast loads).  Control flow
// is uniform across the warp; only the (rare) top-k insertions diverge.
// One warp's search over slots t (this lane) of the batch; `live` slots exist.
template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__device__ __forceinline__ void kd_search_warp(const KdParams& p, uint32_t t, uint32_t live, unsigned char* smem) {
    const uint32_t warp_first = t & ~31u;
    if (warp_first >= live) return;  // whole warp idle; no block-wide barriers below
    const bool active = t < live;
    uint64_t* sh_nn = reinterpret_cast<uint64_t*>(smem);
    uint32_t* sh_st = reinterpret_cast<uint32_t*>(smem + tracker_smem_bytes(SHNN, KMAX, blockDim.x));

    const uint32_t qi = active ? (p.order ? p.order[t] - p.order_base : t) : 0u;
    float q[DP];
    load_query<DP>(p.queries, p.dims, qi, q);
    // Idle lanes (past the end of the batch) search with radius -1: they never want a node.
    const float r2 = active ? (p.radii ? p.radii[qi] : p.max_d2) : 0.0f;

    Tracker<KMAX, HEAP, SHNN> tr;
    tr.init(p.k, r2, sh_nn + threadIdx.x, blockDim.x);
    Stack<SHST> st;
    st.init(sh_st, blockDim.x);
    st.push(0, active ? 0.0f : INFINITY);
    LocalCounters lc;
    bool overflow = false;

    while (st.top) {  // st.top is warp-uniform: every lane pushes and pops together
        uint32_t node;
        float bound;
        st.pop(&node, &bound);
        if (!__any_sync(0xFFFFFFFFu, bound <= tr.radius())) continue;
        uint32_t depth = heap_depth(node);
        bool pruned = false;
        while (depth < p.stop_depth) {
            const uint32_t dim = depth % p.aux;
            const float diff = __fsub_rn(pick<DP>(q, dim), __ldg(p.split + node));
            const float b = fmaxf(bound, __fmul_rn(diff, diff));
            const bool want = bound <= tr.radius();
            const bool go_left = diff < 0.0f;
            const uint32_t left_votes = __popc(__ballot_sync(0xFFFFFFFFu, want && go_left));
            const uint32_t right_votes = __popc(__ballot_sync(0xFFFFFFFFu, want && !go_left));
            const bool first_left = left_votes >= right_votes;
            const uint32_t l = 2 * node + 1;
            // This lane's bound for each child: its inherited bound on its own side, the plane
            // bound on the other.
            const float b_left = go_left ? bound : b;
            const float b_right = go_left ? b : bound;
            const float b_first = first_left ? b_left : b_right;
            const float b_second = first_left ? b_right : b_left;
            ++lc.nodes;
            if (__any_sync(0xFFFFFFFFu, b_second <= tr.radius())) overflow |= !st.push(first_left ? l + 1 : l, b_second);
            node = first_left ? l : l + 1;
            bound = b_first;
            ++depth;
            if (!__any_sync(0xFFFFFFFFu, bound <= tr.radius())) {
                pruned = true;
                break;
            }
        }
        if (pruned) continue;
        const SlotRange r = subtree_slots(node, depth, p.node_depth, p.node_count, p.leaf_slots);
        const float* slot = p.leaf + r.first * p.leaf_stride;
        const bool want = bound <= tr.radius();
        lc.leaves += want ? 1u : 0u;
        for (uint32_t s = 0; s < r.count; ++s, slot += p.leaf_stride) {
            int32_t id;
            const float d2 = slot_dist<DP>(q, slot, &id);
            if (id < 0) continue;
            if (want) {
                ++lc.points;
                tr.offer(make_key(d2, id));
            }
        }
    }
    if (!active) return;
    tr.emit(p.k, p.out_idx + static_cast<size_t>(qi) * p.k, p.out_dist + static_cast<size_t>(qi) * p.k);
    if (p.counters) {
        lc.flush(p.counters);
        if (overflow) atomicExch(&p.counters->error, 1);
    }
}

template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__global__ void __launch_bounds__(256) kd_knn_warp_kernel(const KdParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t live = p.count_dev ? *p.count_dev : p.nq;
    kd_search_warp<DP, KMAX, HEAP, SHNN, SHST>(p, t, live, smem);
}

// Sort key of a query: the node it reaches after `levels` closer-child steps (path bits).
template <int DP>
__global__ void kd_leaf_key_kernel(const float* __restrict__ split, uint32_t aux, uint32_t levels,
                                   const float* __restrict__ queries, uint32_t dims, uint32_t nq,
                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    float q[DP];
    load_query<DP>(queries, dims, t, q);
    uint32_t node = 0;
    for (uint32_t d = 0; d < levels; ++d) {
        const float diff = pick<DP>(q, d % aux) - __ldg(split + node);
        node = 2 * node + (diff < 0.0f ? 1u : 2u);
    }
    keys[t] = node - ((1u << levels) - 1u);
    vals[t] = t;
}

template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
static int launch_kd(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order,
                     cudaStream_t s) {
    const uint32_t block = plan.block ? plan.block : 128;
    const size_t smem = tracker_smem_bytes(SHNN, KMAX, block) + stack_smem_bytes(SHST, block);
    auto kern = plan.warp ? kd_knn_warp_kernel<DP, KMAX, HEAP, SHNN, SHST> : kd_knn_kernel<DP, KMAX, HEAP, SHNN, SHST>;
    if (smem > 48 * 1024)
        KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    KdParams p{};
    p.split = ix->split.as<float>();
    p.leaf = ix->leaf.as<float>();
    p.leaf_stride = ix->leaf_stride;
    p.node_count = ix->node_count;
    p.node_depth = ix->node_depth;
    p.stop_depth = scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan);
    p.leaf_slots = ix->leaf_slots;
    p.aux = ix->aux_dims;
    p.queries = a.queries;
    p.dims = ix->dims;
    p.nq = a.count;
    p.order = order;
    p.count_dev = a.count_dev;
    p.max_d2 = a.max_d2;
    p.radii = a.radii;
    p.k = a.k;
    p.out_idx = a.out_idx;
    p.out_dist = a.out_dist;
    p.counters = a.counters;
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern0, s));
    kern<<<ceil_div(a.count, block), block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern1, s));
    return KNN_OK;
}

template <int DP, int KMAX>
static int launch_kd_variant(knn_index* ix, const QueryArgs& a, const QueryPlan& p, const uint32_t* order,
                             cudaStream_t s) {
#define KNN_KD_CASE(H, N, S)                                            \
    if (p.heap == H && p.sh_nn == N && p.sh_stack == S)                 \
        return launch_kd<DP, KMAX, H, N, S>(ix, a, p, order, s);
    KNN_KD_CASE(false, false, false)
    KNN_KD_CASE(false, false, true)
    KNN_KD_CASE(false, true, false)
    KNN_KD_CASE(false, true, true)
    KNN_KD_CASE(true, false, false)
    KNN_KD_CASE(true, false, true)
    KNN_KD_CASE(true, true, false)
    KNN_KD_CASE(true, true, true)
#undef KNN_KD_CASE
    return fail(KNN_ERR_INVALID_ARGUMENT, "bad query plan");
}

// Query order for locality: queries sorted by the node they reach after up to 24 greedy
// descent steps (stable radix sort on the path bits).  The order lives in the index workspace
// until the next query.
template <uint32_t DP>
int kd_order_dp(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order) {
    *order = nullptr;
    const uint32_t levels = std::min<uint32_t>(ix->node_depth, 24);
    if (levels == 0) return KNN_OK;
    const size_t nq = a.count;
    const size_t need = carve_bytes({nq * 4, nq * 4, nq * 4, nq * 4, radix_sort_temp_bytes(a.count)});
    KNN_TRY(ix->workspace.reserve(need));
    Carver c(ix->workspace.ptr);
    uint32_t* keys = c.take<uint32_t>(nq);
    uint32_t* vals = c.take<uint32_t>(nq);
    uint32_t* keys_alt = c.take<uint32_t>(nq);
    uint32_t* vals_alt = c.take<uint32_t>(nq);
    void* temp = c.take<uint8_t>(radix_sort_temp_bytes(a.count));
    kd_leaf_key_kernel<DP><<<ceil_div(a.count, 256), 256, 0, s>>>(ix->split.as<float>(), ix->aux_dims, levels,
                                                       a.queries, ix->dims, a.count, keys, vals);
    KNN_LAUNCHED();
    bool in_alt = false;
    KNN_TRY(radix_sort_pairs(keys, vals, keys_alt, vals_alt, a.count, static_cast<int>(levels), temp, s, &in_alt));
    *order = in_alt ? vals_alt : vals;
    return KNN_OK;
}

template <uint32_t DP>
int kd_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    const uint32_t* order = a.order;
    if (!order && p.reorder && a.count >= 4096) KNN_TRY(kd_order_dp<DP>(ix, a, s, &order));
    switch (k_class(a.k)) {
        case 8: return launch_kd_variant<DP, 8>(ix, a, p, order, s);
        case 16: return launch_kd_variant<DP, 16>(ix, a, p, order, s);
        case 32: return launch_kd_variant<DP, 32>(ix, a, p, order, s);
        case 64: return launch_kd_variant<DP, 64>(ix, a, p, order, s);
        default: return launch_kd_variant<DP, 128>(ix, a, p, order, s);
    }
}

template int kd_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);
template int kd_order_dp<KNN_DP>(knn_index*, const QueryArgs&, cudaStream_t, const uint32_t**);


// ---- batches of independent sets (one persistent kernel per class of sets) -----------------------
struct KdBatchSet {
    KdParams p;                 // the set's search parameters; p.order is the class order, p.order_base its offset
    uint32_t first_block;  // first work block of this set in the class
    uint32_t query_offset; // first query of this set in the class-wide numbering
    uint32_t levels;       // descent depth of the locality key
};

__device__ __forceinline__ uint32_t kd_find_set(const KdBatchSet* sets, uint32_t nsets, uint32_t item, bool by_query) {
    uint32_t lo = 0, hi = nsets;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if ((by_query ? sets[mid].query_offset : sets[mid].first_block) <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Locality key of every query of the class: (set << 24) | descent path scaled to 24 bits.
template <int DP>
__global__ void kd_batch_key_kernel(const KdBatchSet* __restrict__ sets, uint32_t nsets, uint32_t total,
                                     uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const uint32_t si = kd_find_set(sets, nsets, g, true);
    const KdParams& p = sets[si].p;
    float q[DP];
    load_query<DP>(p.queries, p.dims, g - sets[si].query_offset, q);
    const uint32_t levels = sets[si].levels;
    uint32_t node = 0;
    for (uint32_t d = 0; d < levels; ++d) {
        const float diff = pick<DP>(q, d % p.aux) - __ldg(p.split + node);
        node = 2 * node + (diff < 0.0f ? 1u : 2u);
    }
    keys[g] = (si << 24) | ((node - ((1u << levels) - 1u)) << (24 - levels));
    vals[g] = g;
}

// Persistent kernel: blocks take work blocks (blockDim queries of one set) from a shared counter
// until the class is done; sets of very different sizes share the GPU without a launch each.
template <int DP, int KMAX, bool WARP>
__global__ void __launch_bounds__(256) kd_batch_kernel(const KdBatchSet* __restrict__ sets, uint32_t nsets,
                                                        uint32_t total_blocks, uint32_t* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t item_s;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) item_s = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t item = item_s;
        if (item >= total_blocks) break;
        const uint32_t si = kd_find_set(sets, nsets, item, false);
        const KdParams& p = sets[si].p;
        const uint32_t t = (item - sets[si].first_block) * blockDim.x + threadIdx.x;
        if constexpr (WARP) {
            kd_search_warp<DP, KMAX, false, false, false>(p, t, p.nq, smem);
        } else {
            if (t < p.nq) kd_search_thread<DP, KMAX, false, false, false>(p, t, smem);
        }
    }
}

template <uint32_t DP>
int kd_batch_launch(const void* sets, uint32_t nsets, uint32_t total_queries, uint32_t total_blocks, uint32_t kmax,
                       bool warp, uint32_t block, uint32_t* counter, uint32_t* keys, uint32_t* vals, bool key_pass,
                       cudaStream_t s) {
    using Set = KdBatchSet;
    const Set* d_sets = static_cast<const Set*>(sets);
    if (key_pass) {
        kd_batch_key_kernel<DP><<<ceil_div(total_queries, 256), 256, 0, s>>>(d_sets, nsets, total_queries, keys, vals);
        KNN_LAUNCHED();
        return KNN_OK;
    }
#define KNN_BATCH(KM, W)                                                                              \
    if (kmax == KM && warp == W) {                                                                    \
        auto kern = kd_batch_kernel<DP, KM, W>;                                                    \
        int per_sm = 0;                                                                               \
        KNN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0));         \
        const uint32_t grid = std::max(1, per_sm) * static_cast<uint32_t>(sm_count());                \
        kern<<<std::min(grid, total_blocks), block, 0, s>>>(d_sets, nsets, total_blocks, counter);   \
        KNN_LAUNCHED();                                                                               \
        return KNN_OK;                                                                                \
    }
    KNN_BATCH(8, false) KNN_BATCH(16, false) KNN_BATCH(32, false) KNN_BATCH(64, false) KNN_BATCH(128, false)
    KNN_BATCH(8, true) KNN_BATCH(16, true) KNN_BATCH(32, true) KNN_BATCH(64, true) KNN_BATCH(128, true)
#undef KNN_BATCH
    return fail(KNN_ERR_INVALID_ARGUMENT, "batch class k %u", kmax);
}

#if KNN_DP == 1
// Fills the search parameters of one batch set from its index and item.
size_t kd_batch_set_bytes() { return sizeof(KdBatchSet); }

void kd_batch_set_fill(void* out, const knn_index* ix, const QueryArgs& a, const QueryPlan& plan,
                        const uint32_t* order, uint32_t order_base, uint32_t first_block, uint32_t query_offset) {
    KdBatchSet bs{};
    KdParams& p = bs.p;
    p.split = ix->split.as<float>();
    p.aux = ix->aux_dims;
    p.leaf = ix->leaf.as<float>();
    p.leaf_stride = ix->leaf_stride;
    p.node_count = ix->node_count;
    p.node_depth = ix->node_depth;
    p.stop_depth = scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan);
    p.leaf_slots = ix->leaf_slots;
    p.queries = a.queries;
    p.dims = ix->dims;
    p.nq = a.count;
    p.order = order;
    p.order_base = order_base;
    p.max_d2 = a.max_d2;
    p.k = a.k;
    p.out_idx = a.out_idx;
    p.out_dist = a.out_dist;
    bs.first_block = first_block;
    bs.query_offset = query_offset;
    bs.levels = std::min<uint32_t>(ix->node_depth, 24);
    std::memcpy(out, &bs, sizeof(bs));
}
#endif

template int kd_batch_launch<KNN_DP>(const void*, uint32_t, uint32_t, uint32_t, uint32_t, bool, uint32_t, uint32_t*,
                                      uint32_t*, uint32_t*, bool, cudaStream_t);

}  // namespace knn
