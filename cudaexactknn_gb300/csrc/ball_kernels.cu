// Ball tree query kernels, one translation unit per padded dimension count (KNN_DP).
//
// Replaces BallTreeKernels::knnDevice and its four storage variants (src/BallTreeGpu.cuh:36-200).
// Same depth-first search: at each internal node measure the query's distance to both child
// balls, descend into the closer one, push the farther one when it can still hold a neighbour,
// stop the descent when even the closer ball is out of range (src/BallTreeGpu.cuh:82-92).
// The reference's border distance sqrt(d2) - r (with -use_fast_math's approximate sqrt) can
// round above a point's own float distance and prune a true neighbour; here knn::ball_bound
// uses directed rounding and relative margins so it never exceeds the float dist2 of any point
// in the ball, and a ball is pruned only when its bound > the k-th distance.

#include <algorithm>
#include <cstring>

#include "tree_query.cuh"

#ifndef KNN_DP
#error "compile with -DKNN_DP=<padded dims>"
#endif

namespace knn {

struct BallParams {
    const float* ball;     // node i: centre (DP floats), radius at [DP]
    uint32_t ball_stride;
    const float* leaf;
    uint32_t leaf_stride;
    uint32_t node_count;
    uint32_t node_depth;
    uint32_t stop_depth;
    uint32_t leaf_slots;
    float margin;
    const float* queries;
    uint32_t dims;
    uint32_t nq;
    const uint32_t* order;
    const uint32_t* count_dev;
    uint32_t order_base;  // subtracted from order entries (batched orders hold batch-wide ids)
    float max_d2;
    const float* radii;
    uint32_t k;
    int32_t* out_idx;
    float* out_dist;
    DevCounters* counters;
};

// Float dist2 from q to a ball's centre; the radius comes back through *r.
template <int DP>
__device__ __forceinline__ float centre_dist(const float (&q)[DP], const float* __restrict__ b, float* r) {
    if constexpr (DP < 4) {
        const float4 v = *reinterpret_cast<const float4*>(b);
        const float w[4] = {v.x, v.y, v.z, v.w};
        *r = w[DP];
        float acc = 0.0f;
#pragma unroll
        for (int d = 0; d < DP; ++d) {
            const float t = __fsub_rn(q[d], w[d]);
            acc = __fmaf_rn(t, t, acc);
        }
        return acc;
    } else {
        *r = b[DP];
        return dist2_vec4<DP>(q, reinterpret_cast<const float4*>(b));
    }
}

// One thread's search: query slot t of the batch (its query is p.order[t] - p.order_base, or t).
template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__device__ __forceinline__ void ball_search_thread(const BallParams& p, uint32_t t, unsigned char* smem) {
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
        bool pruned = false;
        uint32_t depth = heap_depth(node);
        while (depth < p.stop_depth) {
            const uint32_t l = 2 * node + 1;
            float rl, rr;
            const float sl = centre_dist<DP>(q, p.ball + static_cast<size_t>(l) * p.ball_stride, &rl);
            const float sr = centre_dist<DP>(q, p.ball + static_cast<size_t>(l + 1) * p.ball_stride, &rr);
            const float bl = ball_bound(sl, rl, p.margin);
            const float br = ball_bound(sr, rr, p.margin);
            ++lc.nodes;
            // Visit order only (not a bound): the nearer border first.
            const bool left_first = sqrtf(sl) - rl < sqrtf(sr) - rr;
            const uint32_t close_child = left_first ? l : l + 1;
            const float close_b = left_first ? bl : br;
            const float far_b = left_first ? br : bl;
            if (close_b > tr.radius()) {
                // The farther ball's bound is at least as large in the common case, but the
                // order above is approximate, so it is checked on its own.
                if (far_b <= tr.radius()) {
                    node = left_first ? l + 1 : l;
                    ++depth;
                    continue;
                }
                pruned = true;
                break;
            }
            if (far_b <= tr.radius()) overflow |= !st.push(left_first ? l + 1 : l, far_b);
            node = close_child;
            ++depth;
        }
        if (pruned) continue;
        const SlotRange r = subtree_slots(node, depth, p.node_depth, p.node_count, p.leaf_slots);
        const float* slot = p.leaf + r.first * p.leaf_stride;
        ++lc.leaves;
        for (uint32_t s = 0; s < r.count; ++s, slot += p.leaf_stride) {
            int32_t id;
            const float d2 = slot_dist<DP>(q, slot, &id);
            if (id < 0) continue;
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
__global__ void __launch_bounds__(256) ball_knn_kernel(const BallParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (p.count_dev ? *p.count_dev : p.nq)) return;  // no block-wide barriers below
    ball_search_thread<DP, KMAX, HEAP, SHNN, SHST>(p, t, smem);
}

// Warp-coherent variant (see kd_knn_warp_kernel): the warp's queries walk the tree together,
// descending first into the child most still-interested lanes are closer to; each lane's bound
// for a child is max(its inherited bound, its rigorous bound to the child's ball).
// One warp's search over slots t (this lane) of the batch; `live` slots exist.
template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
__device__ __forceinline__ void ball_search_warp(const BallParams& p, uint32_t t, uint32_t live, unsigned char* smem) {
    if ((t & ~31u) >= live) return;
    const bool active = t < live;
    uint64_t* sh_nn = reinterpret_cast<uint64_t*>(smem);
    uint32_t* sh_st = reinterpret_cast<uint32_t*>(smem + tracker_smem_bytes(SHNN, KMAX, blockDim.x));

    const uint32_t qi = active ? (p.order ? p.order[t] - p.order_base : t) : 0u;
    float q[DP];
    load_query<DP>(p.queries, p.dims, qi, q);
    const float r2 = active ? (p.radii ? p.radii[qi] : p.max_d2) : 0.0f;

    Tracker<KMAX, HEAP, SHNN> tr;
    tr.init(p.k, r2, sh_nn + threadIdx.x, blockDim.x);
    Stack<SHST> st;
    st.init(sh_st, blockDim.x);
    st.push(0, active ? 0.0f : INFINITY);
    LocalCounters lc;
    bool overflow = false;

    while (st.top) {
        uint32_t node;
        float bound;
        st.pop(&node, &bound);
        if (!__any_sync(0xFFFFFFFFu, bound <= tr.radius())) continue;
        uint32_t depth = heap_depth(node);
        bool pruned = false;
        while (depth < p.stop_depth) {
            const uint32_t l = 2 * node + 1;
            float rl, rr;
            const float sl = centre_dist<DP>(q, p.ball + static_cast<size_t>(l) * p.ball_stride, &rl);
            const float sr = centre_dist<DP>(q, p.ball + static_cast<size_t>(l + 1) * p.ball_stride, &rr);
            const float bl = fmaxf(bound, ball_bound(sl, rl, p.margin));
            const float br = fmaxf(bound, ball_bound(sr, rr, p.margin));
            const bool want = bound <= tr.radius();
            const bool left_near = sqrtf(sl) - rl < sqrtf(sr) - rr;
            const uint32_t left_votes = __popc(__ballot_sync(0xFFFFFFFFu, want && left_near));
            const uint32_t right_votes = __popc(__ballot_sync(0xFFFFFFFFu, want && !left_near));
            const bool first_left = left_votes >= right_votes;
            const float b_first = first_left ? bl : br;
            const float b_second = first_left ? br : bl;
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
__global__ void __launch_bounds__(256) ball_knn_warp_kernel(const BallParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t live = p.count_dev ? *p.count_dev : p.nq;
    ball_search_warp<DP, KMAX, HEAP, SHNN, SHST>(p, t, live, smem);
}

// Sort key of a query: the node reached after `levels` steps towards the nearer child centre.
template <int DP>
__global__ void ball_leaf_key_kernel(const float* __restrict__ ball, uint32_t ball_stride, uint32_t levels,
                                     const float* __restrict__ queries, uint32_t dims, uint32_t nq,
                                     uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    float q[DP];
    load_query<DP>(queries, dims, t, q);
    uint32_t node = 0;
    for (uint32_t d = 0; d < levels; ++d) {
        const uint32_t l = 2 * node + 1;
        float rl, rr;
        const float sl = centre_dist<DP>(q, ball + static_cast<size_t>(l) * ball_stride, &rl);
        const float sr = centre_dist<DP>(q, ball + static_cast<size_t>(l + 1) * ball_stride, &rr);
        node = sl <= sr ? l : l + 1;
    }
    keys[t] = node - ((1u << levels) - 1u);
    vals[t] = t;
}

template <int DP, int KMAX, bool HEAP, bool SHNN, bool SHST>
static int launch_ball(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order,
                       cudaStream_t s) {
    const uint32_t block = plan.block ? plan.block : 128;
    const size_t smem = tracker_smem_bytes(SHNN, KMAX, block) + stack_smem_bytes(SHST, block);
    auto kern = plan.warp ? ball_knn_warp_kernel<DP, KMAX, HEAP, SHNN, SHST> : ball_knn_kernel<DP, KMAX, HEAP, SHNN, SHST>;
    if (smem > 48 * 1024)
        KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    BallParams p{};
    p.ball = ix->ball.as<float>();
    p.ball_stride = ix->ball_stride;
    p.leaf = ix->leaf.as<float>();
    p.leaf_stride = ix->leaf_stride;
    p.node_count = ix->node_count;
    p.node_depth = ix->node_depth;
    p.stop_depth = scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan);
    p.leaf_slots = ix->leaf_slots;
    p.margin = rel_margin(ix->dims);
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
    if (plan.timing) KNN_TRY(ix->timing.begin(s));
    kern<<<ceil_div(a.count, block), block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY(ix->timing.end(s));
    return KNN_OK;
}

template <int DP, int KMAX>
static int launch_ball_variant(knn_index* ix, const QueryArgs& a, const QueryPlan& p, const uint32_t* order,
                               cudaStream_t s) {
#define KNN_BALL_CASE(H, N, S)                                          \
    if (p.heap == H && p.sh_nn == N && p.sh_stack == S)                 \
        return launch_ball<DP, KMAX, H, N, S>(ix, a, p, order, s);
    KNN_BALL_CASE(false, false, false)
    KNN_BALL_CASE(false, false, true)
    KNN_BALL_CASE(false, true, false)
    KNN_BALL_CASE(false, true, true)
    KNN_BALL_CASE(true, false, false)
    KNN_BALL_CASE(true, false, true)
    KNN_BALL_CASE(true, true, false)
    KNN_BALL_CASE(true, true, true)
#undef KNN_BALL_CASE
    return fail(KNN_ERR_INVALID_ARGUMENT, "bad query plan");
}

// Query order for locality: queries sorted by the node they reach after up to 24 greedy
// descent steps (stable radix sort on the path bits).  The order lives in the index workspace
// until the next query.
template <uint32_t DP>
int ball_order_dp(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order) {
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
    ball_leaf_key_kernel<DP><<<ceil_div(a.count, 256), 256, 0, s>>>(ix->ball.as<float>(), ix->ball_stride, levels,
                                                       a.queries, ix->dims, a.count, keys, vals);
    KNN_LAUNCHED();
    bool in_alt = false;
    KNN_TRY(radix_sort_pairs(keys, vals, keys_alt, vals_alt, a.count, static_cast<int>(levels), temp, s, &in_alt));
    *order = in_alt ? vals_alt : vals;
    return KNN_OK;
}

template <uint32_t DP>
int ball_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    const uint32_t* order = a.order;
    if (!order && p.reorder && a.count >= 4096) KNN_TRY(ball_order_dp<DP>(ix, a, s, &order));
    switch (k_class(a.k)) {
        case 8: return launch_ball_variant<DP, 8>(ix, a, p, order, s);
        case 16: return launch_ball_variant<DP, 16>(ix, a, p, order, s);
        case 32: return launch_ball_variant<DP, 32>(ix, a, p, order, s);
        case 64: return launch_ball_variant<DP, 64>(ix, a, p, order, s);
        default: return launch_ball_variant<DP, 128>(ix, a, p, order, s);
    }
}

template int ball_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);
template int ball_order_dp<KNN_DP>(knn_index*, const QueryArgs&, cudaStream_t, const uint32_t**);


// ---- batches of independent sets (one persistent kernel per class of sets) -----------------------
struct BallBatchSet {
    BallParams p;                 // the set's search parameters; p.order is the class order, p.order_base its offset
    uint32_t first_block;  // first work block of this set in the class
    uint32_t query_offset; // first query of this set in the class-wide numbering
    uint32_t levels;       // descent depth of the locality key
};

__device__ __forceinline__ uint32_t ball_find_set(const BallBatchSet* sets, uint32_t nsets, uint32_t item, bool by_query) {
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
__global__ void ball_batch_key_kernel(const BallBatchSet* __restrict__ sets, uint32_t nsets, uint32_t total,
                                     uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const uint32_t si = ball_find_set(sets, nsets, g, true);
    const BallParams& p = sets[si].p;
    float q[DP];
    load_query<DP>(p.queries, p.dims, g - sets[si].query_offset, q);
    const uint32_t levels = sets[si].levels;
    uint32_t node = 0;
    for (uint32_t d = 0; d < levels; ++d) {
        const uint32_t l = 2 * node + 1;
        float rl, rr;
        const float sl = centre_dist<DP>(q, p.ball + static_cast<size_t>(l) * p.ball_stride, &rl);
        const float sr = centre_dist<DP>(q, p.ball + static_cast<size_t>(l + 1) * p.ball_stride, &rr);
        node = sl <= sr ? l : l + 1;
    }
    keys[g] = (si << 24) | ((node - ((1u << levels) - 1u)) << (24 - levels));
    vals[g] = g;
}

// Persistent kernel: blocks take work blocks (blockDim queries of one set) from a shared counter
// until the class is done; sets of very different sizes share the GPU without a launch each.
template <int DP, int KMAX, bool WARP>
__global__ void __launch_bounds__(256) ball_batch_kernel(const BallBatchSet* __restrict__ sets, uint32_t nsets,
                                                        uint32_t total_blocks, uint32_t* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t item_s;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) item_s = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t item = item_s;
        if (item >= total_blocks) break;
        const uint32_t si = ball_find_set(sets, nsets, item, false);
        const BallParams& p = sets[si].p;
        const uint32_t t = (item - sets[si].first_block) * blockDim.x + threadIdx.x;
        if constexpr (WARP) {
            ball_search_warp<DP, KMAX, false, false, false>(p, t, p.nq, smem);
        } else {
            if (t < p.nq) ball_search_thread<DP, KMAX, false, false, false>(p, t, smem);
        }
    }
}

template <uint32_t DP>
int ball_batch_launch(const void* sets, uint32_t nsets, uint32_t total_queries, uint32_t total_blocks, uint32_t kmax,
                       bool warp, uint32_t block, uint32_t* counter, uint32_t* keys, uint32_t* vals, bool key_pass,
                       cudaStream_t s) {
    using Set = BallBatchSet;
    const Set* d_sets = static_cast<const Set*>(sets);
    if (key_pass) {
        ball_batch_key_kernel<DP><<<ceil_div(total_queries, 256), 256, 0, s>>>(d_sets, nsets, total_queries, keys, vals);
        KNN_LAUNCHED();
        return KNN_OK;
    }
#define KNN_BATCH(KM, W)                                                                              \
    if (kmax == KM && warp == W) {                                                                    \
        auto kern = ball_batch_kernel<DP, KM, W>;                                                    \
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
size_t ball_batch_set_bytes() { return sizeof(BallBatchSet); }

void ball_batch_set_fill(void* out, const knn_index* ix, const QueryArgs& a, const QueryPlan& plan,
                        const uint32_t* order, uint32_t order_base, uint32_t first_block, uint32_t query_offset) {
    BallBatchSet bs{};
    BallParams& p = bs.p;
    p.ball = ix->ball.as<float>();
    p.ball_stride = ix->ball_stride;
    p.margin = rel_margin(ix->dims);
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

template int ball_batch_launch<KNN_DP>(const void*, uint32_t, uint32_t, uint32_t, uint32_t, bool, uint32_t, uint32_t*,
                                      uint32_t*, uint32_t*, bool, cudaStream_t);

}  // namespace knn
