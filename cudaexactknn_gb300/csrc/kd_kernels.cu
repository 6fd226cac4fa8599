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
    if (plan.timing) KNN_TRY(ix->timing.begin(s));
    kern<<<ceil_div(a.count, block), block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY(ix->timing.end(s));
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
int kd_order_dp(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order, uint32_t max_levels) {
    *order = nullptr;
    const uint32_t levels = std::min<uint32_t>(ix->node_depth, std::min<uint32_t>(max_levels, 24));
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
int kd_group_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order,
                      float* seeds, uint32_t* fb_list, uint32_t* fb_count, float seed_scale, cudaStream_t s);

template <uint32_t DP>
int kd_box_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order, cudaStream_t s);

template <uint32_t DP>
int kd_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    const uint32_t* order = a.order;
    if (!order && p.reorder && a.count >= 4096) KNN_TRY(kd_order_dp<DP>(ix, a, s, &order, 24));
    if (p.group && !a.count_dev) return kd_group_query_dp<DP>(ix, a, p, order, nullptr, nullptr, nullptr, 1.0f, s);
    if (p.box) return kd_box_query_dp<DP>(ix, a, p, order, s);
    switch (k_class(a.k)) {
        case 8: return launch_kd_variant<DP, 8>(ix, a, p, order, s);
        case 16: return launch_kd_variant<DP, 16>(ix, a, p, order, s);
        case 32: return launch_kd_variant<DP, 32>(ix, a, p, order, s);
        case 64: return launch_kd_variant<DP, 64>(ix, a, p, order, s);
        default: return launch_kd_variant<DP, 128>(ix, a, p, order, s);
    }
}

// ---- warp-group search ---------------------------------------------------------------------------
//
// The 32 lanes of a warp hold 32 neighbouring queries (locality order) and a radius each (a seed
// from the radius model or from the query's own subtree, never below its k-th distance for most
// queries).  The warp walks the tree once for all of them, bounding every node by the distance
// from each lane's query to the node's tight bounding box; a node is entered when some lane's
// bound is within that lane's radius.  Leaf buckets are collected as (bucket, lanes) entries,
// and the (bucket, query) pairs are then dealt out over the warp's lanes one pair per lane, so a
// warp does the sum of its queries' bucket scans rather than their union.  A point within its
// query's radius is appended to that query's candidate list in shared memory; at the end each
// lane sorts its query's list.  A query with fewer than k candidates inside a radius below the
// caller's grows its radius by the density it saw and walks again; one whose list overflows, or
// that is still short after a few rounds, goes to a list that the box-bounded per-thread search
// answers.  Every
// answer is exact: a bucket is skipped only when its box bound exceeds the radius, and the box
// bound is a rigorous lower bound on the float distance of every point inside (below).
constexpr uint32_t kGroupWarps = 4;
constexpr uint32_t kGroupList = 64;   // bucket entries collected before they are scanned
constexpr uint32_t kGroupFan = 3;     // levels the walk descends per step (up to 8 boxes tested at once)
constexpr uint32_t kGroupStack = 96;  // node stack (at most 7 net entries per step, 11 steps deep)
constexpr uint32_t kGroupRounds = 6;  // radius growth rounds before the per-thread fallback

__host__ __device__ constexpr uint32_t group_cap(int kmax) { return kmax <= 8 ? 32u : (kmax <= 16 ? 48u : 80u); }
__host__ __device__ constexpr int box_qs(int dp) { return dp < 4 ? 4 : dp; }

template <int DP, int KMAX>
struct GroupWarpSmem {
    uint32_t buf[group_cap(KMAX)][32];  // candidates' leaf slots, slot-major (entry i of lane l at [i][l])
    uint64_t list[kGroupList];          // (bucket node << 32) | lanes
    float qv[32][box_qs(DP)];           // the warp's queries
    float rad[32];                      // radius of each lane this round (-1: none)
    uint32_t cnt[32];                   // candidates appended per lane
    uint32_t pre[32];                   // inclusive prefix of pairs per list entry
    uint32_t stack[kGroupStack];
};

template <int DP, int KMAX>
constexpr size_t group_smem_bytes() { return kGroupWarps * sizeof(GroupWarpSmem<DP, KMAX>); }

struct KdGroupParams {
    KdParams p;              // tree, queries, locality order, caller's radius (max_d2 / radii), outputs
    const float* box;        // per node (depth <= box depth): lo[box_qs(DP)], hi[box_qs(DP)]
    float* seeds;            // per query radius to start from (<= the caller's); fallback radius on exit
    uint32_t* fb_list;       // queries left to the per-thread search
    uint32_t* fb_count;
    uint32_t* group_counter; // next group of 32 queries (zero before the launch)
    uint32_t box_stride;     // floats per box
    float seed_scale;        // seeds are multiplied by this (capped by the caller's radius)
};

// Lower bound on the float dist2 from q to any point of the box (lo, hi): per dimension the gap
// o = max(fl(lo - q), fl(q - hi), 0), then the same fused sum as dist2 in dimension order.  For a
// point p of the box, |fl(q - p)| >= o (p lies beyond lo or hi, and rounding is monotone), and
// fma(t, t, acc) is non-decreasing in |t| and acc >= 0, so the bound never exceeds dist2(q, p).
// An empty box (lo = +inf, hi = -inf) gives +inf.
template <int DP>
__device__ __forceinline__ float box_bound(const float (&q)[DP], const float* __restrict__ box) {
    constexpr int QS = box_qs(DP);
    const float4* lo4 = reinterpret_cast<const float4*>(box);
    const float4* hi4 = reinterpret_cast<const float4*>(box + QS);
    float acc = 0.0f;
#pragma unroll
    for (int v = 0; v < (DP + 3) / 4; ++v) {
        const float4 lo = __ldg(lo4 + v), hi = __ldg(hi4 + v);
        const float l[4] = {lo.x, lo.y, lo.z, lo.w};
        const float h[4] = {hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (4 * v + c < DP) {
                const float o = fmaxf(fmaxf(__fsub_rn(l[c], q[4 * v + c]), __fsub_rn(q[4 * v + c], h[c])), 0.0f);
                acc = __fmaf_rn(o, o, acc);
            }
        }
    }
    return acc;
}

template <int DP, int KMAX>
__global__ void __launch_bounds__(kGroupWarps * 32) kd_group_kernel(const KdGroupParams gp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Sm = GroupWarpSmem<DP, KMAX>;
    constexpr uint32_t C = group_cap(KMAX);
    constexpr int QS = box_qs(DP);
    constexpr uint32_t FULL = 0xFFFFFFFFu;
    Sm& sm = reinterpret_cast<Sm*>(smem_raw)[threadIdx.x >> 5];
    const KdParams& p = gp.p;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stop = p.stop_depth;
    const uint32_t bucket_slots = p.leaf_slots << (p.node_depth - stop);
    uint32_t nodes = 0, pairs = 0;
    bool stack_error = false;
    // Persistent warps: each takes the next group of 32 queries from a counter until the batch is
    // done, so that no partial last wave of blocks is left and regions of uneven cost balance.
    for (;;) {
        uint32_t grp = 0;
        if (lane == 0) grp = atomicAdd(gp.group_counter, 1u);
        const uint32_t g = __shfl_sync(FULL, grp, 0) * 32u;
        if (g >= p.nq) break;
        const uint32_t t = g + lane;
        const bool active = t < p.nq;
        const uint32_t qi = active ? (p.order ? p.order[t] : t) : 0u;
        float q[DP];
        load_query<DP>(p.queries, p.dims, qi, q);
#pragma unroll
        for (int d = 0; d < QS; ++d) sm.qv[lane][d] = d < DP ? q[d] : 0.0f;
        const float R = active ? (p.radii ? p.radii[qi] : p.max_d2) : -1.0f;
        float r = active ? gp.seeds[qi] * gp.seed_scale : -1.0f;
        if (!(r <= R)) r = R;  // a seed above the caller's radius (or NaN) starts at the caller's
        bool pending = active;

        // Scans the collected (bucket, lanes) entries, one (bucket, query) pair per lane at a time.
        auto scan = [&](uint32_t n) {
            for (uint32_t base = 0; base < n; base += 32) {
                const uint32_t e = base + lane;
                const uint32_t m = e < n ? static_cast<uint32_t>(sm.list[e]) : 0u;
                uint32_t incl = __popc(m);
#pragma unroll
                for (uint32_t o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += v;
                }
                const uint32_t total = __shfl_sync(FULL, incl, 31);
                sm.pre[lane] = incl;
                __syncwarp();
                for (uint32_t it = lane; it < total; it += 32) {
                    uint32_t j = 0;  // first entry whose inclusive prefix exceeds it
#pragma unroll
                    for (uint32_t step = 16; step; step >>= 1)
                        if (sm.pre[j + step - 1] <= it) j += step;
                    const uint64_t ent = sm.list[base + j];
                    const uint32_t excl = j ? sm.pre[j - 1] : 0u;
                    const uint32_t ql = nth_set_bit(static_cast<uint32_t>(ent), it - excl);
                    float qq[DP];
#pragma unroll
                    for (int d = 0; d < DP; ++d) qq[d] = sm.qv[ql][d];
                    const float rq = sm.rad[ql];
                    const uint32_t bucket = static_cast<uint32_t>(ent >> 32);
                    if (heap_depth(bucket) != stop) {  // cannot happen (the walk lists buckets only); recorded
                        stack_error = true;
                        continue;
                    }
                    const SlotRange sr = subtree_slots(bucket, stop, p.node_depth, p.node_count, p.leaf_slots);
                    const float* slot = p.leaf + sr.first * p.leaf_stride;
#pragma unroll 4
                    for (uint32_t s = 0; s < bucket_slots; ++s, slot += p.leaf_stride) {
                        int32_t id;
                        const float d2 = slot_dist<DP>(qq, slot, &id);
                        if (id >= 0 && d2 <= rq) {
                            // The slot is kept, not the key: half the shared memory, and the owner lane
                            // recomputes the same distance from it when it sorts its list.
                            const uint32_t pos = atomicAdd(&sm.cnt[ql], 1u);
                            if (pos < C) sm.buf[pos][ql] = static_cast<uint32_t>(sr.first) + s;
                        }
                    }
                    ++pairs;
                }
                __syncwarp();
            }
        };

        for (uint32_t round = 0; __any_sync(FULL, pending); ++round) {
            const float rl = pending ? r : -1.0f;
            sm.cnt[lane] = 0;
            sm.rad[lane] = rl;
            __syncwarp();
            uint32_t top = 0, nlist = 0;
            const uint32_t m0 = __ballot_sync(FULL, box_bound<DP>(q, gp.box) <= rl);
            if (m0) {
                if (stop == 0) {
                    if (lane == 0) sm.list[0] = m0;
                    nlist = 1;
                } else {
                    if (lane == 0) sm.stack[0] = 0;
                    top = 1;
                }
            }
            while (top) {
                __syncwarp();
                const uint32_t node = sm.stack[--top];
                // The node's descendants `levels` below (up to 8, contiguous in the heap order) are
                // tested at once: their box loads are independent, so they overlap in flight.
                const uint32_t levels = min(kGroupFan, stop - heap_depth(node));
                const uint32_t fan = 1u << levels;
                const uint32_t first = ((node + 1) << levels) - 1;
                uint32_t want[1u << kGroupFan];
#pragma unroll
                for (uint32_t j = 0; j < (1u << kGroupFan); ++j) {
                    // (j < fan first: with an unbounded radius an infinite bound is still "within".)
                    const bool in = j < fan && box_bound<DP>(q, gp.box + static_cast<size_t>(first + j) * gp.box_stride) <= rl;
                    want[j] = __ballot_sync(FULL, in);
                }
                ++nodes;
                if (heap_depth(node) + levels == stop) {
#pragma unroll
                    for (uint32_t j = 0; j < (1u << kGroupFan); ++j) {
                        if (want[j]) {
                            if (lane == 0) sm.list[nlist] = (static_cast<uint64_t>(first + j) << 32) | want[j];
                            ++nlist;
                        }
                    }
                    if (nlist + (1u << kGroupFan) > kGroupList) {
                        __syncwarp();
                        scan(nlist);
                        nlist = 0;
                    }
                } else {
                    if (top + (1u << kGroupFan) > kGroupStack) {  // cannot happen (see kGroupStack); recorded
                        stack_error = true;
                        continue;
                    }
#pragma unroll
                    for (uint32_t j = (1u << kGroupFan); j-- > 0;) {
                        if (want[j]) {
                            if (lane == 0) sm.stack[top] = first + j;
                            ++top;
                        }
                    }
                }
            }
            if (nlist) {
                __syncwarp();
                scan(nlist);
            }
            __syncwarp();
            if (pending) {
                const uint32_t c = sm.cnt[lane];
                // The k smallest keys among the first n listed candidates (their distances
                // recomputed from the slots, four loads in flight).
                auto select = [&](Tracker<KMAX, false, false>& tr, uint32_t n) {
                    uint32_t i = 0;
                    for (; i + 4 <= n; i += 4) {
                        int32_t id[4];
                        float d2[4];
#pragma unroll
                        for (uint32_t u = 0; u < 4; ++u)
                            d2[u] = slot_dist<DP>(q, p.leaf + static_cast<size_t>(sm.buf[i + u][lane]) * p.leaf_stride, &id[u]);
#pragma unroll
                        for (uint32_t u = 0; u < 4; ++u) tr.offer(make_key(d2[u], id[u]));
                    }
                    for (; i < n; ++i) {
                        int32_t id;
                        const float d2 = slot_dist<DP>(q, p.leaf + static_cast<size_t>(sm.buf[i][lane]) * p.leaf_stride, &id);
                        tr.offer(make_key(d2, id));
                    }
                };
                if (c > C) {
                    // More candidates than the list holds.  The k-th smallest distance among the C
                    // kept bounds the k-th neighbour's (k real points lie within it): the
                    // per-thread search starts from it.  (Walking again with a radius shrunk by the
                    // density was tried: the extra rounds cost more than the searches they save.)
                    Tracker<KMAX, false, false> tr;
                    tr.init(p.k, r, nullptr, 0);
                    select(tr, C);
                    const uint32_t pos = atomicAdd(gp.fb_count, 1u);
                    gp.fb_list[pos] = qi;
                    gp.seeds[qi] = fminf(tr.radius(), r);
                    if (p.counters) atomicAdd(&p.counters->fallback, 1ull);
                    pending = false;
                } else if (c >= p.k || !(r < R)) {
                    Tracker<KMAX, false, false> tr;
                    tr.init(p.k, R, nullptr, 0);
                    select(tr, c);
                    tr.emit(p.k, p.out_idx + static_cast<size_t>(qi) * p.k, p.out_dist + static_cast<size_t>(qi) * p.k);
                    pending = false;
                } else if (round + 1 >= kGroupRounds) {
                    const uint32_t pos = atomicAdd(gp.fb_count, 1u);
                    gp.fb_list[pos] = qi;
                    gp.seeds[qi] = R;
                    if (p.counters) atomicAdd(&p.counters->fallback, 1ull);
                    pending = false;
                } else {
                    // Fewer than k within r: grow r^2 by the volume ratio k points need at the density
                    // seen, (1.5 k / c)^(2 / dims), between 1.25 and 16.
                    const float ce = fmaxf(static_cast<float>(c), 0.5f);
                    const float grow = fminf(fmaxf(exp2f(log2f(1.5f * static_cast<float>(p.k) / ce) * (2.0f / p.dims)),
                                                   1.25f), 16.0f);
                    r = fminf(R, fmaxf(r * grow, 1e-30f));
                }
            }
            __syncwarp();
        }
    }
    if (p.counters) {
        // nodes: walk steps (each tests up to 8 descendants); leaves: (bucket, query) pairs.
        if (lane == 0) {
            atomicAdd(&p.counters->nodes, static_cast<unsigned long long>(nodes));
            if (stack_error) atomicExch(&p.counters->error, 1);
        }
        if (pairs) {
            atomicAdd(&p.counters->leaves, static_cast<unsigned long long>(pairs));
            atomicAdd(&p.counters->points, static_cast<unsigned long long>(pairs) * bucket_slots);
        }
    }
}

// Per-thread search over the tight node boxes (traversal 3, and the group search's leftovers):
// depth first, the closer child first, a node skipped when its box bound exceeds the current k-th
// distance, buckets at depth `stop` scanned whole; from radius r2, results to the query's row.
// Box bounds matter most far from the data, where a single splitting plane prunes little.
template <int DP, int KMAX>
__device__ __forceinline__ void kd_box_search(const KdParams& p, const float* __restrict__ box, uint32_t box_stride,
                                              uint32_t stop, uint32_t qi, float r2) {
    float q[DP];
    load_query<DP>(p.queries, p.dims, qi, q);
    Tracker<KMAX, false, false> tr;
    tr.init(p.k, r2, nullptr, 0);
    Stack<false> st;
    st.init(nullptr, 0);
    st.push(0, box_bound<DP>(q, box));
    bool overflow = false;
    LocalCounters lc;
    while (st.top) {
        uint32_t node;
        float bound;
        st.pop(&node, &bound);
        if (bound > tr.radius()) continue;
        if (heap_depth(node) == stop) {
            const SlotRange sr = subtree_slots(node, stop, p.node_depth, p.node_count, p.leaf_slots);
            const float* slot = p.leaf + sr.first * p.leaf_stride;
            ++lc.leaves;
            for (uint32_t s = 0; s < sr.count; ++s, slot += p.leaf_stride) {
                int32_t id;
                const float d2 = slot_dist<DP>(q, slot, &id);
                if (id < 0) continue;
                ++lc.points;
                tr.offer(make_key(d2, id));
            }
            continue;
        }
        ++lc.nodes;
        const uint32_t l = 2 * node + 1;
        const float bl = box_bound<DP>(q, box + static_cast<size_t>(l) * box_stride);
        const float br = box_bound<DP>(q, box + static_cast<size_t>(l + 1) * box_stride);
        const bool left_first = bl <= br;  // pushed last, popped first
        const uint32_t far_node = left_first ? l + 1 : l, near_node = left_first ? l : l + 1;
        const float far_b = left_first ? br : bl, near_b = left_first ? bl : br;
        if (far_b <= tr.radius()) overflow |= !st.push(far_node, far_b);
        if (near_b <= tr.radius()) overflow |= !st.push(near_node, near_b);
    }
    tr.emit(p.k, p.out_idx + static_cast<size_t>(qi) * p.k, p.out_dist + static_cast<size_t>(qi) * p.k);
    if (p.counters) {
        lc.flush(p.counters);
        if (overflow) atomicExch(&p.counters->error, 1);
    }
}

// The group search's leftovers, from each one's radius in `seeds`: one query per warp (lane 0),
// warps striding over the list.  The leftovers lie scattered in space, so 32 of them in one warp
// would take 32 different paths one after another; a warp each runs them side by side.
template <int DP, int KMAX>
__global__ void __launch_bounds__(128) kd_fallback_kernel(const KdGroupParams gp) {
    if ((threadIdx.x & 31u) != 0) return;
    const uint32_t n = *gp.fb_count;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; t < n; t += warps) {
        const uint32_t qi = gp.fb_list[t];
        kd_box_search<DP, KMAX>(gp.p, gp.box, gp.box_stride, gp.p.stop_depth, qi, gp.seeds[qi]);
    }
}

// ---- one query per warp: the group search's leftovers -----------------------------------------
// The leftovers are mostly queries far from the data (their k-th distance is large and the ball
// brushes many buckets of a dense cluster) or queries whose seed held far more points than a
// list: searched by one thread each they took up to ~0.6 ms apiece and set the length of the
// whole pass.  Here a warp searches one of them: each step tests the up-to-32 descendants five
// levels below a node, one per lane (the box bound against the current k-th distance), scans the
// wanted buckets one per lane, and merges the candidates into a top-32 held across the warp
// (lane i the i-th smallest key) by bitonic sorting networks over shuffles.  Exact as the other
// searches: a subtree is skipped only when its box bound exceeds the current k-th distance.
constexpr uint32_t kSoloFan = 5;     // levels per step: up to 32 descendants, one per lane
constexpr uint32_t kSoloStack = 256; // at most 31 net entries per step, 7 steps deep
constexpr uint32_t kSoloCand = 1024; // candidates of one step: 32 buckets of at most 32 slots

struct SoloWarpSmem {
    uint64_t cand[kSoloCand];
    uint32_t stack[kSoloStack];
    uint32_t ncand;
};

__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, uint32_t m) {
    const uint32_t lo = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(v), m);
    const uint32_t hi = __shfl_xor_sync(0xFFFFFFFFu, static_cast<uint32_t>(v >> 32), m);
    return (static_cast<uint64_t>(hi) << 32) | lo;
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, uint32_t src) {
    const uint32_t lo = __shfl_sync(0xFFFFFFFFu, static_cast<uint32_t>(v), src);
    const uint32_t hi = __shfl_sync(0xFFFFFFFFu, static_cast<uint32_t>(v >> 32), src);
    return (static_cast<uint64_t>(hi) << 32) | lo;
}

// Ascending bitonic sort of 32 keys, one per lane.
__device__ __forceinline__ uint64_t warp_sort64(uint64_t v, uint32_t lane) {
#pragma unroll
    for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const uint64_t o = shfl_xor64(v, j);
            const bool up = (lane & k) == 0, lower = (lane & j) == 0;
            v = (lower == up) ? (v < o ? v : o) : (v < o ? o : v);
        }
    }
    return v;
}

// The 32 smallest of two ascending 32-key sequences (one key per lane each), ascending.
__device__ __forceinline__ uint64_t warp_merge_low64(uint64_t a, uint64_t b, uint32_t lane) {
    const uint64_t rb = shfl64(b, 31 - lane);
    uint64_t v = a < rb ? a : rb;  // a bitonic sequence holding the 32 smallest
#pragma unroll
    for (uint32_t j = 16; j > 0; j >>= 1) {
        const uint64_t o = shfl_xor64(v, j);
        v = (lane & j) == 0 ? (v < o ? v : o) : (v < o ? o : v);
    }
    return v;
}

template <int DP, int KMAX>
__global__ void __launch_bounds__(128) kd_solo_kernel(const KdGroupParams gp) {
    static_assert(KMAX <= 32, "the top-k is held one key per lane");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SoloWarpSmem& sm = reinterpret_cast<SoloWarpSmem*>(smem_raw)[threadIdx.x >> 5];
    const KdParams& p = gp.p;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stop = p.stop_depth;
    const uint32_t n = *gp.fb_count;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    LocalCounters lc;
    bool stack_error = false;
    for (uint32_t t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; t < n; t += warps) {
        const uint32_t qi = gp.fb_list[t];
        float q[DP];
        load_query<DP>(p.queries, p.dims, qi, q);
        const float r2 = gp.seeds[qi];
        uint64_t top = make_key(r2, -1);  // lane i: the i-th smallest key so far
        float kth = r2;
        if (lane == 0) sm.stack[0] = 0;
        uint32_t depth_n = 1;  // stack entries
        while (depth_n) {
            __syncwarp();
            const uint32_t node = sm.stack[--depth_n];
            const uint32_t levels = min(kSoloFan, stop - heap_depth(node));
            const uint32_t fan = 1u << levels;
            const uint32_t first = ((node + 1) << levels) - 1;
            const bool want =
                lane < fan && box_bound<DP>(q, gp.box + static_cast<size_t>(first + lane) * gp.box_stride) <= kth;
            const uint32_t wm = __ballot_sync(0xFFFFFFFFu, want);
            if (heap_depth(node) + levels == stop) {
                if (lane == 0) sm.ncand = 0;
                __syncwarp();
                if (want) {
                    const SlotRange sr = subtree_slots(first + lane, stop, p.node_depth, p.node_count, p.leaf_slots);
                    const float* slot = p.leaf + sr.first * p.leaf_stride;
                    ++lc.leaves;
                    for (uint32_t s = 0; s < sr.count; ++s, slot += p.leaf_stride) {
                        int32_t id;
                        const float d2 = slot_dist<DP>(q, slot, &id);
                        if (id < 0) continue;
                        ++lc.points;
                        if (d2 <= kth) {
                            const uint32_t pos = atomicAdd(&sm.ncand, 1u);
                            if (pos < kSoloCand) sm.cand[pos] = make_key(d2, id);
                        }
                    }
                }
                __syncwarp();
                const uint32_t nc = min(sm.ncand, kSoloCand);  // at most 32 buckets of <= 32 slots
                for (uint32_t base = 0; base < nc; base += 32) {
                    const uint64_t x = base + lane < nc ? sm.cand[base + lane] : ~0ull;
                    top = warp_merge_low64(top, warp_sort64(x, lane), lane);
                }
                kth = key_dist(shfl64(top, p.k - 1));
            } else {
                ++lc.nodes;
                const uint32_t cnt = __popc(wm);
                if (depth_n + cnt > kSoloStack) {  // cannot happen (see kSoloStack); recorded
                    stack_error = true;
                    continue;
                }
                // The lowest-numbered descendant ends on top (popped first).
                if (want) sm.stack[depth_n + cnt - 1 - __popc(wm & ((1u << lane) - 1u))] = first + lane;
                depth_n += cnt;
            }
        }
        if (lane < p.k) {
            p.out_idx[static_cast<size_t>(qi) * p.k + lane] = key_index(top);
            p.out_dist[static_cast<size_t>(qi) * p.k + lane] = key_dist(top);
        }
    }
    if (p.counters) {
        lc.flush(p.counters);
        if (stack_error) atomicExch(&p.counters->error, 1);
    }
}

// Traversal 3: one box-bounded search per thread, in the batch's locality order.
template <int DP, int KMAX>
__global__ void __launch_bounds__(128) kd_box_knn_kernel(const KdParams p, const float* __restrict__ box,
                                                         uint32_t box_stride) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (p.count_dev ? *p.count_dev : p.nq)) return;
    const uint32_t qi = p.order ? p.order[t] - p.order_base : t;
    kd_box_search<DP, KMAX>(p, box, box_stride, p.stop_depth, qi, p.radii ? p.radii[qi] : p.max_d2);
}

// Self seeds: each query's k-th distance among the points of the subtree of at least
// max(4k, 32) slots it descends to -- an upper bound on its k-th neighbour distance (those
// points are real points), capped by the caller's radius.  The caller's radius where the
// subtree holds fewer than k points.
template <int DP, int KMAX>
__global__ void __launch_bounds__(128) kd_self_seed_kernel(const KdParams p, uint32_t seed_depth, float* __restrict__ seeds) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.nq) return;
    const uint32_t qi = p.order ? p.order[t] : t;
    float q[DP];
    load_query<DP>(p.queries, p.dims, qi, q);
    const float R = p.radii ? p.radii[qi] : p.max_d2;
    uint32_t node = 0;
    for (uint32_t depth = 0; depth < seed_depth; ++depth) {
        const float diff = pick<DP>(q, depth % p.aux) - __ldg(p.split + node);
        node = 2 * node + (diff < 0.0f ? 1u : 2u);
    }
    Tracker<KMAX, false, false> tr;
    tr.init(p.k, R, nullptr, 0);
    const SlotRange sr = subtree_slots(node, seed_depth, p.node_depth, p.node_count, p.leaf_slots);
    const float* slot = p.leaf + sr.first * p.leaf_stride;
    for (uint32_t s = 0; s < sr.count; ++s, slot += p.leaf_stride) {
        int32_t id;
        const float d2 = slot_dist<DP>(q, slot, &id);
        if (id >= 0) tr.offer(make_key(d2, id));
    }
    seeds[qi] = tr.radius();  // the caller's radius while fewer than k points were offered
}

// Tight boxes of the nodes down to `depth` (per node lo[QS], hi[QS]; padding slots excluded).
template <int DP>
__global__ void kd_box_bottom_kernel(const float* __restrict__ leaf, uint32_t leaf_stride, uint32_t depth,
                                     uint32_t node_depth, uint32_t node_count, uint32_t leaf_slots,
                                     float* __restrict__ box, uint32_t box_stride) {
    constexpr int QS = box_qs(DP);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (1u << depth)) return;
    const uint32_t node = (1u << depth) - 1u + i;
    float lo[QS], hi[QS];
#pragma unroll
    for (int d = 0; d < QS; ++d) {
        lo[d] = d < DP ? INFINITY : 0.0f;
        hi[d] = d < DP ? -INFINITY : 0.0f;
    }
    const SlotRange sr = subtree_slots(node, depth, node_depth, node_count, leaf_slots);
    const float* slot = leaf + sr.first * leaf_stride;
    for (uint32_t s = 0; s < sr.count; ++s, slot += leaf_stride) {
        if (__float_as_int(slot[DP]) < 0) continue;  // padding
#pragma unroll
        for (int d = 0; d < DP; ++d) {
            lo[d] = fminf(lo[d], slot[d]);
            hi[d] = fmaxf(hi[d], slot[d]);
        }
    }
    float* out = box + static_cast<size_t>(node) * box_stride;
#pragma unroll
    for (int d = 0; d < QS; ++d) {
        out[d] = lo[d];
        out[QS + d] = hi[d];
    }
}

template <int QS>
__global__ void kd_box_up_kernel(float* __restrict__ box, uint32_t depth) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (1u << depth)) return;
    const uint32_t node = (1u << depth) - 1u + i;
    const float* a = box + static_cast<size_t>(2 * node + 1) * (2 * QS);
    const float* b = a + 2 * QS;
    float* out = box + static_cast<size_t>(node) * (2 * QS);
#pragma unroll
    for (int d = 0; d < QS; ++d) {
        out[d] = fminf(a[d], b[d]);
        out[QS + d] = fmaxf(a[QS + d], b[QS + d]);
    }
}

template <uint32_t DP>
int kd_box_build_dp(knn_index* ix, cudaStream_t s) {
    constexpr uint32_t QS = box_qs(DP);
    const uint32_t depth = ix->kd_box_depth;
    const size_t nodes = (static_cast<size_t>(2) << depth) - 1;
    ix->kd_box_stride = 2 * QS;
    KNN_TRY(ix->kd_box.alloc(nodes * ix->kd_box_stride * sizeof(float)));
    kd_box_bottom_kernel<DP><<<ceil_div(1u << depth, 256), 256, 0, s>>>(
        ix->leaf.as<float>(), ix->leaf_stride, depth, ix->node_depth, ix->node_count, ix->leaf_slots,
        ix->kd_box.as<float>(), ix->kd_box_stride);
    KNN_LAUNCHED();
    for (uint32_t d = depth; d-- > 0;) {
        kd_box_up_kernel<QS><<<ceil_div(1u << d, 256), 256, 0, s>>>(ix->kd_box.as<float>(), d);
        KNN_LAUNCHED();
    }
    return KNN_OK;
}

inline uint32_t bucket_slots_of(const KdParams& p) { return p.leaf_slots << (p.node_depth - p.stop_depth); }

template <int DP, int KMAX>
static int launch_kd_group(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order,
                           float* seeds, bool self_seed, uint32_t* fb_list, uint32_t* fb_count, float seed_scale,
                           cudaStream_t s) {
    KdGroupParams gp{};
    KdParams& p = gp.p;
    p.split = ix->split.as<float>();
    p.leaf = ix->leaf.as<float>();
    p.leaf_stride = ix->leaf_stride;
    p.node_count = ix->node_count;
    p.node_depth = ix->node_depth;
    p.stop_depth = scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan ? plan.leaf_scan : 8u);
    if (p.stop_depth > ix->kd_box_depth) p.stop_depth = ix->kd_box_depth;
    p.leaf_slots = ix->leaf_slots;
    p.aux = ix->aux_dims;
    p.queries = a.queries;
    p.dims = ix->dims;
    p.nq = a.count;
    p.order = order;
    p.max_d2 = a.max_d2;
    p.radii = a.radii;
    p.k = a.k;
    p.out_idx = a.out_idx;
    p.out_dist = a.out_dist;
    p.counters = a.counters;
    gp.box = ix->kd_box.as<float>();
    gp.box_stride = ix->kd_box_stride;
    gp.seeds = seeds;
    gp.seed_scale = seed_scale;
    gp.fb_list = fb_list;
    gp.fb_count = fb_count;
    gp.group_counter = fb_count + 1;  // the count's scratch slot holds 256 bytes
    KNN_TRY_CUDA(cudaMemsetAsync(fb_count, 0, 2 * sizeof(uint32_t), s));
    if (self_seed) {
        // Subtree of at least max(4k, 32) slots.
        const uint32_t want = std::max<uint32_t>(32u, 4u * a.k);
        uint32_t sd = ix->node_depth;
        while (sd > 0 && (static_cast<uint64_t>(ix->leaf_slots) << (ix->node_depth - sd)) < want) --sd;
        kd_self_seed_kernel<DP, KMAX><<<ceil_div(a.count, 128), 128, 0, s>>>(p, sd, seeds);
        KNN_LAUNCHED();
    }
    constexpr size_t smem = group_smem_bytes<DP, KMAX>();
    auto kern = kd_group_kernel<DP, KMAX>;
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    if (plan.timing) KNN_TRY(ix->timing.begin(s));
    int per_sm = 0;
    KNN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kGroupWarps, smem));
    const uint32_t grid = std::min<uint32_t>(ceil_div(a.count, 32 * kGroupWarps),
                                             static_cast<uint32_t>(std::max(per_sm, 1) * sm_count()));
    kern<<<grid, 32 * kGroupWarps, smem, s>>>(gp);
    KNN_LAUNCHED();
    if (bucket_slots_of(p) <= 32) {
        constexpr size_t solo_smem = 4 * sizeof(SoloWarpSmem);
        KNN_TRY_CUDA(cudaFuncSetAttribute(kd_solo_kernel<DP, KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(solo_smem)));
        kd_solo_kernel<DP, KMAX><<<8 * static_cast<uint32_t>(sm_count()), 128, solo_smem, s>>>(gp);
    } else {
        kd_fallback_kernel<DP, KMAX><<<8 * static_cast<uint32_t>(sm_count()), 128, 0, s>>>(gp);
    }
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY(ix->timing.end(s));
    return KNN_OK;
}

template <uint32_t DP>
int kd_box_prepare_dp(knn_index* ix, cudaStream_t s);

// Builds the node boxes on first use (down to subtrees of at most 4 slots).
template <uint32_t DP>
int kd_box_ensure(knn_index* ix, cudaStream_t s) {
    if (ix->kd_box.ptr) return KNN_OK;
    ix->kd_box_depth = scan_depth_for(ix->node_depth, ix->leaf_slots, 4);
    return kd_box_build_dp<DP>(ix, s);
}

// Traversal 3 (plan.box): per-thread box-bounded search, buckets of plan.leaf_scan slots (0 = 8).
template <uint32_t DP>
int kd_box_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order, cudaStream_t s) {
    if constexpr (DP > 16) {
        return fail(KNN_ERR_INVALID_ARGUMENT, "box search: dims above 16");
    } else {
        KNN_TRY(kd_box_ensure<DP>(ix, s));
        KdParams p{};
        p.split = ix->split.as<float>();
        p.leaf = ix->leaf.as<float>();
        p.leaf_stride = ix->leaf_stride;
        p.node_count = ix->node_count;
        p.node_depth = ix->node_depth;
        p.stop_depth = std::min(scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan ? plan.leaf_scan : 8u),
                                ix->kd_box_depth);
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
        const uint32_t grid = ceil_div(a.count, 128);
        if (plan.timing) KNN_TRY(ix->timing.begin(s));
        switch (k_class(a.k)) {
            case 8: kd_box_knn_kernel<DP, 8><<<grid, 128, 0, s>>>(p, ix->kd_box.as<float>(), ix->kd_box_stride); break;
            case 16: kd_box_knn_kernel<DP, 16><<<grid, 128, 0, s>>>(p, ix->kd_box.as<float>(), ix->kd_box_stride); break;
            case 32: kd_box_knn_kernel<DP, 32><<<grid, 128, 0, s>>>(p, ix->kd_box.as<float>(), ix->kd_box_stride); break;
            case 64: kd_box_knn_kernel<DP, 64><<<grid, 128, 0, s>>>(p, ix->kd_box.as<float>(), ix->kd_box_stride); break;
            default: kd_box_knn_kernel<DP, 128><<<grid, 128, 0, s>>>(p, ix->kd_box.as<float>(), ix->kd_box_stride); break;
        }
        KNN_LAUNCHED();
        if (plan.timing) KNN_TRY(ix->timing.end(s));
        return KNN_OK;
    }
}

// Warp-group search (plan.group) with per-query seeds (or self seeds when `seeds` holds none):
// boxes built on first use, locality order, the group kernel and the fallback list.  Scratch
// (seeds when self-seeded, the fallback list) comes from the index workspace after the order.
template <uint32_t DP>
int kd_group_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, const uint32_t* order,
                      float* seeds, uint32_t* fb_list, uint32_t* fb_count, float seed_scale, cudaStream_t s) {
    if constexpr (DP > 16) {
        return fail(KNN_ERR_INVALID_ARGUMENT, "group search: dims above 16");
    } else {
        if (a.k > 32) return fail(KNN_ERR_INVALID_ARGUMENT, "group search: k above 32");
        KNN_TRY(kd_box_ensure<DP>(ix, s));
        const bool self_seed = seeds == nullptr;
        const size_t n = a.count;
        if (self_seed) {
            KNN_TRY(ix->group_ws.reserve(carve_bytes({n * 4, n * 4, 256})));
            Carver c(ix->group_ws.ptr);
            seeds = c.take<float>(n);
            fb_list = c.take<uint32_t>(n);
            fb_count = c.take<uint32_t>(1);
        }
        switch (k_class(a.k)) {
            case 8: return launch_kd_group<DP, 8>(ix, a, plan, order, seeds, self_seed, fb_list, fb_count, seed_scale, s);
            case 16: return launch_kd_group<DP, 16>(ix, a, plan, order, seeds, self_seed, fb_list, fb_count, seed_scale, s);
            default: return launch_kd_group<DP, 32>(ix, a, plan, order, seeds, self_seed, fb_list, fb_count, seed_scale, s);
        }
    }
}

template int kd_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);
template int kd_box_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, const uint32_t*, cudaStream_t);
template <>
int kd_box_prepare_dp<KNN_DP>(knn_index* ix, cudaStream_t s) {
    if constexpr (KNN_DP > 16) return fail(KNN_ERR_INVALID_ARGUMENT, "box search: dims above 16");
    else return kd_box_ensure<KNN_DP>(ix, s);
}
template int kd_group_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, const uint32_t*, float*,
                                        uint32_t*, uint32_t*, float, cudaStream_t);
template int kd_order_dp<KNN_DP>(knn_index*, const QueryArgs&, cudaStream_t, const uint32_t**, uint32_t);


// ---- batches of independent sets (one persistent kernel per class of sets) -----------------------
struct KdBatchSet {
    KdParams p;                 // the set's search parameters; p.order is the class order, p.order_base its offset
    uint32_t first_block;  // first work block of this set in the class
    uint32_t query_offset; // first query of this set in the class-wide numbering
    uint32_t levels;       // descent depth of the locality key
    const float* box;      // the index's node boxes (box-search classes), or null
    uint32_t box_stride;
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
// MODE: 0 per-thread search, 1 warp-coherent search, 2 per-thread box search (dims <= 16).
template <int DP, int KMAX, int MODE>
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
        if constexpr (MODE == 1) {
            kd_search_warp<DP, KMAX, false, false, false>(p, t, p.nq, smem);
        } else if constexpr (MODE == 2 && DP <= 16) {
            if (t < p.nq) {
                const uint32_t qi = p.order ? p.order[t] - p.order_base : t;
                kd_box_search<DP, KMAX>(p, sets[si].box, sets[si].box_stride, p.stop_depth, qi,
                                        p.radii ? p.radii[qi] : p.max_d2);
            }
        } else {
            if (t < p.nq) kd_search_thread<DP, KMAX, false, false, false>(p, t, smem);
        }
    }
}

template <uint32_t DP>
int kd_batch_launch(const void* sets, uint32_t nsets, uint32_t total_queries, uint32_t total_blocks, uint32_t kmax,
                       uint32_t mode, uint32_t block, uint32_t* counter, uint32_t* keys, uint32_t* vals, bool key_pass,
                       cudaStream_t s) {
    using Set = KdBatchSet;
    const Set* d_sets = static_cast<const Set*>(sets);
    if (key_pass) {
        kd_batch_key_kernel<DP><<<ceil_div(total_queries, 256), 256, 0, s>>>(d_sets, nsets, total_queries, keys, vals);
        KNN_LAUNCHED();
        return KNN_OK;
    }
#define KNN_BATCH(KM, W)                                                                              \
    if (kmax == KM && mode == W) {                                                                    \
        auto kern = kd_batch_kernel<DP, KM, W>;                                                    \
        int per_sm = 0;                                                                               \
        KNN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0));         \
        const uint32_t grid = std::max(1, per_sm) * static_cast<uint32_t>(sm_count());                \
        kern<<<std::min(grid, total_blocks), block, 0, s>>>(d_sets, nsets, total_blocks, counter);   \
        KNN_LAUNCHED();                                                                               \
        return KNN_OK;                                                                                \
    }
    KNN_BATCH(8, 0) KNN_BATCH(16, 0) KNN_BATCH(32, 0) KNN_BATCH(64, 0) KNN_BATCH(128, 0)
    KNN_BATCH(8, 1) KNN_BATCH(16, 1) KNN_BATCH(32, 1) KNN_BATCH(64, 1) KNN_BATCH(128, 1)
    KNN_BATCH(8, 2) KNN_BATCH(16, 2) KNN_BATCH(32, 2) KNN_BATCH(64, 2) KNN_BATCH(128, 2)
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
    if (plan.box && ix->kd_box.ptr) {  // prepared by kd_box_prepare before the batch is captured
        bs.box = ix->kd_box.as<float>();
        bs.box_stride = ix->kd_box_stride;
        p.stop_depth = std::min(scan_depth_for(ix->node_depth, ix->leaf_slots, plan.leaf_scan ? plan.leaf_scan : 8u),
                                ix->kd_box_depth);
    }
    std::memcpy(out, &bs, sizeof(bs));
}
#endif

template int kd_batch_launch<KNN_DP>(const void*, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t*,
                                      uint32_t*, uint32_t*, bool, cudaStream_t);

}  // namespace knn
