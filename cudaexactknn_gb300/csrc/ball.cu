// Ball tree: construction and the query dispatcher.
//
// Replaces BallTreeGpu's constructor and mSplitPoints (src/BallTreeGpu.cuh:480-624).  Same
// tree: node_depth = log2Ceil(n) - skips levels (skips >= 1, src/BallTreeGpu.cuh:615), a node's
// split dimension is the one with the largest sum of squared deviations from the node's
// centroid (strict >, first wins, src/BallTreeGpu.cuh:296-306), the left child takes ceil(n/2)
// points in order along that dimension, and every node carries a ball: centroid = mean of its
// points, radius >= the distance to its farthest point.
//
// Differences by design:
//   * centroids come from deterministic chunked sums of the coordinates (fixed order), not from
//     differences of float prefix sums over all n points (src/BallTreeGpu.cuh:253-255), which
//     lose precision for large n;
//   * the radius is rounded up to a rigorous bound on the exact farthest distance
//     (knn::ball_radius), so traversal bounds never cut off a point that belongs in the answer;
//   * balls are stored per node (node i's own ball at index i, leaves included) instead of in
//     the parent's {left, right} record (src/KnnTrees.cuh:31-37); siblings are adjacent, so a
//     visit still reads both children's balls from one place.

#include <algorithm>
#include <vector>

#include "tree_build.cuh"

namespace knn {

template <uint32_t DP>
int ball_query_dp(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);
template <uint32_t DP>
int ball_order_dp(knn_index*, const QueryArgs&, cudaStream_t, const uint32_t**);
void leaf_layout(uint32_t dp, uint32_t* stride, uint32_t* id_at);

namespace {

constexpr uint32_t kChunk = 1024;  // positions per reduction item (one warp)

struct LevelView {
    const uint32_t* ord;      // any order (positions -> point id)
    const uint32_t* off;
    const uint32_t* size;
    uint32_t count;           // nodes at this level
    uint32_t cpn;             // chunks per node
};

// Per (node, chunk): sum of the coordinates of the chunk's points.
template <int DP>
__global__ void __launch_bounds__(128) partial_sum_kernel(const LevelView lv, const float* __restrict__ pts,
                                                          uint32_t dims, float* __restrict__ partial) {
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (item >= lv.count * lv.cpn) return;
    const uint32_t j = item / lv.cpn, c = item % lv.cpn;
    const uint32_t o = lv.off[j], sz = lv.size[j];
    const uint32_t lo = o + min(sz, c * kChunk), hi = o + min(sz, (c + 1) * kChunk);
    float acc[DP];
#pragma unroll
    for (int d = 0; d < DP; ++d) acc[d] = 0.0f;
    for (uint32_t p = lo + lane; p < hi; p += 32) {
        const float* x = pts + static_cast<size_t>(lv.ord[p]) * dims;
#pragma unroll
        for (int d = 0; d < DP; ++d)
            if (static_cast<uint32_t>(d) < dims) acc[d] += x[d];
    }
#pragma unroll
    for (int d = 0; d < DP; ++d) {
        float v = acc[d];
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o2);
        if (lane == 0) partial[static_cast<size_t>(item) * DP + d] = v;
    }
}

// Centroid of every node of the level; also stored as the node's ball centre.
template <int DP>
__global__ void centroid_kernel(const LevelView lv, const float* __restrict__ partial, uint32_t dims,
                                float* __restrict__ cent, float* __restrict__ ball, uint32_t ball_stride,
                                uint32_t node_base) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= lv.count) return;
    const float inv_n = static_cast<float>(lv.size[j]);
    float* b = ball + static_cast<size_t>(node_base + j) * ball_stride;
    for (uint32_t d = 0; d < static_cast<uint32_t>(DP); ++d) {
        float s = 0.0f;
        for (uint32_t c = 0; c < lv.cpn; ++c) s += partial[(static_cast<size_t>(j) * lv.cpn + c) * DP + d];
        const float v = (d < dims && lv.size[j] > 0) ? __fdiv_rn(s, inv_n) : 0.0f;
        cent[static_cast<size_t>(j) * DP + d] = v;
        b[d] = v;
    }
}

// Per (node, chunk): per-dimension sum of squared deviations from the centroid, and the largest
// float dist2 from the centroid (same arithmetic as the queries' distances).
template <int DP>
__global__ void __launch_bounds__(128) partial_spread_kernel(const LevelView lv, const float* __restrict__ pts,
                                                             uint32_t dims, const float* __restrict__ cent,
                                                             float* __restrict__ partial,
                                                             float* __restrict__ partial_max) {
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (item >= lv.count * lv.cpn) return;
    const uint32_t j = item / lv.cpn, c = item % lv.cpn;
    const uint32_t o = lv.off[j], sz = lv.size[j];
    const uint32_t lo = o + min(sz, c * kChunk), hi = o + min(sz, (c + 1) * kChunk);
    float cc[DP], acc[DP];
#pragma unroll
    for (int d = 0; d < DP; ++d) {
        cc[d] = cent[static_cast<size_t>(j) * DP + d];
        acc[d] = 0.0f;
    }
    float mx = 0.0f;
    for (uint32_t p = lo + lane; p < hi; p += 32) {
        const float* x = pts + static_cast<size_t>(lv.ord[p]) * dims;
        float xd[DP];
#pragma unroll
        for (int d = 0; d < DP; ++d) xd[d] = static_cast<uint32_t>(d) < dims ? x[d] : 0.0f;
        mx = fmaxf(mx, dist2<DP>(xd, cc));
#pragma unroll
        for (int d = 0; d < DP; ++d) {
            const float t = xd[d] - cc[d];
            acc[d] = __fmaf_rn(t, t, acc[d]);
        }
    }
#pragma unroll
    for (int d = 0; d < DP; ++d) {
        float v = acc[d];
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o2);
        if (lane == 0) partial[static_cast<size_t>(item) * DP + d] = v;
    }
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o2));
    if (lane == 0) partial_max[item] = mx;
}

// Split dimension (largest spread, strict >, first wins) and ball radius of every node.
template <int DP>
__global__ void spread_kernel(const LevelView lv, const float* __restrict__ partial,
                              const float* __restrict__ partial_max, uint32_t dims, float margin,
                              uint32_t* __restrict__ node_dim, float* __restrict__ ball, uint32_t ball_stride,
                              uint32_t node_base) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= lv.count) return;
    float best = 0.0f, mx = 0.0f;
    uint32_t best_dim = 0;
    for (uint32_t d = 0; d < dims; ++d) {
        float s = 0.0f;
        for (uint32_t c = 0; c < lv.cpn; ++c) s += partial[(static_cast<size_t>(j) * lv.cpn + c) * DP + d];
        if (s > best) {
            best = s;
            best_dim = d;
        }
    }
    for (uint32_t c = 0; c < lv.cpn; ++c) mx = fmaxf(mx, partial_max[static_cast<size_t>(j) * lv.cpn + c]);
    if (node_dim) node_dim[j] = best_dim;
    ball[static_cast<size_t>(node_base + j) * ball_stride + DP] = ball_radius(mx, margin);
}

// Side flags from each node's split dimension order.
struct OrderTable {
    const uint32_t* ord[kMaxDims];
};

__global__ void ball_side_kernel(const OrderTable ot, const uint32_t* __restrict__ node_of,
                                 const uint32_t* __restrict__ off, const uint32_t* __restrict__ size,
                                 const uint32_t* __restrict__ node_dim, uint32_t n, uint8_t* __restrict__ side) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t j = node_of[p];
    const uint32_t rel = p - off[j], left = (size[j] + 1) / 2;
    side[ot.ord[node_dim[j]][p]] = rel >= left ? 1 : 0;
}

__global__ void write_ball_leaves_kernel(const uint32_t* __restrict__ ord, const float* __restrict__ pts,
                                         uint32_t dims, uint32_t slots, uint32_t leaves,
                                         const uint32_t* __restrict__ off, const uint32_t* __restrict__ size,
                                         uint32_t stride, uint32_t id_at, float* __restrict__ leaf) {
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= static_cast<uint64_t>(slots) * leaves) return;
    const uint32_t j = static_cast<uint32_t>(s / slots), r = static_cast<uint32_t>(s % slots);
    float* out = leaf + s * stride;
    int32_t id = -1;
    if (r < size[j]) id = static_cast<int32_t>(ord[off[j] + r]);
    for (uint32_t d = 0; d < stride; ++d) out[d] = 0.0f;
    if (id >= 0)
        for (uint32_t d = 0; d < dims; ++d) out[d] = pts[static_cast<size_t>(id) * dims + d];
    out[id_at] = __int_as_float(id);
}

__global__ void init_root_kernel(uint32_t* off, uint32_t* size, uint32_t n, uint32_t* node_of) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        off[0] = 0;
        size[0] = n;
    }
    if (p < n) node_of[p] = 0;
}

template <int DP>
int level_balls(const LevelView& lv, const float* pts, uint32_t dims, float margin, float* partial,
                float* partial_max, float* cent, uint32_t* node_dim, float* ball, uint32_t ball_stride,
                uint32_t node_base, cudaStream_t s) {
    const uint32_t items = lv.count * lv.cpn;
    const uint32_t blocks = ceil_div(items, 4);
    partial_sum_kernel<DP><<<blocks, 128, 0, s>>>(lv, pts, dims, partial);
    centroid_kernel<DP><<<ceil_div(lv.count, 128), 128, 0, s>>>(lv, partial, dims, cent, ball, ball_stride, node_base);
    partial_spread_kernel<DP><<<blocks, 128, 0, s>>>(lv, pts, dims, cent, partial, partial_max);
    spread_kernel<DP><<<ceil_div(lv.count, 128), 128, 0, s>>>(lv, partial, partial_max, dims, margin, node_dim, ball,
                                                             ball_stride, node_base);
    KNN_LAUNCHED_N(4);
    return KNN_OK;
}

int level_balls_dp(uint32_t dp, const LevelView& lv, const float* pts, uint32_t dims, float margin, float* partial,
                   float* partial_max, float* cent, uint32_t* node_dim, float* ball, uint32_t ball_stride,
                   uint32_t node_base, cudaStream_t s) {
#define KNN_LB(D_) \
    case D_: return level_balls<D_>(lv, pts, dims, margin, partial, partial_max, cent, node_dim, ball, ball_stride, node_base, s);
    switch (dp) {
        KNN_LB(1) KNN_LB(2) KNN_LB(3) KNN_LB(4) KNN_LB(8) KNN_LB(16) KNN_LB(32) KNN_LB(64) KNN_LB(128)
        default: return fail(KNN_ERR_UNSUPPORTED, "dims");
    }
#undef KNN_LB
}

}  // namespace

int ball_build(knn_index* ix, const float* d_points, uint32_t, cudaStream_t s) {
    const uint32_t n = ix->n, D = ix->dims, nd = ix->node_depth, dp = ix->dp;
    const uint32_t leaves = 1u << nd;
    const uint32_t total_nodes = 2 * leaves - 1;
    leaf_layout(dp, &ix->leaf_stride, &ix->leaf_id_at);
    ix->ball_stride = ix->leaf_stride;  // centre (dp floats), radius at index dp
    KNN_TRY(ix->ball.alloc(sizeof(float) * static_cast<size_t>(total_nodes) * ix->ball_stride));
    KNN_TRY(ix->leaf.alloc(sizeof(float) * static_cast<size_t>(leaves) * ix->leaf_slots * ix->leaf_stride));
    KNN_TRY_CUDA(cudaMemsetAsync(ix->ball.ptr, 0, ix->ball.bytes, s));
    ix->device_bytes = ix->ball.bytes + ix->leaf.bytes;
    const float margin = rel_margin(D);

    // Reduction scratch: one partial row per (node, chunk) item; items <= n/kChunk + nodes.
    const size_t max_items = static_cast<size_t>(n) / kChunk + 2 * static_cast<size_t>(leaves) + 2;
    DevBuf red;
    KNN_TRY(red.alloc(carve_bytes({max_items * dp * 4, max_items * 4, static_cast<size_t>(leaves) * dp * 4,
                                   static_cast<size_t>(leaves) * 4})));
    Carver rc(red.ptr);
    float* partial = rc.take<float>(max_items * dp);
    float* partial_max = rc.take<float>(max_items);
    float* cent = rc.take<float>(static_cast<size_t>(leaves) * dp);
    uint32_t* node_dim = rc.take<uint32_t>(leaves);

    DevBuf scratch_buf;
    KNN_TRY(scratch_buf.alloc(build::scratch_bytes(n, D, leaves)));
    build::Scratch sc{};
    build::carve_scratch(sc, scratch_buf.ptr, n, D, leaves);
    for (uint32_t a = 0; a < D; ++a) KNN_TRY(build::sort_dimension(sc, d_points, n, D, a, a, s));

    init_root_kernel<<<ceil_div(n, 256), 256, 0, s>>>(sc.off[0], sc.size[0], n, sc.node_of[0]);
    KNN_LAUNCHED();
    int cur = 0, tab = 0, nof = 0;
    std::vector<uint32_t> all(D);
    for (uint32_t b = 0; b < D; ++b) all[b] = b;
    for (uint32_t level = 0; level <= nd; ++level) {
        const uint32_t count = 1u << level;
        const uint32_t max_size = static_cast<uint32_t>((static_cast<uint64_t>(n) + count - 1) / count);
        LevelView lv{sc.ord[cur][0], sc.off[tab], sc.size[tab], count, std::max(1u, ceil_div(max_size, kChunk))};
        KNN_TRY(level_balls_dp(dp, lv, d_points, D, margin, partial, partial_max, cent,
                               level < nd ? node_dim : nullptr, ix->ball.as<float>(), ix->ball_stride, count - 1, s));
        if (level == nd) break;
        OrderTable ot{};
        for (uint32_t b = 0; b < D; ++b) ot.ord[b] = sc.ord[cur][b];
        ball_side_kernel<<<ceil_div(n, 256), 256, 0, s>>>(ot, sc.node_of[nof], sc.off[tab], sc.size[tab], node_dim, n,
                                                          sc.side);
        KNN_LAUNCHED();
        KNN_TRY(build::partition_orders(sc, all.data(), D, cur, sc.node_of[nof], sc.off[tab], sc.size[tab], n, s));
        build::next_node_of_kernel<<<ceil_div(n, 256), 256, 0, s>>>(sc.node_of[nof], sc.off[tab], sc.size[tab], n,
                                                                    sc.node_of[nof ^ 1]);
        build::children_kernel<<<ceil_div(count, 256), 256, 0, s>>>(sc.off[tab], sc.size[tab], count,
                                                                    sc.off[tab ^ 1], sc.size[tab ^ 1]);
        KNN_LAUNCHED_N(2);
        cur ^= 1;
        tab ^= 1;
        nof ^= 1;
    }
    const uint64_t total_slots = static_cast<uint64_t>(leaves) * ix->leaf_slots;
    write_ball_leaves_kernel<<<static_cast<uint32_t>((total_slots + 255) / 256), 256, 0, s>>>(
        sc.ord[cur][0], d_points, D, ix->leaf_slots, leaves, sc.off[tab], sc.size[tab], ix->leaf_stride,
        ix->leaf_id_at, ix->leaf.as<float>());
    KNN_LAUNCHED();
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    return KNN_OK;
}

int ball_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    switch (ix->dp) {
        case 1: return ball_query_dp<1>(ix, a, p, s);
        case 2: return ball_query_dp<2>(ix, a, p, s);
        case 3: return ball_query_dp<3>(ix, a, p, s);
        case 4: return ball_query_dp<4>(ix, a, p, s);
        case 8: return ball_query_dp<8>(ix, a, p, s);
        case 16: return ball_query_dp<16>(ix, a, p, s);
        case 32: return ball_query_dp<32>(ix, a, p, s);
        case 64: return ball_query_dp<64>(ix, a, p, s);
        case 128: return ball_query_dp<128>(ix, a, p, s);
        default: return fail(KNN_ERR_UNSUPPORTED, "dims %u", ix->dims);
    }
}

int ball_order(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order) {
    switch (ix->dp) {
        case 1: return ball_order_dp<1>(ix, a, s, order);
        case 2: return ball_order_dp<2>(ix, a, s, order);
        case 3: return ball_order_dp<3>(ix, a, s, order);
        case 4: return ball_order_dp<4>(ix, a, s, order);
        case 8: return ball_order_dp<8>(ix, a, s, order);
        case 16: return ball_order_dp<16>(ix, a, s, order);
        case 32: return ball_order_dp<32>(ix, a, s, order);
        case 64: return ball_order_dp<64>(ix, a, s, order);
        case 128: return ball_order_dp<128>(ix, a, s, order);
        default: return fail(KNN_ERR_UNSUPPORTED, "dims %u", ix->dims);
    }
}

}  // namespace knn
