// k-d tree: construction and the query dispatcher over padded dimension counts.
//
// Replaces KdTreeGpu's constructor and mSplitPoints (src/KdTreeGpu.cuh:297-385).  Same tree:
// node_depth = log2Ceil(n) - skips levels of internal nodes in an implicit heap, split
// dimension = depth % aux_dims, a node of n points sends ceil(n/2) to the left child, the split
// value is the largest left value along the split dimension (src/KdTreeGpu.cuh:229-238), and
// leaves hold 2^skips slots padded with index -1 (src/KdTreeGpu.cuh:354-363).  The
// construction is the presorted-orders scheme of tree_build.cuh: aux_dims radix sorts up front,
// then per level one split kernel and one stable partition of the other orders.

#include <algorithm>
#include <vector>

#include "tree_build.cuh"

namespace knn {

template <uint32_t DP>
int kd_query_dp(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);
template <uint32_t DP>
int kd_order_dp(knn_index*, const QueryArgs&, cudaStream_t, const uint32_t**, uint32_t);
template <uint32_t DP>
int kd_group_query_dp(knn_index*, const QueryArgs&, const QueryPlan&, const uint32_t*, float*, uint32_t*, uint32_t*,
                      float, cudaStream_t);
template <uint32_t DP>
int kd_box_prepare_dp(knn_index*, cudaStream_t);

namespace {

// Split value and side flags of level `level` from the split dimension's order.
__global__ void kd_split_kernel(const uint32_t* __restrict__ ord, const float* __restrict__ pts, uint32_t n,
                                uint32_t dims, uint32_t dim, const uint32_t* __restrict__ node_of,
                                const uint32_t* __restrict__ off, const uint32_t* __restrict__ size,
                                float* __restrict__ split_level, uint8_t* __restrict__ side) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t j = node_of[p];
    const uint32_t rel = p - off[j], left = (size[j] + 1) / 2;
    const uint32_t id = ord[p];
    side[id] = rel >= left ? 1 : 0;
    if (rel + 1 == left) split_level[j] = pts[static_cast<size_t>(id) * dims + dim];
}

// Leaf slots: coordinates (zero padded to the leaf stride) then the index bits; empty slots
// carry index -1.
__global__ void write_leaves_kernel(const uint32_t* __restrict__ ord, const float* __restrict__ pts,
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

__global__ void init_root_kernel(uint32_t* off, uint32_t* size, uint32_t n, uint32_t* node_of, uint32_t count) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        off[0] = 0;
        size[0] = n;
    }
    if (p < count) node_of[p] = 0;
}

}  // namespace

// Leaf slot stride (floats) and position of the index within a slot.
void leaf_layout(uint32_t dp, uint32_t* stride, uint32_t* id_at) {
    if (dp < 4) {
        *stride = 4;
        *id_at = dp;
    } else {
        *stride = dp + 4;
        *id_at = dp;
    }
}

int kd_build(knn_index* ix, const float* d_points, uint32_t, cudaStream_t s) {
    const uint32_t n = ix->n, A = ix->aux_dims, nd = ix->node_depth;
    const uint32_t leaves = 1u << nd;
    leaf_layout(ix->dp, &ix->leaf_stride, &ix->leaf_id_at);
    KNN_TRY(ix->split.alloc(sizeof(float) * std::max<uint32_t>(ix->node_count, 1)));
    KNN_TRY(ix->leaf.alloc(sizeof(float) * static_cast<size_t>(leaves) * ix->leaf_slots * ix->leaf_stride));
    ix->device_bytes = ix->split.bytes + ix->leaf.bytes;

    DevBuf scratch_buf;
    KNN_TRY(scratch_buf.alloc(build::scratch_bytes(n, A, leaves)));
    build::Scratch sc{};
    build::carve_scratch(sc, scratch_buf.ptr, n, A, leaves);

    for (uint32_t a = 0; a < A; ++a) KNN_TRY(build::sort_dimension(sc, d_points, n, ix->dims, a, a, s));

    init_root_kernel<<<ceil_div(n, 256), 256, 0, s>>>(sc.off[0], sc.size[0], n, sc.node_of[0], n);
    KNN_LAUNCHED();
    int cur = 0, tab = 0, nof = 0;
    std::vector<uint32_t> others;
    for (uint32_t level = 0; level < nd; ++level) {
        const uint32_t count = 1u << level;
        const uint32_t dim = level % A;
        kd_split_kernel<<<ceil_div(n, 256), 256, 0, s>>>(sc.ord[cur][dim], d_points, n, ix->dims, dim,
                                                         sc.node_of[nof], sc.off[tab], sc.size[tab],
                                                         ix->split.as<float>() + (count - 1), sc.side);
        KNN_LAUNCHED();
        others.clear();
        for (uint32_t b = 0; b < A; ++b)
            if (b != dim) others.push_back(b);
        KNN_TRY(build::partition_orders(sc, others.data(), static_cast<uint32_t>(others.size()), cur,
                                        sc.node_of[nof], sc.off[tab], sc.size[tab], n, s));
        // The split order is already partitioned: its left entries lead each segment.
        std::swap(sc.ord[0][dim], sc.ord[1][dim]);
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
    write_leaves_kernel<<<static_cast<uint32_t>((total_slots + 255) / 256), 256, 0, s>>>(
        sc.ord[cur][0], d_points, ix->dims, ix->leaf_slots, leaves, sc.off[tab], sc.size[tab], ix->leaf_stride,
        ix->leaf_id_at, ix->leaf.as<float>());
    KNN_LAUNCHED();
    KNN_TRY_CUDA(cudaStreamSynchronize(s));  // scratch is freed on return
    return KNN_OK;
}

int kd_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    switch (ix->dp) {
        case 1: return kd_query_dp<1>(ix, a, p, s);
        case 2: return kd_query_dp<2>(ix, a, p, s);
        case 3: return kd_query_dp<3>(ix, a, p, s);
        case 4: return kd_query_dp<4>(ix, a, p, s);
        case 8: return kd_query_dp<8>(ix, a, p, s);
        case 16: return kd_query_dp<16>(ix, a, p, s);
        case 32: return kd_query_dp<32>(ix, a, p, s);
        case 64: return kd_query_dp<64>(ix, a, p, s);
        case 128: return kd_query_dp<128>(ix, a, p, s);
        default: return fail(KNN_ERR_UNSUPPORTED, "dims %u", ix->dims);
    }
}

int kd_group_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, const uint32_t* order, float* seeds,
                   uint32_t* fb_list, uint32_t* fb_count, float seed_scale, cudaStream_t s) {
    switch (ix->dp) {
        case 1: return kd_group_query_dp<1>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        case 2: return kd_group_query_dp<2>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        case 3: return kd_group_query_dp<3>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        case 4: return kd_group_query_dp<4>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        case 8: return kd_group_query_dp<8>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        case 16: return kd_group_query_dp<16>(ix, a, p, order, seeds, fb_list, fb_count, seed_scale, s);
        default: return fail(KNN_ERR_INVALID_ARGUMENT, "group search: dims above 16");
    }
}

int kd_box_prepare(knn_index* ix, cudaStream_t s) {
    switch (ix->dp) {
        case 1: return kd_box_prepare_dp<1>(ix, s);
        case 2: return kd_box_prepare_dp<2>(ix, s);
        case 3: return kd_box_prepare_dp<3>(ix, s);
        case 4: return kd_box_prepare_dp<4>(ix, s);
        case 8: return kd_box_prepare_dp<8>(ix, s);
        case 16: return kd_box_prepare_dp<16>(ix, s);
        default: return fail(KNN_ERR_INVALID_ARGUMENT, "box search: dims above 16");
    }
}

int kd_order(knn_index* ix, const QueryArgs& a, cudaStream_t s, const uint32_t** order, uint32_t max_levels) {
    switch (ix->dp) {
        case 1: return kd_order_dp<1>(ix, a, s, order, max_levels);
        case 2: return kd_order_dp<2>(ix, a, s, order, max_levels);
        case 3: return kd_order_dp<3>(ix, a, s, order, max_levels);
        case 4: return kd_order_dp<4>(ix, a, s, order, max_levels);
        case 8: return kd_order_dp<8>(ix, a, s, order, max_levels);
        case 16: return kd_order_dp<16>(ix, a, s, order, max_levels);
        case 32: return kd_order_dp<32>(ix, a, s, order, max_levels);
        case 64: return kd_order_dp<64>(ix, a, s, order, max_levels);
        case 128: return kd_order_dp<128>(ix, a, s, order, max_levels);
        default: return fail(KNN_ERR_UNSUPPORTED, "dims %u", ix->dims);
    }
}

}  // namespace knn
