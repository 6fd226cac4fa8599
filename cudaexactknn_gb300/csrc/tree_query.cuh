// Pieces shared by the k-d and ball tree query kernels: leaf-slot distance, the traversal
// stack, and query reordering by the leaf each query descends to.
#pragma once

#include "knn_internal.h"
#include "tracker.cuh"

namespace knn {

// Distance from q to a leaf slot and the slot's point index.  Slot layout: DP < 4 -> one
// float4 {coords..., index bits}; DP >= 4 -> DP/4 float4 of coordinates, then the index.
template <int DP>
__device__ __forceinline__ float slot_dist(const float (&q)[DP], const float* __restrict__ slot, int32_t* id) {
    const float4* s4 = reinterpret_cast<const float4*>(slot);
    if constexpr (DP < 4) {
        const float4 v = s4[0];
        const float c[3] = {v.x, v.y, v.z};
        const float w[4] = {v.x, v.y, v.z, v.w};
        *id = __float_as_int(w[DP]);
        float acc = 0.0f;
#pragma unroll
        for (int d = 0; d < DP; ++d) {
            const float t = __fsub_rn(q[d], c[d]);
            acc = __fmaf_rn(t, t, acc);
        }
        return acc;
    } else {
        *id = __float_as_int(slot[DP]);
        return dist2_vec4<DP>(q, s4);
    }
}

// Slots under node `node` at depth `depth` of a tree whose leaves sit at depth `leaf_depth`:
// the subtree's leaves are contiguous, so its slots are one range.
struct SlotRange {
    size_t first;
    uint32_t count;
};
__device__ __forceinline__ SlotRange subtree_slots(uint32_t node, uint32_t depth, uint32_t leaf_depth,
                                                  uint32_t node_count, uint32_t leaf_slots) {
    const uint32_t span = leaf_depth - depth;
    const uint64_t first_leaf = ((static_cast<uint64_t>(node) + 1) << span) - 1 - node_count;
    return SlotRange{static_cast<size_t>(first_leaf) * leaf_slots, leaf_slots << span};
}

// Scan depth for a plan: stop `levels` above the leaves so that a scanned range holds at most
// `max_points` slots (0 keeps the tree's own leaves).
inline uint32_t scan_depth_for(uint32_t node_depth, uint32_t leaf_slots, uint32_t max_points) {
    uint32_t levels = 0;
    while (levels < node_depth && (static_cast<uint64_t>(leaf_slots) << (levels + 1)) <= max_points) ++levels;
    return node_depth - levels;
}

// Index of the point in a leaf slot, without its coordinates.
template <int DP>
__device__ __forceinline__ int32_t slot_id(const float* __restrict__ slot) {
    return __float_as_int(slot[DP]);
}

// Depth-first stack of (node, bound) entries: registers/local memory, or shared memory laid
// out entry-major (entry e of thread t at e*block + t) so a warp's pushes hit distinct banks.
template <bool SHARED>
struct Stack {
    uint32_t node_l[SHARED ? 1 : kMaxTreeDepth + 1];
    float bound_l[SHARED ? 1 : kMaxTreeDepth + 1];
    uint32_t* node_s;
    float* bound_s;
    uint32_t stride;
    uint32_t top;

    __device__ __forceinline__ void init(uint32_t* sh, uint32_t block) {
        top = 0;
        if constexpr (SHARED) {
            node_s = sh + threadIdx.x;
            bound_s = reinterpret_cast<float*>(sh + (kMaxTreeDepth + 1) * block) + threadIdx.x;
            stride = block;
        }
    }
    // Returns false when full (cannot happen for trees of depth <= 32: the stack holds at most
    // one entry per level); the caller records a device error instead of writing past it.
    __device__ __forceinline__ bool push(uint32_t node, float bound) {
        if (top > kMaxTreeDepth) return false;
        if constexpr (SHARED) {
            node_s[top * stride] = node;
            bound_s[top * stride] = bound;
        } else {
            node_l[top] = node;
            bound_l[top] = bound;
        }
        ++top;
        return true;
    }
    __device__ __forceinline__ void pop(uint32_t* node, float* bound) {
        --top;
        if constexpr (SHARED) {
            *node = node_s[top * stride];
            *bound = bound_s[top * stride];
        } else {
            *node = node_l[top];
            *bound = bound_l[top];
        }
    }
};

__host__ __device__ constexpr size_t stack_smem_bytes(bool shared, uint32_t block) {
    return shared ? 2ull * (kMaxTreeDepth + 1) * block * sizeof(uint32_t) : 0;
}

// Loads a query (dims floats, zero padded to DP).
template <int DP>
__device__ __forceinline__ void load_query(const float* __restrict__ queries, uint32_t dims, uint32_t qi, float (&q)[DP]) {
    const float* src = queries + static_cast<size_t>(qi) * dims;
#pragma unroll
    for (int d = 0; d < DP; ++d) q[d] = static_cast<uint32_t>(d) < dims ? src[d] : 0.0f;
}

// Per-thread counters flushed once per thread (instrumented runs only).
struct LocalCounters {
    uint32_t nodes = 0, leaves = 0, points = 0;
    __device__ __forceinline__ void flush(DevCounters* c) const {
        if (!c) return;
        atomicAdd(&c->nodes, static_cast<unsigned long long>(nodes));
        atomicAdd(&c->leaves, static_cast<unsigned long long>(leaves));
        atomicAdd(&c->points, static_cast<unsigned long long>(points));
    }
};

}  // namespace knn
