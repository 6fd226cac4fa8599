// Brute-force kernel templates, shared by bf_kernels.cu (one translation unit per padded
// dimension count) and bf_noalloc.cu (the allocation-free entry point).
#pragma once

#include "knn_internal.h"
#include "tracker.cuh"

namespace knn {

struct BfParams {
    const float* points;  // [n][ps], zero padded
    uint32_t n;
    const float* queries;  // [nq][dims]
    uint32_t dims;
    uint32_t nq;
    float max_d2;
    const float* radii;
    const uint32_t* order;      // thread -> query, or null
    const uint32_t* count_dev;  // live thread count on the device, or null
    uint32_t k;
    uint32_t chunk;  // points per split
    uint32_t tile;   // points per shared-memory tile
    uint64_t* partial;  // [splits][nq][k] sorted keys, or null (single split)
    int32_t* out_idx;
    float* out_dist;
};

// RAW: points are read straight from the caller's [n][dims] array (zero padded while staging)
// instead of the index's padded copy.
template <int DP, int KMAX, bool HEAP, bool SHNN, bool RAW = false>
__global__ void __launch_bounds__(256) bf_knn_kernel(const BfParams p) {
    constexpr int PS = (DP + 3) / 4 * 4;
    extern __shared__ __align__(16) unsigned char smem[];
    float4* tile4 = reinterpret_cast<float4*>(smem);
    uint64_t* sh_nn = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(p.tile) * PS * sizeof(float));

    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t live = p.count_dev ? *p.count_dev : p.nq;
    if (blockIdx.x * blockDim.x >= live) return;  // the whole block is past the live list
    const bool active = t < live;
    const uint32_t qi = active ? (p.order ? p.order[t] : t) : 0u;
    float q[PS];
#pragma unroll
    for (int d = 0; d < PS; ++d)
        q[d] = (active && static_cast<uint32_t>(d) < p.dims) ? p.queries[static_cast<size_t>(qi) * p.dims + d] : 0.0f;
    const float r2 = active ? (p.radii ? p.radii[qi] : p.max_d2) : 0.0f;

    Tracker<KMAX, HEAP, SHNN> tr;
    tr.init(p.k, r2, sh_nn + threadIdx.x, blockDim.x);

    const uint32_t lo = blockIdx.y * p.chunk;
    const uint32_t hi = min(p.n, lo + p.chunk);
    const float4* src = reinterpret_cast<const float4*>(p.points);
    for (uint32_t base = lo; base < hi; base += p.tile) {
        const uint32_t cnt = min(p.tile, hi - base);
        __syncthreads();
        if constexpr (RAW) {
            float* tile = reinterpret_cast<float*>(tile4);
            for (uint32_t i = threadIdx.x; i < cnt * PS; i += blockDim.x) {
                const uint32_t j = i / PS, d = i % PS;
                tile[i] = d < p.dims ? p.points[static_cast<size_t>(base + j) * p.dims + d] : 0.0f;
            }
        } else {
            for (uint32_t i = threadIdx.x; i < cnt * (PS / 4); i += blockDim.x)
                tile4[i] = src[static_cast<size_t>(base) * (PS / 4) + i];
        }
        __syncthreads();
        if (active) {
            uint32_t j = 0;
            for (; j + 1 < cnt; j += 2) {
                // Two independent fused chains per step for instruction-level parallelism.
                const float d0 = dist2_vec4<PS>(q, tile4 + j * (PS / 4));
                const float d1 = dist2_vec4<PS>(q, tile4 + (j + 1) * (PS / 4));
                tr.offer(make_key(d0, static_cast<int32_t>(base + j)));
                tr.offer(make_key(d1, static_cast<int32_t>(base + j + 1)));
            }
            if (j < cnt) tr.offer(make_key(dist2_vec4<PS>(q, tile4 + j * (PS / 4)), static_cast<int32_t>(base + j)));
        }
    }
    if (!active) return;
    if (p.partial)
        tr.emit_keys(p.k, p.partial + (static_cast<size_t>(blockIdx.y) * p.nq + t) * p.k);
    else
        tr.emit(p.k, p.out_idx + static_cast<size_t>(qi) * p.k, p.out_dist + static_cast<size_t>(qi) * p.k);
}

// Combines the per-split sorted key lists of each query into its final row.
template <int KMAX>
__global__ void __launch_bounds__(128) bf_merge_kernel(const uint64_t* __restrict__ partial, uint32_t splits,
                                                       uint32_t nq, uint32_t k, float max_d2,
                                                       const float* __restrict__ radii,
                                                       const uint32_t* __restrict__ order,
                                                       const uint32_t* __restrict__ count_dev,
                                                       int32_t* __restrict__ out_idx,
                                                       float* __restrict__ out_dist) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (count_dev ? *count_dev : nq)) return;
    const uint32_t qi = order ? order[t] : t;
    Tracker<KMAX, false, false> tr;
    tr.init(k, radii ? radii[qi] : max_d2, nullptr, 0);
    for (uint32_t s = 0; s < splits; ++s) {
        const uint64_t* row = partial + (static_cast<size_t>(s) * nq + t) * k;
        for (uint32_t i = 0; i < k; ++i)
            if (!tr.offer(row[i])) break;  // rows are ascending
    }
    tr.emit(k, out_idx + static_cast<size_t>(qi) * k, out_dist + static_cast<size_t>(qi) * k);
}

}  // namespace knn
