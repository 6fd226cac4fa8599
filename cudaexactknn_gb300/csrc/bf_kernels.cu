// Brute-force exact kNN kernels, one translation unit per padded dimension count (KNN_DP).
//
// Replaces BruteForceKernels::knnKernel / knnShKernel (src/BruteForceGpu.cuh:9-50), where one
// thread scans all n points for its query straight from global memory.  Here:
//   * a block stages tiles of points in shared memory with 16-byte vector loads; every thread
//     of the block reads the same point at once (a shared-memory broadcast);
//   * each thread keeps its query in registers and its top-k in the tracker the plan selects;
//   * when there are too few queries to fill the GPU, the point range is split across
//     gridDim.y and a merge kernel combines the per-split sorted lists.
// Distances are the reference's sequential fused sums (knn::dist2_vec4), so keys, ties and
// results equal the reference's brute force bit for bit.

#include <algorithm>

#include "knn_internal.h"
#include "tracker.cuh"

#ifndef KNN_DP
#error "compile with -DKNN_DP=<padded dims>"
#endif

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

template <int DP, int KMAX, bool HEAP, bool SHNN>
__global__ void __launch_bounds__(256) bf_knn_kernel(const BfParams p) {
    constexpr int PS = (DP + 3) / 4 * 4;
    extern __shared__ __align__(16) unsigned char smem[];
    float4* tile4 = reinterpret_cast<float4*>(smem);
    uint64_t* sh_nn = reinterpret_cast<uint64_t*>(smem + static_cast<size_t>(p.tile) * PS * sizeof(float));

    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < (p.count_dev ? *p.count_dev : p.nq);
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
        for (uint32_t i = threadIdx.x; i < cnt * (PS / 4); i += blockDim.x)
            tile4[i] = src[static_cast<size_t>(base) * (PS / 4) + i];
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

template <int DP, int KMAX, bool HEAP, bool SHNN>
static int launch_bf(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, cudaStream_t s) {
    constexpr int PS = (DP + 3) / 4 * 4;
    const uint32_t block = plan.block ? plan.block : 128;
    const uint32_t tile = std::max(32u, 8192u / PS);
    const size_t smem = static_cast<size_t>(tile) * PS * sizeof(float) + tracker_smem_bytes(SHNN, KMAX, block);
    auto kern = bf_knn_kernel<DP, KMAX, HEAP, SHNN>;
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));

    int per_sm = 0;
    KNN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
    if (per_sm <= 0) return fail(KNN_ERR_INVALID_ARGUMENT, "brute-force launch does not fit: block %u, %zu B shared", block, smem);
    const uint32_t qblocks = ceil_div(a.count, block);
    // Split the point range until the grid covers the GPU about four times over, keeping at
    // least four tiles per split.
    const uint64_t want = 4ull * sm_count() * per_sm;
    uint32_t splits = std::min<uint32_t>(ceil_div(static_cast<uint32_t>(std::min<uint64_t>(want, 0xFFFFFFFFu)), qblocks), 0xFFFFu);
    splits = std::max(1u, std::min(splits, ceil_div(ix->n, 4 * tile)));
    const uint32_t chunk = ceil_div(ceil_div(ix->n, splits), tile) * tile;
    splits = ceil_div(ix->n, chunk);

    BfParams p{};
    p.points = ix->points.as<float>();
    p.n = ix->n;
    p.queries = a.queries;
    p.dims = ix->dims;
    p.nq = a.count;
    p.max_d2 = a.max_d2;
    p.radii = a.radii;
    p.order = a.order;
    p.count_dev = a.count_dev;
    p.k = a.k;
    p.chunk = chunk;
    p.tile = tile;
    p.out_idx = a.out_idx;
    p.out_dist = a.out_dist;
    if (splits > 1) {
        const size_t need = static_cast<size_t>(splits) * a.count * a.k * sizeof(uint64_t) + 256;
        KNN_TRY(ix->workspace.reserve(need));
        p.partial = ix->workspace.as<uint64_t>();
    }
    dim3 grid(qblocks, splits);
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern0, s));
    kern<<<grid, block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern1, s));
    if (splits > 1) {
        bf_merge_kernel<KMAX><<<ceil_div(a.count, 128), 128, 0, s>>>(p.partial, splits, a.count, a.k, a.max_d2,
                                                                      a.radii, a.order, a.count_dev, a.out_idx,
                                                                      a.out_dist);
        KNN_LAUNCHED();
    }
    return KNN_OK;
}

template <int DP, int KMAX>
static int launch_bf_variant(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    if (p.heap)
        return p.sh_nn ? launch_bf<DP, KMAX, true, true>(ix, a, p, s) : launch_bf<DP, KMAX, true, false>(ix, a, p, s);
    return p.sh_nn ? launch_bf<DP, KMAX, false, true>(ix, a, p, s) : launch_bf<DP, KMAX, false, false>(ix, a, p, s);
}

template <uint32_t DP>
int bf_query_dp(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    switch (k_class(a.k)) {
        case 8: return launch_bf_variant<DP, 8>(ix, a, p, s);
        case 16: return launch_bf_variant<DP, 16>(ix, a, p, s);
        case 32: return launch_bf_variant<DP, 32>(ix, a, p, s);
        case 64: return launch_bf_variant<DP, 64>(ix, a, p, s);
        default: return launch_bf_variant<DP, 128>(ix, a, p, s);
    }
}

template int bf_query_dp<KNN_DP>(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);

}  // namespace knn
