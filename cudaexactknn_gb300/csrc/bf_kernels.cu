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

#include "bf_kernels.cuh"

#ifndef KNN_DP
#error "compile with -DKNN_DP=<padded dims>"
#endif

namespace knn {

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
    if (plan.timing) KNN_TRY(ix->timing.begin(s));
    kern<<<grid, block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY(ix->timing.end(s));
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
