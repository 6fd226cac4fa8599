// Brute-force kNN that allocates no device memory: for callers that cannot call cudaMalloc at
// query time (code running inside a CUDA graph being captured, an allocator-owning framework
// that forbids side allocations, a real-time loop that must not touch the allocator) and that
// cannot keep an index either, since creating one allocates.  The caller passes its own device
// points, queries and result buffers; the only scratch the query needs (the per-split partial
// top-k lists of the brute-force kernel) lives in a fixed array compiled into this library.
//
// Limits and sharing:
//   * the scratch is a 16 MiB file-scope __device__ array; every GPU that loads this library
//     holds it until the process exits;
//   * count * k must be at most 1,048,576 (two split partial lists of 8-byte keys per query and
//     slot must fit); larger batches are rejected with KNN_ERR_UNSUPPORTED before any launch;
//   * every call on a device shares the one array: calls whose work overlaps on the GPU (other
//     streams, other threads) race on it and must be serialised by the caller;
//   * the array keeps whatever the last call left in it; nothing in it has to start at zero,
//     because the merge kernel reads only slots the search kernel wrote earlier in the same call;
//   * the first call on each device looks up the array's device address (cudaGetSymbolAddress,
//     with that device current) and caches it; make that first call before any stream capture.
//     The cached address belongs to the device's primary context: after a cudaDeviceReset of
//     that device (which also invalidates every index of this library on it) it is stale, so do
//     not call this entry point again in a process that has reset the device.

#include <algorithm>
#include <mutex>

#include "bf_kernels.cuh"

namespace knn {

namespace {

constexpr size_t kScratchBytes = 16u << 20;
constexpr size_t kScratchKeys = kScratchBytes / sizeof(uint64_t);
constexpr uint64_t kMaxCountTimesK = kScratchKeys / 2;  // at least two splits must fit
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchKeys];

std::mutex g_scratch_mutex;
uint64_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
int scratch_address(uint64_t** out) {
    int dev = 0;
    KNN_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KNN_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)", __FILE__, __LINE__);
        g_scratch_ptr[dev] = static_cast<uint64_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return KNN_OK;
}

template <int DP, int KMAX>
int run(const float* points, uint32_t n, uint32_t dims, const float* queries, uint32_t count, float max_d2,
        uint32_t k, int32_t* idx, float* dist, uint64_t* scratch, cudaStream_t s) {
    constexpr int PS = (DP + 3) / 4 * 4;
    constexpr uint32_t block = 128;
    const uint32_t tile = std::max(32u, 8192u / PS);
    const size_t smem = static_cast<size_t>(tile) * PS * sizeof(float);
    auto kern = bf_knn_kernel<DP, KMAX, false, false, true>;
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int per_sm = 0;
    KNN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
    const uint32_t qblocks = ceil_div(count, block);
    // As many point-range splits as fill the GPU about four times over, limited by the scratch.
    const uint64_t want = 4ull * sm_count() * std::max(per_sm, 1);
    uint32_t splits = static_cast<uint32_t>(std::min<uint64_t>(ceil_div(static_cast<uint32_t>(std::min<uint64_t>(want, 0xFFFFFFFFu)), qblocks), 0xFFFFu));
    splits = std::min<uint64_t>(splits, kScratchKeys / (static_cast<uint64_t>(count) * k));
    splits = std::max(2u, std::min(splits, ceil_div(n, tile)));
    const uint32_t chunk = ceil_div(ceil_div(n, splits), tile) * tile;
    splits = ceil_div(n, chunk);
    BfParams p{};
    p.points = points;
    p.n = n;
    p.queries = queries;
    p.dims = dims;
    p.nq = count;
    p.max_d2 = max_d2;
    p.k = k;
    p.chunk = chunk;
    p.tile = tile;
    p.out_idx = idx;
    p.out_dist = dist;
    p.partial = splits > 1 ? scratch : nullptr;
    kern<<<dim3(qblocks, splits), block, smem, s>>>(p);
    KNN_LAUNCHED();
    if (splits > 1) {
        bf_merge_kernel<KMAX><<<ceil_div(count, 128), 128, 0, s>>>(scratch, splits, count, k, max_d2, nullptr, nullptr,
                                                                    nullptr, idx, dist);
        KNN_LAUNCHED();
    }
    return KNN_OK;
}

template <int DP>
int run_k(const float* points, uint32_t n, uint32_t dims, const float* queries, uint32_t count, float max_d2,
          uint32_t k, int32_t* idx, float* dist, uint64_t* scratch, cudaStream_t s) {
    switch (k_class(k)) {
        case 8: return run<DP, 8>(points, n, dims, queries, count, max_d2, k, idx, dist, scratch, s);
        case 16: return run<DP, 16>(points, n, dims, queries, count, max_d2, k, idx, dist, scratch, s);
        case 32: return run<DP, 32>(points, n, dims, queries, count, max_d2, k, idx, dist, scratch, s);
        case 64: return run<DP, 64>(points, n, dims, queries, count, max_d2, k, idx, dist, scratch, s);
        default: return run<DP, 128>(points, n, dims, queries, count, max_d2, k, idx, dist, scratch, s);
    }
}

}  // namespace

}  // namespace knn

extern "C" int knn_bf_query_noalloc(const float* d_points, uint32_t n, uint32_t dims, const float* d_queries,
                                    uint32_t count, float max_distance2, uint32_t k, int32_t* d_indexes,
                                    float* d_distances, void* stream) {
    using namespace knn;
    if (dims == 0 || k == 0) return fail(KNN_ERR_INVALID_ARGUMENT, "dims and k must be >= 1");
    if (dims > kMaxDims || k > kMaxK) return fail(KNN_ERR_UNSUPPORTED, "dims %u / k %u beyond 128", dims, k);
    if (!(max_distance2 >= 0.0f)) return fail(KNN_ERR_INVALID_ARGUMENT, "max_distance2 must be >= 0");
    if (static_cast<uint64_t>(count) * k > kMaxCountTimesK)
        return fail(KNN_ERR_UNSUPPORTED,
                    "count * k = %llu exceeds %llu, the most the allocation-free query's 16 MiB scratch holds",
                    static_cast<unsigned long long>(count) * k, static_cast<unsigned long long>(kMaxCountTimesK));
    if (count == 0) return KNN_OK;
    if (!d_queries || !d_indexes || !d_distances || (n > 0 && !d_points))
        return fail(KNN_ERR_INVALID_ARGUMENT, "null pointer");
    if (n > 0x7FFFFFFFu) return fail(KNN_ERR_UNSUPPORTED, "n %u >= 2^31", n);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        QueryArgs a{d_queries, count, max_distance2, nullptr, k, d_indexes, d_distances, nullptr};
        return fill_empty_rows(a, s);
    }
    uint64_t* scratch = nullptr;
    KNN_TRY(scratch_address(&scratch));
    switch (padded_dims(dims)) {
        case 1: return run_k<1>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 2: return run_k<2>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 3: return run_k<3>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 4: return run_k<4>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 8: return run_k<8>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 16: return run_k<16>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 32: return run_k<32>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        case 64: return run_k<64>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
        default: return run_k<128>(d_points, n, dims, d_queries, count, max_distance2, k, d_indexes, d_distances, scratch, s);
    }
}
