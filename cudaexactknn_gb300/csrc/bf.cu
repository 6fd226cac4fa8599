// Brute force: construction (BruteForceGpu's constructor, src/BruteForceGpu.cuh:63-68, copies
// the caller's device points) and the query dispatcher over padded dimension counts.

#include "knn_internal.h"

namespace knn {

template <uint32_t DP>
int bf_query_dp(knn_index*, const QueryArgs&, const QueryPlan&, cudaStream_t);

namespace {

// Copies [n][dims] points into [n][stride] rows with zero padding.
__global__ void pad_rows_kernel(const float* __restrict__ src, uint32_t n, uint32_t dims, uint32_t stride,
                                float* __restrict__ dst) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<uint64_t>(n) * stride) return;
    const uint64_t row = i / stride;
    const uint32_t col = static_cast<uint32_t>(i % stride);
    dst[i] = col < dims ? src[row * dims + col] : 0.0f;
}

}  // namespace

int bf_build(knn_index* ix, const float* d_points, cudaStream_t s) {
    ix->point_stride = round_up4(ix->dp);
    const size_t elems = static_cast<size_t>(ix->n) * ix->point_stride;
    KNN_TRY(ix->points.alloc(elems * sizeof(float)));
    ix->device_bytes = ix->points.bytes;
    if (elems) {
        pad_rows_kernel<<<static_cast<uint32_t>((elems + 255) / 256), 256, 0, s>>>(d_points, ix->n, ix->dims,
                                                                                   ix->point_stride, ix->points.as<float>());
        KNN_LAUNCHED();
    }
    return KNN_OK;
}

int bf_query(knn_index* ix, const QueryArgs& a, const QueryPlan& p, cudaStream_t s) {
    switch (ix->dp) {
        case 1: return bf_query_dp<1>(ix, a, p, s);
        case 2: return bf_query_dp<2>(ix, a, p, s);
        case 3: return bf_query_dp<3>(ix, a, p, s);
        case 4: return bf_query_dp<4>(ix, a, p, s);
        case 8: return bf_query_dp<8>(ix, a, p, s);
        case 16: return bf_query_dp<16>(ix, a, p, s);
        case 32: return bf_query_dp<32>(ix, a, p, s);
        case 64: return bf_query_dp<64>(ix, a, p, s);
        case 128: return bf_query_dp<128>(ix, a, p, s);
        default: return fail(KNN_ERR_UNSUPPORTED, "dims %u", ix->dims);
    }
}

}  // namespace knn
