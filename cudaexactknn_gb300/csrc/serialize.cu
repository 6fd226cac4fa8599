// Serialised form of a built index, so that a tree built once can be reused by another process
// or on another GPU without rebuilding it.  The reference has no such format: its trees are device
// arrays held by the class instance only (src/KdTreeGpu.cuh:293-294, src/BallTreeGpu.cuh:461-462).
//
// Layout (little-endian, as on both x86-64 and aarch64):
//   Header (fixed size, below), then the payload: the structure's device arrays in a fixed order
//   (brute-force points, k-d splits, tree leaf slots, ball nodes, learned-radius model), each
//   exactly as it lies in device memory.  The header states each array's byte count, and a 64-bit
//   FNV-1a checksum covers the payload.
// Loading recomputes every array's size from (structure, n, dims, aux_dims, depth_skips) with the
// same rules construction uses and rejects a blob whose sizes, checksum, magic or version differ,
// before any device memory is touched: a tree whose arrays disagree with its shape would send the
// search kernels out of bounds.  The tensor-core filter's layout and the autotuned plans are not
// stored (they are rebuilt on first use, and plans are timed on the GPU at hand).

#include <cstring>
#include <new>

#include "knn_internal.h"

namespace knn {
void leaf_layout(uint32_t dp, uint32_t* stride, uint32_t* id_at);
}

namespace {

constexpr char kMagic[8] = {'C', 'E', 'K', 'N', 'N', 'I', 'X', '1'};
constexpr uint32_t kVersion = 1;

struct Header {
    char magic[8];
    uint32_t version;
    uint32_t structure, n, dims, aux_dims, depth_skips;
    uint32_t has_model, model_k;
    uint64_t bytes[5];  // points, split, leaf, ball, model
    uint64_t checksum;  // FNV-1a 64 over the payload
};
static_assert(sizeof(Header) == 88, "header layout");

uint64_t fnv1a(const uint8_t* p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

// The shape fields construction derives from (structure, n, dims, aux_dims, skips), and the byte
// count of each array.  Mirrors knn_*_create + {bf,kd,ball}_build.
struct Shape {
    uint32_t dp = 0, skips = 0, node_depth = 0, leaf_slots = 0, node_count = 0;
    uint32_t point_stride = 0, leaf_stride = 0, leaf_id_at = 0, ball_stride = 0;
    uint64_t bytes[4] = {0, 0, 0, 0};
};

int derive_shape(uint32_t structure, uint32_t n, uint32_t dims, uint32_t aux_dims, uint32_t skips, Shape* sh) {
    if (dims < 1 || dims > knn::kMaxDims) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: dims %u", dims);
    // Construction accepts n < 2^31 only; beyond it the tree shape arithmetic below would shift
    // a 32-bit value by 32.
    if (n > 0x7FFFFFFFu) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: n %u >= 2^31", n);
    if (structure != KNN_BRUTE_FORCE && structure != KNN_KD_TREE && structure != KNN_BALL_TREE)
        return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: structure %u", structure);
    if (aux_dims < 1 || aux_dims > dims || (structure != KNN_KD_TREE && aux_dims != dims))
        return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: aux_dims %u", aux_dims);
    sh->dp = knn::padded_dims(dims);
    if (structure == KNN_BRUTE_FORCE) {
        sh->point_stride = (sh->dp + 3) & ~3u;
        sh->bytes[0] = static_cast<uint64_t>(n) * sh->point_stride * 4;
        return KNN_OK;
    }
    if (n == 0) return KNN_OK;
    // Tree shape: the clamped skips exactly as construction stores them (tree_shape in capi.cu).
    const uint32_t l2 = knn::log2_ceil(n);
    const bool ball = structure == KNN_BALL_TREE;
    uint32_t s = skips;
    if (ball && s < 1) s = 1;
    if (s > l2 - 1) s = l2 - 1;
    if (s != skips) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: depth_skips %u", skips);
    sh->skips = s;
    sh->node_depth = l2 - s;
    sh->leaf_slots = 1u << s;
    sh->node_count = (1u << sh->node_depth) - 1;
    knn::leaf_layout(sh->dp, &sh->leaf_stride, &sh->leaf_id_at);
    const uint64_t leaves = 1ull << sh->node_depth;
    sh->bytes[2] = 4ull * leaves * sh->leaf_slots * sh->leaf_stride;
    if (ball) {
        sh->ball_stride = sh->leaf_stride;
        sh->bytes[3] = 4ull * (2 * leaves - 1) * sh->ball_stride;
    } else {
        sh->bytes[1] = 4ull * (sh->node_count > 0 ? sh->node_count : 1u);
    }
    return KNN_OK;
}

knn::DevBuf* array_of(knn_index* ix, int i) {
    switch (i) {
        case 0: return &ix->points;
        case 1: return &ix->split;
        case 2: return &ix->leaf;
        case 3: return &ix->ball;
        default: return &ix->model;
    }
}

}  // namespace

extern "C" {

int knn_index_serialize(const knn_index* index, void* host_buf, size_t capacity, size_t* size, void* stream) {
    if (!index || !size) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    knn_index* ix = const_cast<knn_index*>(index);
    Header h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.structure = static_cast<uint32_t>(ix->structure);
    h.n = ix->n;
    h.dims = ix->dims;
    h.aux_dims = ix->aux_dims;
    h.depth_skips = ix->skips;
    h.has_model = ix->has_model ? 1u : 0u;
    h.model_k = ix->model_k;
    size_t total = sizeof(Header);
    for (int i = 0; i < 5; ++i) {
        const knn::DevBuf* b = array_of(ix, i);
        h.bytes[i] = (i == 4 && !ix->has_model) ? 0 : b->bytes;
        total += h.bytes[i];
    }
    *size = total;
    if (!host_buf) return KNN_OK;
    if (capacity < total) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "buffer of %zu bytes, %zu needed", capacity, total);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint8_t* out = static_cast<uint8_t*>(host_buf);
    size_t off = sizeof(Header);
    for (int i = 0; i < 5; ++i) {
        if (h.bytes[i]) KNN_TRY_CUDA(cudaMemcpyAsync(out + off, array_of(ix, i)->ptr, h.bytes[i], cudaMemcpyDeviceToHost, s));
        off += h.bytes[i];
    }
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    h.checksum = fnv1a(out + sizeof(Header), total - sizeof(Header));
    std::memcpy(out, &h, sizeof(Header));
    return KNN_OK;
}

int knn_index_deserialize(const void* host_buf, size_t size, void* stream, knn_index** out) {
    if (out) *out = nullptr;
    if (!host_buf || !out) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "null argument");
    if (size < sizeof(Header)) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: %zu bytes", size);
    Header h;
    std::memcpy(&h, host_buf, sizeof(Header));
    if (std::memcmp(h.magic, kMagic, 8) != 0) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: bad magic");
    if (h.version != kVersion) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: version %u", h.version);
    Shape sh;
    KNN_TRY(derive_shape(h.structure, h.n, h.dims, h.aux_dims, h.depth_skips, &sh));
    for (int i = 0; i < 4; ++i)
        if (h.bytes[i] != sh.bytes[i])
            return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: array %d holds %llu bytes, the shape needs %llu", i,
                             static_cast<unsigned long long>(h.bytes[i]), static_cast<unsigned long long>(sh.bytes[i]));
    const uint64_t model_bytes = h.has_model ? 4ull * knn::model_floats(h.dims) : 0ull;
    if (h.bytes[4] != model_bytes || (h.has_model && (h.model_k < 1 || h.model_k > knn::kMaxK)) || h.has_model > 1)
        return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: radius model");
    uint64_t total = sizeof(Header);
    for (int i = 0; i < 5; ++i) total += h.bytes[i];
    if (total != size) return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: %zu bytes, the header needs %llu", size,
                                        static_cast<unsigned long long>(total));
    const uint8_t* in = static_cast<const uint8_t*>(host_buf);
    if (fnv1a(in + sizeof(Header), size - sizeof(Header)) != h.checksum)
        return knn::fail(KNN_ERR_INVALID_ARGUMENT, "serialised index: checksum mismatch");

    auto* ix = new (std::nothrow) knn_index();
    if (!ix) return knn::fail(KNN_ERR_OUT_OF_MEMORY, "host allocation failed");
    cudaGetDevice(&ix->device);
    ix->structure = static_cast<int>(h.structure);
    ix->n = h.n;
    ix->dims = h.dims;
    ix->dp = sh.dp;
    ix->aux_dims = h.aux_dims;
    ix->skips = sh.skips;
    ix->node_depth = sh.node_depth;
    ix->leaf_slots = sh.leaf_slots;
    ix->node_count = sh.node_count;
    ix->point_stride = sh.point_stride;
    ix->leaf_stride = sh.leaf_stride;
    ix->leaf_id_at = sh.leaf_id_at;
    ix->ball_stride = sh.ball_stride;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = KNN_OK;
    size_t off = sizeof(Header);
    for (int i = 0; i < 5 && rc == KNN_OK; ++i) {
        if (h.bytes[i]) {
            knn::DevBuf* b = array_of(ix, i);
            rc = b->alloc(h.bytes[i]);
            if (rc == KNN_OK) {
                const cudaError_t e = cudaMemcpyAsync(b->ptr, in + off, h.bytes[i], cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) rc = knn::cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__);
            }
        }
        off += h.bytes[i];
    }
    if (rc == KNN_OK) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = knn::cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
    }
    if (rc == KNN_OK) rc = ix->counters.alloc(sizeof(knn::DevCounters));
    if (rc != KNN_OK) {
        delete ix;
        return rc;
    }
    ix->has_model = h.has_model != 0;
    ix->model_k = h.model_k;
    if (ix->has_model) {  // the model's margin is its last parameter (at the end of the blob)
        float m = 0.0f;
        std::memcpy(&m, in + size - sizeof(float), sizeof(float));
        ix->model_margin = m;
    }
    ix->device_bytes = h.bytes[0] + h.bytes[1] + h.bytes[2] + h.bytes[3];
    *out = ix;
    return KNN_OK;
}

}  // extern "C"
