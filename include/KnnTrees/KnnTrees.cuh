// KnnTrees.cuh -- drop-in replacement of the reference's core header (src/KnnTrees.cuh of
// rezvoj/CudaExactKnn) for the GB300 engine.
//
// It provides the same names with the same meaning, so code written against the reference
// (including the reference's own CPU classes BruteForce/KdTree/BallTree and its tests) compiles
// unchanged:
//   Array<T,N>, IndexPoint<D>, BallNode<D>, Query<D,K>            src/KnnTrees.cuh:7-37,224-231
//   CudaException, Cuda::check / H2D / D2H / D2D / blockCount /
//   synchronizeStream(s)                                           src/KnnTrees.cuh:20-23,191-222
//   calcDistance2, pow2, log2Ceil, leftChildOf, parentOf, swap,
//   fillArray, copyArray                                           src/KnnTrees.cuh:39-103
//   encodeUintUFloat, encodeUintSFloat, encodeUFloatInt,
//   decodeEncoded1UFloat                                           src/KnnTrees.cuh:105-134
//   arrayConsider, heapConsider                                    src/KnnTrees.cuh:136-189
//   pinnedMalloc, pinnedFree                                       src/KnnTrees.cuh:233-243
// The GPU classes live in BruteForceGpu.cuh, KdTreeGpu.cuh and BallTreeGpu.cuh beside this file
// and run on the engine's C ABI (cudaexactknn.h; link with -lcudaexactknn).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <sys/types.h>

#include "cudaexactknn.h"  // needs -I<repo>/include

namespace KnnTrees {

template <typename Type, uint Size>
struct Array {
    Type arr[Size];
    __forceinline__ __host__ __device__ Type& operator[](uint i) { return arr[i]; }
    __forceinline__ __host__ __device__ const Type& operator[](uint i) const { return arr[i]; }
};

// Thrown for CUDA runtime failures (as in the reference) and for engine status codes.
class CudaException : public std::runtime_error {
  public:
    explicit CudaException(const cudaError_t error) : std::runtime_error(cudaGetErrorString(error)) {}
    CudaException(int status, const char* message)
        : std::runtime_error(std::string(message ? message : "") + " [" + knn_status_string(status) + "]"),
          mStatus(status) {}
    int status() const { return mStatus; }

  private:
    int mStatus = KNN_ERR_CUDA;
};

template <uint Dims>
struct IndexPoint {
    int index;
    Array<float, Dims> point;
};

template <uint Dims>
struct BallNode {
    Array<float, Dims> leftCentroid;
    float leftRadius;
    Array<float, Dims> rightCentroid;
    float rightRadius;
};

template <typename Type>
__forceinline__ __host__ __device__ void swap(Type& a, Type& b) {
    Type t = a;
    a = b;
    b = t;
}

template <typename Type, uint Size>
__forceinline__ __host__ __device__ void fillArray(Type* array, const Type& value) {
    for (uint i = 0; i < Size; ++i) array[i] = value;
}

template <typename Type, uint Size>
__forceinline__ __host__ __device__ void copyArray(const Type* from, Type* to) {
    for (uint i = 0; i < Size; ++i) to[i] = from[i];
}

// Squared distance: sequential sum over dimensions of the squared differences.
template <uint Dims>
__forceinline__ __host__ __device__ float calcDistance2(const Array<float, Dims>& a, const Array<float, Dims>& b) {
    float acc = 0.0f;
    for (uint d = 0; d < Dims; ++d) {
        const float t = a[d] - b[d];
        acc += t * t;
    }
    return acc;
}

__forceinline__ __host__ __device__ uint pow2(const uint exponent) { return 1u << exponent; }

// Smallest r >= 1 with 2^r >= input.
__forceinline__ __host__ __device__ uint log2Ceil(const uint input) {
    uint r = 1;
    unsigned long long c = 2;
    while (c < input) {
        c <<= 1;
        ++r;
    }
    return r;
}

__forceinline__ __host__ __device__ uint leftChildOf(const uint idx) { return 2 * idx + 1; }
__forceinline__ __host__ __device__ uint parentOf(const uint idx) { return (idx - 1) / 2; }

namespace detail {
__forceinline__ __host__ __device__ uint32_t bits(float f) {
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
    return u;
}
}  // namespace detail

// (integer << 32) | bits(non-negative float)
__forceinline__ __host__ __device__ uint64_t encodeUintUFloat(const uint integer, const float value) {
    return (static_cast<uint64_t>(integer) << 32) | detail::bits(value);
}

// (integer << 32) | order-preserving bits of a signed float
__forceinline__ __host__ __device__ uint64_t encodeUintSFloat(const uint integer, const float value) {
    const uint32_t u = detail::bits(value);
    const uint32_t ordered = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return (static_cast<uint64_t>(integer) << 32) | ordered;
}

// Result key: (bits(dist2) << 32) | uint32(index).
__forceinline__ __host__ __device__ uint64_t encodeUFloatInt(const float value, const int integer) {
    return (static_cast<uint64_t>(detail::bits(value)) << 32) | static_cast<uint32_t>(integer);
}

__forceinline__ __host__ __device__ float decodeEncoded1UFloat(const uint64_t key) {
    const uint32_t hi = static_cast<uint32_t>(key >> 32);
    float f;
    memcpy(&f, &hi, sizeof(f));
    return f;
}

// K keys kept ascending; returns the k-th distance.
template <uint K>
__forceinline__ __host__ __device__ float arrayConsider(uint64_t* nn, const int index, const float distance2) {
    uint64_t x = encodeUFloatInt(distance2, index);
    if (x < nn[K - 1]) {
        for (uint i = 0; i < K; ++i) {
            const uint64_t c = nn[i];
            nn[i] = c < x ? c : x;
            x = c < x ? x : c;
        }
    }
    return decodeEncoded1UFloat(nn[K - 1]);
}

// K keys kept as a max-heap rooted at slot 0; returns the k-th (largest kept) distance.
template <uint K>
__forceinline__ __host__ __device__ float heapConsider(uint64_t* nn, const int index, const float distance2) {
    const uint64_t x = encodeUFloatInt(distance2, index);
    if (x < nn[0]) {
        uint pos = 0;
        for (;;) {
            const uint l = 2 * pos + 1;
            if (l >= K) break;
            uint big = l;
            if (l + 1 < K && nn[l + 1] > nn[l]) big = l + 1;
            if (nn[big] <= x) break;
            nn[pos] = nn[big];
            pos = big;
        }
        nn[pos] = x;
    }
    return decodeEncoded1UFloat(nn[0]);
}

namespace Cuda {
constexpr cudaMemcpyKind H2D = cudaMemcpyHostToDevice;
constexpr cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
constexpr cudaMemcpyKind D2D = cudaMemcpyDeviceToDevice;

inline void check(const cudaError_t error) {
    if (error != cudaSuccess) throw CudaException(error);
}

// Engine status codes become exceptions with the engine's message.
inline void check(const knn_status status) {
    if (status != KNN_OK) throw CudaException(status, knn_last_error());
}

inline uint blockCount(const uint threadCount, const uint blockSize) { return (threadCount + blockSize - 1) / blockSize; }

inline void synchronizeStream(const cudaStream_t stream) { check(cudaStreamSynchronize(stream)); }

template <uint Size>
inline void synchronizeStreams(const cudaStream_t* streams) {
    for (uint i = 0; i < Size; ++i) check(cudaStreamSynchronize(streams[i]));
}
}  // namespace Cuda

template <uint Dims, uint K>
struct Query {
    const Array<float, Dims>* points;
    const uint count;
    const float maxDistance2;
    Array<int, K>* rIndexes;
    Array<float, K>* rDistances;
};

template <typename Type>
Type* pinnedMalloc(const uint size) {
    Type* p = nullptr;
    Cuda::check(cudaMallocHost(&p, sizeof(Type) * size));
    return p;
}

template <typename Type>
void pinnedFree(Type* pointer) {
    Cuda::check(cudaFreeHost(pointer));
}

namespace detail {
inline void run(const int status) { Cuda::check(static_cast<knn_status>(status)); }

// batchKnn's template arguments as engine query options; the call is synchronous like the
// reference's (it ends with a device-wide synchronisation).
inline knn_query_opts options(uint blockSize, bool heap, bool shNN, bool shStack) {
    knn_query_opts o;
    memset(&o, 0, sizeof(o));
    o.block_size = blockSize;
    o.heap_tracking = heap ? 1u : 0u;
    o.shmem_tracking = shNN ? 1u : 0u;
    o.shmem_stack = shStack ? 1u : 0u;
    return o;
}

template <uint Dims, uint K>
inline void query(knn_index* index, Query<Dims, K>& q, const knn_query_opts& o) {
    run(knn_query(index, reinterpret_cast<const float*>(q.points), q.count, q.maxDistance2, K,
                  reinterpret_cast<int32_t*>(q.rIndexes), reinterpret_cast<float*>(q.rDistances), &o, nullptr));
    Cuda::check(cudaDeviceSynchronize());
}
}  // namespace detail

}  // namespace KnnTrees
