// KdTreeGpu.cuh -- drop-in replacement of src/KdTreeGpu.cuh (rezvoj/CudaExactKnn) on the GB300
// engine.  Same class template (AuxDims defaults to Dims, CBlockSize to 256), constructor with
// depthSkips, and batchKnn<K, BLOCK_SIZE, HEAP, SH_NN, SH_STACK> (src/KdTreeGpu.cuh:282-412; constructor
// 375-385, batchKnn 393-410).
#pragma once

// Standard headers the reference's version brings in (directly or through <cub/cub.cuh>);
// code written against the reference may rely on them.
#include <algorithm>
#include <cassert>
#include <cstring>
#include <limits>
#include <numeric>

#include "KnnTrees.cuh"

namespace KnnTrees {

template <uint Dims, uint AuxDims = Dims, uint CBlockSize = 256>
class KdTreeGpu {
    static_assert(AuxDims >= 1 && AuxDims <= Dims, "AuxDims must be in [1, Dims]");

  public:
    using Point = Array<float, Dims>;

    // `points`: device memory, read during construction only.
    KdTreeGpu(const Point* points, const uint size, const uint depthSkips = 0) {
        detail::run(knn_kd_create(reinterpret_cast<const float*>(points), size, Dims, AuxDims, depthSkips,
                                  CBlockSize, nullptr, &mIndex));
        Cuda::check(cudaDeviceSynchronize());
    }
    ~KdTreeGpu() { knn_destroy(mIndex); }
    KdTreeGpu(const KdTreeGpu&) = delete;
    KdTreeGpu& operator=(const KdTreeGpu&) = delete;
    KdTreeGpu(KdTreeGpu&& o) noexcept : mIndex(o.mIndex) { o.mIndex = nullptr; }

    template <uint K, uint BlockSize, bool HeapNN, bool SharedMemNN, bool SharedMemStack>
    void batchKnn(Query<Dims, K>& query) const {
        detail::query(mIndex, query, detail::options(BlockSize, HeapNN, SharedMemNN, SharedMemStack));
    }

    knn_index* handle() const { return mIndex; }

  private:
    knn_index* mIndex = nullptr;
};

}  // namespace KnnTrees
