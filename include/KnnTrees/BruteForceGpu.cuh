// BruteForceGpu.cuh -- drop-in replacement of src/BruteForceGpu.cuh (rezvoj/CudaExactKnn) on the
// GB300 engine.  Same class, constructor and batchKnn template as the reference
// (src/BruteForceGpu.cuh:54-85); the work runs in the engine (knn_bf_create / knn_query).
#pragma once

#include "KnnTrees.cuh"

namespace KnnTrees {

template <uint Dims>
class BruteForceGpu {
  public:
    using Point = Array<float, Dims>;

    // `points`: device memory, `size` points; copied into the index (as the reference does).
    BruteForceGpu(const Point* points, const uint size) {
        detail::run(knn_bf_create(reinterpret_cast<const float*>(points), size, Dims, nullptr, &mIndex));
        Cuda::check(cudaDeviceSynchronize());
    }
    ~BruteForceGpu() { knn_destroy(mIndex); }
    // The index owns device memory: copying it would free it twice (the reference's class has
    // that defect), so copies are disabled and moves transfer ownership.
    BruteForceGpu(const BruteForceGpu&) = delete;
    BruteForceGpu& operator=(const BruteForceGpu&) = delete;
    BruteForceGpu(BruteForceGpu&& o) noexcept : mIndex(o.mIndex) { o.mIndex = nullptr; }

    template <uint K, uint BlockSize, bool HeapNN, bool SharedMem>
    void batchKnn(Query<Dims, K>& query) const {
        detail::query(mIndex, query, detail::options(BlockSize, HeapNN, SharedMem, false));
    }

    knn_index* handle() const { return mIndex; }

  private:
    knn_index* mIndex = nullptr;
};

}  // namespace KnnTrees
