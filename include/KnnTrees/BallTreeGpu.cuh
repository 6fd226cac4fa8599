// BallTreeGpu.cuh -- drop-in replacement of src/BallTreeGpu.cuh (rezvoj/CudaExactKnn) on the
// GB300 engine.  Same class template (CBlockSize defaults to 256), constructor with depthSkips
// (default 1, at least 1), and batchKnn<K, BLOCK_SIZE, HEAP, SH_NN, SH_STACK>
// (src/BallTreeGpu.cuh:463-650).
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

template <uint Dims, uint CBlockSize = 256>
class BallTreeGpu {
  public:
    using Point = Array<float, Dims>;

    BallTreeGpu(const Point* points, const uint size, const uint depthSkips = 1) {
        detail::run(knn_ball_create(reinterpret_cast<const float*>(points), size, Dims, depthSkips, CBlockSize,
                                    nullptr, &mIndex));
        Cuda::check(cudaDeviceSynchronize());
    }
    ~BallTreeGpu() { knn_destroy(mIndex); }
    BallTreeGpu(const BallTreeGpu&) = delete;
    BallTreeGpu& operator=(const BallTreeGpu&) = delete;
    BallTreeGpu(BallTreeGpu&& o) noexcept : mIndex(o.mIndex) { o.mIndex = nullptr; }

    template <uint K, uint BlockSize, bool HeapNN, bool SharedMemNN, bool SharedMemStack>
    void batchKnn(Query<Dims, K>& query) const {
        detail::query(mIndex, query, detail::options(BlockSize, HeapNN, SharedMemNN, SharedMemStack));
    }

    knn_index* handle() const { return mIndex; }

  private:
    knn_index* mIndex = nullptr;
};

}  // namespace KnnTrees
