// extern "C" bridge around the reference's own CPU classes, used to pin the oracle.
//
// TEST INFRASTRUCTURE ONLY.  This file holds no algorithm: it includes the reference's
// headers where they lie (the Makefile beside it passes -I<reference>/src) and instantiates
// BruteForce<D>, KdTree<D> and BallTree<D> for the (dims, k) pairs the golden fixtures and
// the CPU baseline use.  The result is oracle/_ref/libknn_ref*.so, which is never committed.
//
// Reference interfaces called:
//   BruteForce<D>(points, n)             src/BruteForce.cuh:20-23;  batchKnn<K,Heap> 27-44
//   KdTree<D>(points, n, depthSkips)     src/KdTree.cuh:56-71;      batchKnn<K,Heap> 146-158
//   BallTree<D>(points, n, depthSkips)   src/BallTree.cuh:123-137;  batchKnn<K,Heap> 225-237
//   Query<D,K>                           src/KnnTrees.cuh:224-231

#include <cstdint>
#include <thread>
#include <vector>

#include "BallTree.cuh"
#include "BruteForce.cuh"
#include "KdTree.cuh"

namespace {

template <uint D, uint K, class Tree>
void run_slices(const Tree& tree, const float* q, uint32_t nq, float max_dist2, int heap,
                int32_t* out_idx, float* out_dist, int threads) {
    using P = KnnTrees::Array<float, D>;
    auto body = [&](uint32_t lo, uint32_t hi) {
        if (hi <= lo) return;
        KnnTrees::Query<D, K> query = {reinterpret_cast<const P*>(q) + lo, hi - lo, max_dist2,
                                       reinterpret_cast<KnnTrees::Array<int, K>*>(out_idx) + lo,
                                       reinterpret_cast<KnnTrees::Array<float, K>*>(out_dist) + lo};
        if (heap)
            tree.template batchKnn<K, true>(query);
        else
            tree.template batchKnn<K, false>(query);
    };
    if (threads <= 1) {
        body(0, nq);
        return;
    }
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; ++i) {
        const uint32_t lo = static_cast<uint32_t>(static_cast<uint64_t>(nq) * i / threads);
        const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(nq) * (i + 1) / threads);
        pool.emplace_back(body, lo, hi);
    }
    for (auto& t : pool) t.join();
}

template <uint D, uint K>
int run(int kind, const float* pts, uint32_t n, const float* q, uint32_t nq, float max_dist2,
        uint32_t skips, int heap, int32_t* out_idx, float* out_dist, int threads) {
    using P = KnnTrees::Array<float, D>;
    const P* p = reinterpret_cast<const P*>(pts);
    if (kind == 0) {
        KnnTrees::BruteForce<D> t(p, n);
        run_slices<D, K>(t, q, nq, max_dist2, heap, out_idx, out_dist, threads);
    } else if (kind == 1) {
        KnnTrees::KdTree<D> t(p, n, skips);
        run_slices<D, K>(t, q, nq, max_dist2, heap, out_idx, out_dist, threads);
    } else {
        KnnTrees::BallTree<D> t(p, n, skips);
        run_slices<D, K>(t, q, nq, max_dist2, heap, out_idx, out_dist, threads);
    }
    return 0;
}

}  // namespace

// (dims, k) pairs instantiated: golden fixtures and the CPU-baseline workloads.
#define KNN_REF_PAIRS(X) \
    X(1, 4)              \
    X(2, 5)              \
    X(3, 1)              \
    X(3, 8)              \
    X(3, 16)             \
    X(4, 10)             \
    X(5, 10)             \
    X(8, 5)              \
    X(8, 10)             \
    X(16, 32)            \
    X(32, 64)            \
    X(128, 100)

extern "C" int ref_knn(int kind, const float* pts, uint32_t n, uint32_t dims, const float* q,
                       uint32_t nq, float max_dist2, uint32_t k, uint32_t skips, int heap,
                       int32_t* out_idx, float* out_dist, int threads) {
#define KNN_REF_CASE(D_, K_)                                                                   \
    if (dims == D_ && k == K_)                                                                 \
        return run<D_, K_>(kind, pts, n, q, nq, max_dist2, skips, heap, out_idx, out_dist, threads);
    KNN_REF_PAIRS(KNN_REF_CASE)
#undef KNN_REF_CASE
    return -1;  // (dims, k) not instantiated
}

extern "C" int ref_has_pair(uint32_t dims, uint32_t k) {
#define KNN_REF_HAS(D_, K_) \
    if (dims == D_ && k == K_) return 1;
    KNN_REF_PAIRS(KNN_REF_HAS)
#undef KNN_REF_HAS
    return 0;
}
