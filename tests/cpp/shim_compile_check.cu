// Compiles every drop-in class and batchKnn form the reference's tests and benchmarks use
// (tests/FunctionalityTests.cu, tests/Dim3SpeedTests.cu, tests/DimXSpeedTests.cu); host code
// only, nothing runs.
#include "KnnTrees/BallTreeGpu.cuh"
#include "KnnTrees/BruteForceGpu.cuh"
#include "KnnTrees/KdTreeGpu.cuh"

void compile_only(const KnnTrees::Array<float, 4>* dp, KnnTrees::Query<4, 10>& q,
                  const KnnTrees::Array<float, 3>* dp3, KnnTrees::Query<3, 16>& q3) {
    KnnTrees::BruteForceGpu<4> bf(dp, 100);
    bf.batchKnn<10, 16, false, false>(q);
    bf.batchKnn<10, 16, true, true>(q);
    KnnTrees::KdTreeGpu<4, 4, 16> kd(dp, 100, 0);
    kd.batchKnn<10, 16, true, false, true>(q);
    KnnTrees::KdTreeGpu<4, 3, 16> kd2(dp, 100, 3);
    kd2.batchKnn<10, 16, false, true, false>(q);
    KnnTrees::BallTreeGpu<4, 16> ball(dp, 100, 0);
    ball.batchKnn<10, 16, true, true, true>(q);
    KnnTrees::KdTreeGpu<3> kd3(dp3, 100);
    kd3.batchKnn<16, 32, false, false, true>(q3);
    KnnTrees::BallTreeGpu<3> b3(dp3, 100);
    b3.batchKnn<16, 16, true, true, true>(q3);
}
