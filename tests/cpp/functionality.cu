// The reference's correctness test (tests/FunctionalityTests.cu) restated against the drop-in
// headers, with seeded inputs and a stricter check: every variant's rows must equal a CPU brute
// force (fused-multiply-add distance, key order) exactly, not just as index sets.
//
// Build (tests/test_cpp_functionality.py does this):
//   nvcc -std=c++17 -gencode arch=compute_103a,code=sm_103a -I<repo>/include \
//        tests/cpp/functionality.cu -L<repo>/cudaexactknn_gb300 -lcudaexactknn
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "KnnTrees/BallTreeGpu.cuh"
#include "KnnTrees/BruteForceGpu.cuh"
#include "KnnTrees/KdTreeGpu.cuh"

namespace {

constexpr uint kDims = 4;
constexpr uint kPoints = 100000;
constexpr uint kQueries = 50000;
constexpr uint kK = 10;
constexpr uint kChecked = 2000;  // queries checked against the CPU brute force
using P = KnnTrees::Array<float, kDims>;

uint64_t key(float d, int i) {
    uint32_t b;
    std::memcpy(&b, &d, 4);
    return (static_cast<uint64_t>(b) << 32) | static_cast<uint32_t>(i);
}

std::vector<uint64_t> cpu_truth(const std::vector<P>& pts, const std::vector<P>& qs, float r2) {
    std::vector<uint64_t> out(static_cast<size_t>(kChecked) * kK);
    std::vector<uint64_t> best(kK);
    for (uint q = 0; q < kChecked; ++q) {
        std::fill(best.begin(), best.end(), key(r2, -1));
        for (uint i = 0; i < kPoints; ++i) {
            float acc = 0.0f;
            for (uint d = 0; d < kDims; ++d) {
                const float t = qs[q][d] - pts[i][d];
                acc = std::fma(t, t, acc);
            }
            KnnTrees::arrayConsider<kK>(best.data(), static_cast<int>(i), acc);
        }
        std::copy(best.begin(), best.end(), out.begin() + static_cast<size_t>(q) * kK);
    }
    return out;
}

int check(const char* what, KnnTrees::Query<kDims, kK>& dq, const std::vector<uint64_t>& truth) {
    std::vector<int> idx(static_cast<size_t>(kQueries) * kK);
    std::vector<float> dist(idx.size());
    KnnTrees::Cuda::check(cudaMemcpy(idx.data(), dq.rIndexes, idx.size() * 4, KnnTrees::Cuda::D2H));
    KnnTrees::Cuda::check(cudaMemcpy(dist.data(), dq.rDistances, dist.size() * 4, KnnTrees::Cuda::D2H));
    uint bad = 0;
    for (uint q = 0; q < kChecked; ++q)
        for (uint j = 0; j < kK; ++j)
            if (key(dist[q * kK + j], idx[q * kK + j]) != truth[q * kK + j]) {
                ++bad;
                break;
            }
    std::printf("%-44s %s (%u of %u rows differ)\n", what, bad ? "FAIL" : "ok", bad, kChecked);
    cudaMemset(dq.rIndexes, 0xff, idx.size() * 4);
    return bad ? 1 : 0;
}

}  // namespace

int main() {
    std::mt19937 gen(1000);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    std::vector<P> pts(kPoints), qs(kQueries);
    for (auto& p : pts)
        for (uint d = 0; d < kDims; ++d) p[d] = u(gen);
    for (auto& q : qs)
        for (uint d = 0; d < kDims; ++d) q[d] = u(gen);
    const float r2 = 5.9f;
    const auto truth = cpu_truth(pts, qs, r2);

    P *d_pts, *d_qs;
    KnnTrees::Cuda::check(cudaMalloc(&d_pts, sizeof(P) * kPoints));
    KnnTrees::Cuda::check(cudaMalloc(&d_qs, sizeof(P) * kQueries));
    KnnTrees::Cuda::check(cudaMemcpy(d_pts, pts.data(), sizeof(P) * kPoints, KnnTrees::Cuda::H2D));
    KnnTrees::Cuda::check(cudaMemcpy(d_qs, qs.data(), sizeof(P) * kQueries, KnnTrees::Cuda::H2D));
    KnnTrees::Query<kDims, kK> dq = {d_qs, kQueries, r2, nullptr, nullptr};
    KnnTrees::Cuda::check(cudaMalloc(&dq.rIndexes, sizeof(KnnTrees::Array<int, kK>) * kQueries));
    KnnTrees::Cuda::check(cudaMalloc(&dq.rDistances, sizeof(KnnTrees::Array<float, kK>) * kQueries));

    int fails = 0;
    KnnTrees::BruteForceGpu<kDims> bfg(d_pts, kPoints);
    bfg.batchKnn<kK, 16, false, false>(dq);
    fails += check("BruteForceGpu<16,array,regs>", dq, truth);
    bfg.batchKnn<kK, 16, true, false>(dq);
    fails += check("BruteForceGpu<16,heap,regs>", dq, truth);
    bfg.batchKnn<kK, 16, false, true>(dq);
    fails += check("BruteForceGpu<16,array,shared>", dq, truth);

    KnnTrees::KdTreeGpu<kDims, kDims, 16> kdg(d_pts, kPoints, 0);
    kdg.batchKnn<kK, 16, true, false, true>(dq);
    fails += check("KdTreeGpu<4,4,16> skips 0 <heap,regs,shared stack>", dq, truth);
    KnnTrees::KdTreeGpu<kDims, 3, 16> kdg2(d_pts, kPoints, 3);
    kdg2.batchKnn<kK, 16, false, true, false>(dq);
    fails += check("KdTreeGpu<4,3,16> skips 3 <array,shared,local>", dq, truth);

    KnnTrees::BallTreeGpu<kDims, 16> ballg(d_pts, kPoints, 0);
    ballg.batchKnn<kK, 16, true, true, true>(dq);
    fails += check("BallTreeGpu<4,16> skips 0 <heap,shared,shared>", dq, truth);
    KnnTrees::BallTreeGpu<kDims, 16> ballg2(d_pts, kPoints, 2);
    ballg2.batchKnn<kK, 16, false, false, false>(dq);
    fails += check("BallTreeGpu<4,16> skips 2 <array,regs,local>", dq, truth);

    // Errors surface as KnnTrees::CudaException, as in the reference.
    bool threw = false;
    try {
        KnnTrees::Query<kDims, kK> bad = {d_qs, kQueries, -1.0f, dq.rIndexes, dq.rDistances};
        kdg.batchKnn<kK, 16, false, false, false>(bad);
    } catch (const KnnTrees::CudaException& e) {
        threw = true;
        std::printf("negative radius rejected: %s\n", e.what());
    }
    fails += threw ? 0 : 1;

    cudaFree(dq.rIndexes);
    cudaFree(dq.rDistances);
    cudaFree(d_pts);
    cudaFree(d_qs);
    if (fails) {
        std::printf("%d checks failed\n", fails);
        return 1;
    }
    std::printf("All tests passed\n");
    return 0;
}
