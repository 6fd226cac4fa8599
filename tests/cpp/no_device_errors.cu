// Host program for the CPU tests: with no usable CUDA device, the drop-in classes must report
// the runtime's failure as KnnTrees::CudaException (the reference's error type,
// src/KnnTrees.cuh:20-23) rather than crash or return a half-built object.  Prints one line
// per class: "<class> threw: <message>".  Exit code 0 only if all three threw.

#include <cstdio>

#include "KnnTrees/BallTreeGpu.cuh"
#include "KnnTrees/BruteForceGpu.cuh"
#include "KnnTrees/KdTreeGpu.cuh"

template <class Make>
static int expect_throw(const char* name, Make make) {
    try {
        make();
    } catch (const KnnTrees::CudaException& e) {
        std::printf("%s threw: %s\n", name, e.what());
        return 1;
    }
    std::printf("%s did not throw\n", name);
    return 0;
}

int main() {
    // A non-null stand-in for a device pointer: with no device, nothing may dereference it.
    const auto* points = reinterpret_cast<const KnnTrees::Array<float, 3>*>(static_cast<uintptr_t>(0x1000));
    int thrown = 0;
    thrown += expect_throw("BruteForceGpu", [&] { KnnTrees::BruteForceGpu<3> t(points, 100); });
    thrown += expect_throw("KdTreeGpu", [&] { KnnTrees::KdTreeGpu<3> t(points, 100, 0); });
    thrown += expect_throw("BallTreeGpu", [&] { KnnTrees::BallTreeGpu<3> t(points, 100, 1); });
    return thrown == 3 ? 0 : 1;
}
