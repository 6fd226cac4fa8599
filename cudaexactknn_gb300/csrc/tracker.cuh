// Top-k tracker selection for the query kernels: the run-time form of the reference's
// USE_HEAP_TRACKING / USE_TRACKING_SHMEM template switches (src/BruteForceGpu.cuh:42-50,
// src/KdTreeGpu.cuh:92-184).
//
//   HEAP  SHNN  storage
//   no    no    registers, sorted insertion (KMAX <= 32); thread-local array above that
//   no    yes   shared memory, sorted insertion, slot-major (slot i of thread t at i*block+t)
//   yes   no    thread-local array, max-heap
//   yes   yes   shared memory, max-heap
//
// The k-th key is cached in a register, so a rejected candidate costs one 64-bit compare.
#pragma once

#include <type_traits>

#include "knn_common.cuh"

namespace knn {

template <int KMAX, bool HEAP, bool SHNN>
struct Tracker {
    static constexpr bool kReg = !HEAP && !SHNN && KMAX <= 32;
    static constexpr int kLocal = (kReg || SHNN) ? 1 : KMAX;
    using Mem = typename std::conditional<HEAP, MemHeap, MemSorted>::type;

    RegSorted<kReg ? KMAX : 1> reg;
    Mem mem;
    uint64_t local[kLocal];
    uint64_t kth;

    __device__ __forceinline__ void init(uint32_t k, float r2, uint64_t* sh_base, uint32_t sh_stride) {
        const uint64_t fill = make_key(r2, -1);
        if constexpr (kReg) {
            reg.init(k, fill);
        } else {
            if constexpr (SHNN) {
                mem.base = sh_base;
                mem.stride = sh_stride;
            } else {
                mem.base = local;
                mem.stride = 1;
            }
            mem.init(k, fill);
        }
        kth = fill;
    }

    __device__ __forceinline__ float radius() const { return key_dist(kth); }

    // Offers a candidate; returns true when it was accepted.
    __device__ __forceinline__ bool offer(uint64_t key) {
        if (key >= kth) return false;
        if constexpr (kReg) {
            reg.insert(key);
            kth = reg.kth();
        } else {
            mem.insert(key);
            kth = mem.kth();
        }
        return true;
    }

    __device__ __forceinline__ void emit(uint32_t k, int32_t* idx, float* dist) {
        if constexpr (kReg)
            reg.emit(k, idx, dist);
        else
            mem.emit(k, idx, dist);
    }

    __device__ __forceinline__ void emit_keys(uint32_t k, uint64_t* out) {
        if constexpr (kReg)
            reg.emit_keys(k, out);
        else
            mem.emit_keys(k, out);
    }
};

// Shared-memory bytes a block needs for SHNN tracking.
__host__ __device__ constexpr size_t tracker_smem_bytes(bool shnn, uint32_t kmax, uint32_t block) {
    return shnn ? static_cast<size_t>(kmax) * block * sizeof(uint64_t) : 0;
}

}  // namespace knn
