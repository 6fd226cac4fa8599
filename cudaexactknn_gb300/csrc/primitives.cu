// Device primitives used by construction and query preparation: a stable LSD radix sort of
// (u32 key, u32 value) pairs, per-row exclusive scans of block counts, and empty-result rows.
//
// The reference sorts with cub::DeviceRadixSort and scans with cub::DeviceScan
// (src/KdTreeGpu.cuh:313-320, src/BallTreeGpu.cuh:500-505); the engine uses these instead.

#include <atomic>
#include "knn_internal.h"

namespace knn {

namespace {

constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortWarps = kSortThreads / 32;
constexpr uint32_t kSortItemsPerWarp = 512;
constexpr uint32_t kSortTile = kSortWarps * kSortItemsPerWarp;  // 4096 keys per block

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Per-block digit histogram, written digit-major: counts[digit * nblocks + block].
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint32_t* __restrict__ keys,
                                                                  uint32_t n, uint32_t shift,
                                                                  uint32_t* __restrict__ counts,
                                                                  uint32_t nblocks) {
    __shared__ uint32_t h[kSortWarps][256];
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (uint32_t i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kSortTile + warp * kSortItemsPerWarp;
    for (uint32_t it = 0; it < kSortItemsPerWarp; it += 32) {
        const uint64_t idx = base + it + lane;
        const bool valid = idx < n;
        const uint32_t digit = valid ? (keys[idx] >> shift) & 255u : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) h[warp][digit] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    uint32_t total = 0;
#pragma unroll
    for (uint32_t w = 0; w < kSortWarps; ++w) total += h[w][threadIdx.x];
    counts[static_cast<size_t>(threadIdx.x) * nblocks + blockIdx.x] = total;
}

// Stable scatter: each warp owns a contiguous sub-tile and walks it in order, so equal digits
// keep their input order.  offsets[d * nblocks + b] is the exclusive prefix of digit d's counts
// over the blocks before b; each block adds the keys of all smaller digits, from the rows' totals
// (a scan of 256 values per block instead of one serial scan of 256 x nblocks).
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n, uint32_t shift,
    const uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets, uint32_t nblocks,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out) {
    __shared__ uint32_t h[kSortWarps][256];
    __shared__ uint32_t digit_sums[kSortWarps];
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (uint32_t i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kSortTile + warp * kSortItemsPerWarp;
    for (uint32_t it = 0; it < kSortItemsPerWarp; it += 32) {
        const uint64_t idx = base + it + lane;
        const bool valid = idx < n;
        const uint32_t digit = valid ? (keys[idx] >> shift) & 255u : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) h[warp][digit] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const uint32_t d = threadIdx.x;  // one digit per thread (256 threads)
        const size_t last = static_cast<size_t>(d) * nblocks + nblocks - 1;
        const uint32_t total = offsets[last] + counts[last];  // keys of digit d in the whole pass
        uint32_t incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += v;
        }
        if (lane == 31) digit_sums[warp] = incl;
        __syncthreads();
        uint32_t below = incl - total;  // smaller digits in this warp
        for (uint32_t w = 0; w < warp; ++w) below += digit_sums[w];
        uint32_t run = below + offsets[static_cast<size_t>(d) * nblocks + blockIdx.x];
#pragma unroll
        for (uint32_t w = 0; w < kSortWarps; ++w) {
            const uint32_t c = h[w][d];
            h[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    const uint32_t lt = lanemask_lt();
    for (uint32_t it = 0; it < kSortItemsPerWarp; it += 32) {
        const uint64_t idx = base + it + lane;
        const bool valid = idx < n;
        const uint32_t key = valid ? keys[idx] : 0u;
        const uint32_t digit = valid ? (key >> shift) & 255u : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t pos = 0;
        if (valid) pos = h[warp][digit] + __popc(peers & lt);
        __syncwarp();
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) h[warp][digit] += __popc(peers);
        __syncwarp();
        if (valid) {
            keys_out[pos] = key;
            vals_out[pos] = vals[idx];
        }
    }
}

// Exclusive scan of each row of a [rows][cols] u32 matrix; one block of 1024 threads per row.
// The row streams through shared memory in coalesced tiles of 4096 entries with a running carry.
__global__ void __launch_bounds__(1024) scan_rows_kernel(const uint32_t* __restrict__ in,
                                                         uint32_t* __restrict__ out, uint32_t cols) {
    constexpr uint32_t kT = 1024, kTile = 4 * kT;
    __shared__ uint32_t tile[kTile];
    __shared__ uint32_t warp_sums[32];
    const uint32_t* row_in = in + static_cast<size_t>(blockIdx.x) * cols;
    uint32_t* row_out = out + static_cast<size_t>(blockIdx.x) * cols;
    const uint32_t tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < cols; base += kTile) {
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
            const uint32_t idx = base + i * kT + tid;
            tile[i * kT + tid] = idx < cols ? row_in[idx] : 0u;
        }
        __syncthreads();
        const uint32_t a = tile[4 * tid], b = tile[4 * tid + 1], c = tile[4 * tid + 2], d = tile[4 * tid + 3];
        const uint32_t sum = a + b + c + d;
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += v;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= static_cast<uint32_t>(o)) w += v;
            }
            warp_sums[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t excl = carry + incl - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
        tile[4 * tid] = excl;
        tile[4 * tid + 1] = excl + a;
        tile[4 * tid + 2] = excl + a + b;
        tile[4 * tid + 3] = excl + a + b + c;
        const uint32_t tile_total = warp_sums[31];
        __syncthreads();
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
            const uint32_t idx = base + i * kT + tid;
            if (idx < cols) row_out[idx] = tile[i * kT + tid];
        }
        carry += tile_total;
        __syncthreads();
    }
}

__global__ void fill_rows_kernel(uint32_t count, uint32_t k, float max_d2, const float* __restrict__ radii,
                                 int32_t* __restrict__ idx, float* __restrict__ dist) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<uint64_t>(count) * k) return;
    idx[i] = -1;
    dist[i] = radii ? radii[i / k] : max_d2;
}

// dst[i] = src row idx[i'] (rows of `dims` floats), and the per-row radius when given, where
// i' = i, or, with stride > 1, the i%32-th entry of the (i/32 * stride)-th run of 32 entries.
__global__ void gather_rows_kernel(const float* __restrict__ src, const float* __restrict__ src_r,
                                   const uint32_t* __restrict__ idx, uint32_t count, uint32_t dims, uint32_t stride,
                                   float* __restrict__ dst, float* __restrict__ dst_r) {
    const uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= static_cast<uint64_t>(count) * dims) return;
    const uint32_t i = static_cast<uint32_t>(e / dims), d = static_cast<uint32_t>(e % dims);
    const uint32_t j = idx[stride > 1 ? (i / 32) * 32 * stride + i % 32 : i];
    dst[e] = src[static_cast<size_t>(j) * dims + d];
    if (src_r && d == 0) dst_r[i] = src_r[j];
}

}  // namespace

int gather_rows(const float* src, const float* src_radii, const uint32_t* idx, uint32_t count, uint32_t dims,
                uint32_t stride, float* dst, float* dst_radii, cudaStream_t s) {
    if (!count) return KNN_OK;
    const uint64_t total = static_cast<uint64_t>(count) * dims;
    gather_rows_kernel<<<static_cast<uint32_t>((total + 255) / 256), 256, 0, s>>>(src, src_radii, idx, count, dims,
                                                                                stride, dst, dst_radii);
    KNN_LAUNCHED();
    return KNN_OK;
}

size_t radix_sort_temp_bytes(uint32_t n) {
    const size_t nblocks = (static_cast<size_t>(n) + kSortTile - 1) / kSortTile;
    return 2 * 256 * nblocks * sizeof(uint32_t) + 512;
}

int radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt,
                     uint32_t n, int key_bits, void* temp, cudaStream_t s, bool* in_alt) {
    *in_alt = false;
    if (n <= 1 || key_bits <= 0) return KNN_OK;
    const uint32_t nblocks = (n + kSortTile - 1) / kSortTile;
    uint32_t* counts = static_cast<uint32_t*>(temp);
    uint32_t* offsets = counts + 256 * static_cast<size_t>(nblocks);
    uint32_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
    for (int shift = 0; shift < key_bits; shift += 8) {
        radix_hist_kernel<<<nblocks, kSortThreads, 0, s>>>(ki, n, shift, counts, nblocks);
        scan_rows_kernel<<<256, 1024, 0, s>>>(counts, offsets, nblocks);  // one row per digit
        radix_scatter_kernel<<<nblocks, kSortThreads, 0, s>>>(ki, vi, n, shift, counts, offsets, nblocks, ko, vo);
        KNN_LAUNCHED_N(3);
        uint32_t* t = ki;
        ki = ko;
        ko = t;
        t = vi;
        vi = vo;
        vo = t;
        *in_alt = !*in_alt;
    }
    return KNN_OK;
}

int scan_rows_exclusive(const uint32_t* counts, uint32_t* out, uint32_t rows, uint32_t cols,
                        cudaStream_t s) {
    if (rows == 0 || cols == 0) return KNN_OK;
    scan_rows_kernel<<<rows, 1024, 0, s>>>(counts, out, cols);
    KNN_LAUNCHED();
    return KNN_OK;
}

int fill_empty_rows(const QueryArgs& a, cudaStream_t s) {
    const uint64_t total = static_cast<uint64_t>(a.count) * a.k;
    if (total == 0) return KNN_OK;
    const uint32_t blocks = static_cast<uint32_t>((total + 255) / 256);
    fill_rows_kernel<<<blocks, 256, 0, s>>>(a.count, a.k, a.max_d2, a.radii, a.out_idx, a.out_dist);
    KNN_LAUNCHED();
    return KNN_OK;
}

int sm_count() {
    // Cached per device ordinal: a process may query indexes on GPUs of different sizes.
    constexpr int kDevices = 64;
    static std::atomic<int> cached[kDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    const int slot = dev >= 0 && dev < kDevices ? dev : 0;
    int v = cached[slot].load(std::memory_order_relaxed);
    if (v == 0) {
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        v = v > 0 ? v : 1;
        cached[slot].store(v, std::memory_order_relaxed);
    }
    return v;
}

}  // namespace knn
