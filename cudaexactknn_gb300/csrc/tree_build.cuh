// Shared machinery of the k-d and ball tree constructions: balanced splitting of point orders.
//
// Both trees split every node of n points into a left child of ceil(n/2) points and a right
// child of floor(n/2) points along one dimension (src/KdTreeGpu.cuh:233-238,
// src/BallTreeGpu.cuh:335-340).  The reference re-sorts all n (node, value) keys with a 64-bit
// radix sort at every level.  Here each dimension's order is sorted once; a node's points then
// occupy the same contiguous segment [off, off+size) of every order, the split is the
// ceil(n/2)-th entry of the split dimension's segment (an O(1) lookup), and one stable
// segmented partition per level moves each other order's entries to the child segments.
//
// Per level: side flags from the split order, then for the other orders
//   count left flags per tile -> exclusive scan of the tile counts (up to kDirectBlocks tiles:
//   each tile sums the counts before it itself) -> per-position prefix G
//   -> scatter to  off + (G[p] - G[off])                   (left child)
//               or off + left + (p - off) - (G[p] - G[off]) (right child).
#pragma once

#include "knn_internal.h"

namespace knn {
namespace build {
namespace {  // each including translation unit gets its own copy

constexpr uint32_t kThreads = 256;
constexpr uint32_t kItems = 8;
constexpr uint32_t kTile = kThreads * kItems;  // positions per partition block
// Up to this many partition blocks per order, each block sums the counts of the blocks before it
// itself (at most kDirectBlocks / kThreads loads a thread) instead of a separate scan launch.
constexpr uint32_t kDirectBlocks = 4096;

// keys[i] = orderable(points[i][dim]), vals[i] = i.
__global__ void extract_keys_kernel(const float* __restrict__ pts, uint32_t n, uint32_t dims, uint32_t dim,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = orderable(pts[static_cast<size_t>(i) * dims + dim]);
    vals[i] = i;
}

// Node tables of the next level from the current one (children 2j, 2j+1).
__global__ void children_kernel(const uint32_t* __restrict__ off, const uint32_t* __restrict__ size,
                                uint32_t count, uint32_t* __restrict__ noff, uint32_t* __restrict__ nsize) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const uint32_t o = off[j], sz = size[j], left = (sz + 1) / 2;
    noff[2 * j] = o;
    nsize[2 * j] = left;
    noff[2 * j + 1] = o + left;
    nsize[2 * j + 1] = sz - left;
}

// Node of every position at the next level.
__global__ void next_node_of_kernel(const uint32_t* __restrict__ node_of, const uint32_t* __restrict__ off,
                                    const uint32_t* __restrict__ size, uint32_t n,
                                    uint32_t* __restrict__ next) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t j = node_of[p];
    next[p] = 2 * j + ((p - off[j]) >= (size[j] + 1) / 2 ? 1u : 0u);
}

// Orders to partition: y-th order of the batch is orders[y] (device pointer table).
struct OrderSet {
    const uint32_t* cur[kMaxDims];
    uint32_t* nxt[kMaxDims];
    uint32_t* g[kMaxDims];      // per-position exclusive prefix of left flags
    uint32_t count;
};

__global__ void __launch_bounds__(kThreads) flag_count_kernel(const OrderSet os, const uint8_t* __restrict__ side,
                                                              uint32_t n, uint32_t nblk,
                                                              uint32_t* __restrict__ bcnt) {
    __shared__ uint32_t warp_tot[kThreads / 32];
    const uint32_t y = blockIdx.y;
    const uint32_t* ord = os.cur[y];
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t c = 0;
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t p = base + i;
        if (p < n) c += side[ord[p]] == 0 ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x / 32] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < kThreads / 32; ++w) t += warp_tot[w];
        bcnt[static_cast<size_t>(y) * nblk + blockIdx.x] = t;
    }
}

// bpre: the exclusive scan of the block counts, or null: the block sums bcnt's entries before it.
__global__ void __launch_bounds__(kThreads) flag_prefix_kernel(const OrderSet os, const uint8_t* __restrict__ side,
                                                               uint32_t n, uint32_t nblk,
                                                               const uint32_t* __restrict__ bpre,
                                                               const uint32_t* __restrict__ bcnt) {
    __shared__ uint32_t warp_tot[kThreads / 32];
    __shared__ uint32_t warp_before[kThreads / 32];
    const uint32_t y = blockIdx.y;
    const uint32_t* ord = os.cur[y];
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t f[kItems];
    uint32_t c = 0;
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t p = base + i;
        f[i] = (p < n && side[ord[p]] == 0) ? 1u : 0u;
        c += f[i];
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x / 32;
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += v;
    }
    if (lane == 31) warp_tot[warp] = incl;
    uint32_t before;
    if (bpre) {
        __syncthreads();
        before = bpre[static_cast<size_t>(y) * nblk + blockIdx.x];
    } else {
        const uint32_t* row = bcnt + static_cast<size_t>(y) * nblk;
        uint32_t part = 0;
        for (uint32_t j = threadIdx.x; j < blockIdx.x; j += kThreads) part += row[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
        if (lane == 0) warp_before[warp] = part;
        __syncthreads();
        before = 0;
#pragma unroll
        for (uint32_t w = 0; w < kThreads / 32; ++w) before += warp_before[w];
    }
    for (uint32_t w = 0; w < warp; ++w) before += warp_tot[w];
    uint32_t run = before + incl - c;
    uint32_t* g = os.g[y];
#pragma unroll
    for (uint32_t i = 0; i < kItems; ++i) {
        const uint32_t p = base + i;
        if (p < n) g[p] = run;
        run += f[i];
    }
}

__global__ void partition_scatter_kernel(const OrderSet os, const uint8_t* __restrict__ side,
                                         const uint32_t* __restrict__ node_of, const uint32_t* __restrict__ off,
                                         const uint32_t* __restrict__ size, uint32_t n) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t y = blockIdx.y;
    const uint32_t id = os.cur[y][p];
    const uint32_t j = node_of[p];
    const uint32_t o = off[j], left = (size[j] + 1) / 2;
    const uint32_t* g = os.g[y];
    const uint32_t lr = g[p] - g[o];
    const uint32_t dst = side[id] == 0 ? o + lr : o + left + (p - o - lr);
    os.nxt[y][dst] = id;
}

// Device scratch of a balanced construction over `n_orders` dimension orders.
struct Scratch {
    uint32_t* ord[2][kMaxDims];
    uint32_t* g[kMaxDims];
    uint32_t* node_of[2];
    uint32_t* off[2];
    uint32_t* size[2];
    uint8_t* side;
    uint32_t* bcnt;
    uint32_t* bpre;
    uint32_t* sort_keys[2];
    uint32_t* sort_vals;
    void* sort_temp;
    uint32_t nblk;
};

inline size_t scratch_bytes(uint32_t n, uint32_t n_orders, uint32_t max_level_nodes) {
    const size_t nb = (n + kTile - 1) / kTile;
    const size_t w = static_cast<size_t>(n) * sizeof(uint32_t);
    size_t total = 0;
    auto add = [&](size_t b) { total += ((b + 255) / 256) * 256 + 256; };
    for (uint32_t i = 0; i < n_orders; ++i) {
        add(w);
        add(w);
        add(w);
    }
    add(w);
    add(w);
    for (int i = 0; i < 4; ++i) add(static_cast<size_t>(max_level_nodes) * sizeof(uint32_t));
    add(n);
    add(nb * n_orders * sizeof(uint32_t));
    add(nb * n_orders * sizeof(uint32_t));
    add(w);
    add(w);
    add(w);
    add(radix_sort_temp_bytes(n));
    return total + 4096;
}

inline void carve_scratch(Scratch& sc, void* base, uint32_t n, uint32_t n_orders, uint32_t max_level_nodes) {
    Carver c(base);
    for (uint32_t i = 0; i < n_orders; ++i) {
        sc.ord[0][i] = c.take<uint32_t>(n);
        sc.ord[1][i] = c.take<uint32_t>(n);
        sc.g[i] = c.take<uint32_t>(n);
    }
    sc.node_of[0] = c.take<uint32_t>(n);
    sc.node_of[1] = c.take<uint32_t>(n);
    sc.off[0] = c.take<uint32_t>(max_level_nodes);
    sc.off[1] = c.take<uint32_t>(max_level_nodes);
    sc.size[0] = c.take<uint32_t>(max_level_nodes);
    sc.size[1] = c.take<uint32_t>(max_level_nodes);
    sc.side = c.take<uint8_t>(n);
    sc.nblk = (n + kTile - 1) / kTile;
    sc.bcnt = c.take<uint32_t>(static_cast<size_t>(sc.nblk) * n_orders);
    sc.bpre = c.take<uint32_t>(static_cast<size_t>(sc.nblk) * n_orders);
    sc.sort_keys[0] = c.take<uint32_t>(n);
    sc.sort_keys[1] = c.take<uint32_t>(n);
    sc.sort_vals = c.take<uint32_t>(n);
    sc.sort_temp = c.take<uint8_t>(radix_sort_temp_bytes(n));
}

// Sorts point ids by dimension `dim` into sc.ord[0][slot].
inline int sort_dimension(Scratch& sc, const float* pts, uint32_t n, uint32_t dims, uint32_t dim, uint32_t slot,
                          cudaStream_t s) {
    uint32_t* out = sc.ord[0][slot];
    extract_keys_kernel<<<ceil_div(n, 256), 256, 0, s>>>(pts, n, dims, dim, sc.sort_keys[0], out);
    KNN_LAUNCHED();
    bool in_alt = false;
    KNN_TRY(radix_sort_pairs(sc.sort_keys[0], out, sc.sort_keys[1], sc.sort_vals, n, 32, sc.sort_temp, s, &in_alt));
    if (in_alt) KNN_TRY_CUDA(cudaMemcpyAsync(out, sc.sort_vals, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    return KNN_OK;
}

// Stable segmented partition of the orders listed in `which` (slots), from ord[cur] to
// ord[cur^1], using sc.side and the level's node of each position and node tables.
inline int partition_orders(Scratch& sc, const uint32_t* which, uint32_t count, int cur, const uint32_t* node_of,
                            const uint32_t* off, const uint32_t* size, uint32_t n, cudaStream_t s) {
    if (count == 0) return KNN_OK;
    OrderSet os{};
    os.count = count;
    for (uint32_t y = 0; y < count; ++y) {
        os.cur[y] = sc.ord[cur][which[y]];
        os.nxt[y] = sc.ord[cur ^ 1][which[y]];
        os.g[y] = sc.g[which[y]];
    }
    dim3 gb(sc.nblk, count);
    flag_count_kernel<<<gb, kThreads, 0, s>>>(os, sc.side, n, sc.nblk, sc.bcnt);
    KNN_LAUNCHED();
    const bool direct = sc.nblk <= kDirectBlocks;
    if (!direct) KNN_TRY(scan_rows_exclusive(sc.bcnt, sc.bpre, count, sc.nblk, s));
    flag_prefix_kernel<<<gb, kThreads, 0, s>>>(os, sc.side, n, sc.nblk, direct ? nullptr : sc.bpre, sc.bcnt);
    KNN_LAUNCHED();
    dim3 gp(ceil_div(n, 256), count);
    partition_scatter_kernel<<<gp, 256, 0, s>>>(os, sc.side, node_of, off, size, n);
    KNN_LAUNCHED();
    return KNN_OK;
}

}  // namespace
}  // namespace build
}  // namespace knn
