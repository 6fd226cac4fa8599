// Device-side building blocks shared by every kNN kernel of the engine.
//
// Semantics restated from the reference (src/KnnTrees.cuh):
//   * squared distance = sequential sum over dimensions of (a[d]-b[d])^2, one fused
//     multiply-add per dimension in dimension order (src/KnnTrees.cuh:65-77 as nvcc compiles it:
//     `result += difference * difference` contracts to fma(difference, difference, result));
//   * result key = (bits(dist2) << 32) | uint32(index), compared as u64: smaller distance wins,
//     equal distances go to the smaller index (src/KnnTrees.cuh:122-128);
//   * every slot starts as key(maxDistance2, -1), so a point with dist2 == maxDistance2 and
//     index < 0xFFFFFFFF is accepted and unfilled slots come back as (-1, maxDistance2)
//     (src/BruteForceGpu.cuh:17).
// Rows are always returned in ascending key order (the reference's heap tracking returns
// heap order; the set is the same).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace knn {

constexpr uint32_t kMaxTreeDepth = 32;  // N < 2^32 gives at most 32 node levels

__host__ __device__ __forceinline__ uint32_t float_as_u32(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    union {
        float f;
        uint32_t u;
    } c{f};
    return c.u;
#endif
}

__host__ __device__ __forceinline__ float u32_as_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    union {
        uint32_t u;
        float f;
    } c{u};
    return c.f;
#endif
}

__host__ __device__ __forceinline__ uint64_t make_key(float d2, int32_t index) {
    return (static_cast<uint64_t>(float_as_u32(d2)) << 32) | static_cast<uint32_t>(index);
}

__host__ __device__ __forceinline__ float key_dist(uint64_t key) {
    return u32_as_float(static_cast<uint32_t>(key >> 32));
}

__host__ __device__ __forceinline__ int32_t key_index(uint64_t key) {
    return static_cast<int32_t>(static_cast<uint32_t>(key));
}

// Order-preserving map of a float to u32 (negative values reversed, sign bit flipped).
__host__ __device__ __forceinline__ uint32_t orderable(float f) {
    const uint32_t u = float_as_u32(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Squared distance with one rounding per dimension step, in dimension order.  DP is the padded
// dimension count; padded coordinates are zero on both sides and add exactly 0.
template <int DP>
__device__ __forceinline__ float dist2(const float (&q)[DP], const float* __restrict__ p) {
    float acc = 0.0f;
#pragma unroll
    for (int d = 0; d < DP; ++d) {
        const float t = __fsub_rn(q[d], p[d]);
        acc = __fmaf_rn(t, t, acc);
    }
    return acc;
}

template <int DP>
__device__ __forceinline__ float dist2_vec4(const float (&q)[DP], const float4* __restrict__ p4) {
    static_assert(DP % 4 == 0, "vector path needs DP % 4 == 0");
    float acc = 0.0f;
#pragma unroll
    for (int v = 0; v < DP / 4; ++v) {
        const float4 p = p4[v];
        float t = __fsub_rn(q[4 * v + 0], p.x);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q[4 * v + 1], p.y);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q[4 * v + 2], p.z);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q[4 * v + 3], p.w);
        acc = __fmaf_rn(t, t, acc);
    }
    return acc;
}

// Two rows at once: each distance is the same sequential fused sum as dist2_vec4 (identical
// results), the two chains interleaved for instruction-level parallelism.
template <int DP>
__device__ __forceinline__ void dist2_vec4_pair(const float (&q)[DP], const float4* __restrict__ pa,
                                                const float4* __restrict__ pb, float* da, float* db) {
    static_assert(DP % 4 == 0, "vector path needs DP % 4 == 0");
    float acc_a = 0.0f, acc_b = 0.0f;
#pragma unroll
    for (int v = 0; v < DP / 4; ++v) {
        const float4 x = pa[v], y = pb[v];
        float t = __fsub_rn(q[4 * v + 0], x.x), u = __fsub_rn(q[4 * v + 0], y.x);
        acc_a = __fmaf_rn(t, t, acc_a);
        acc_b = __fmaf_rn(u, u, acc_b);
        t = __fsub_rn(q[4 * v + 1], x.y);
        u = __fsub_rn(q[4 * v + 1], y.y);
        acc_a = __fmaf_rn(t, t, acc_a);
        acc_b = __fmaf_rn(u, u, acc_b);
        t = __fsub_rn(q[4 * v + 2], x.z);
        u = __fsub_rn(q[4 * v + 2], y.z);
        acc_a = __fmaf_rn(t, t, acc_a);
        acc_b = __fmaf_rn(u, u, acc_b);
        t = __fsub_rn(q[4 * v + 3], x.w);
        u = __fsub_rn(q[4 * v + 3], y.w);
        acc_a = __fmaf_rn(t, t, acc_a);
        acc_b = __fmaf_rn(u, u, acc_b);
    }
    *da = acc_a;
    *db = acc_b;
}

// Select q[dim] from a register array without dynamic indexing (which would force the array
// into local memory).
template <int DP>
__device__ __forceinline__ float pick(const float (&q)[DP], uint32_t dim) {
    float v = q[0];
#pragma unroll
    for (int d = 1; d < DP; ++d) v = (dim == static_cast<uint32_t>(d)) ? q[d] : v;
    return v;
}

// ---------------------------------------------------------------------------------------------
// Top-k trackers.  All keep the k smallest keys seen and expose the k-th key, which is the
// pruning radius of the tree searches.
// ---------------------------------------------------------------------------------------------

// Sorted insertion held in registers.  KMAX slots, run-time k <= KMAX: the first KMAX-k slots
// hold key 0 (below every real key) and never move, so the k real slots are the last k and
// the k-th key is always slot KMAX-1.  An accepted key bubbles through every slot with a
// min/max pair, which keeps the indexing static (src/KnnTrees.cuh:136-152 does the same
// bubble over K slots).
template <int KMAX>
struct RegSorted {
    uint64_t s[KMAX];

    __device__ __forceinline__ void init(uint32_t k, uint64_t fill) {
#pragma unroll
        for (int i = 0; i < KMAX; ++i) s[i] = (static_cast<uint32_t>(i) + k < KMAX) ? 0ull : fill;
    }
    __device__ __forceinline__ uint64_t kth() const { return s[KMAX - 1]; }
    __device__ __forceinline__ void insert(uint64_t x) {
#pragma unroll
        for (int i = 0; i < KMAX; ++i) {
            const uint64_t c = s[i];
            s[i] = c < x ? c : x;
            x = c < x ? x : c;
        }
    }
    __device__ __forceinline__ void emit(uint32_t k, int32_t* __restrict__ idx,
                                         float* __restrict__ dist) const {
#pragma unroll
        for (int i = 0; i < KMAX; ++i) {
            if (static_cast<uint32_t>(i) + k >= KMAX) {
                const uint32_t o = static_cast<uint32_t>(i) + k - KMAX;
                idx[o] = key_index(s[i]);
                dist[o] = key_dist(s[i]);
            }
        }
    }
    __device__ __forceinline__ void emit_keys(uint32_t k, uint64_t* __restrict__ out) const {
#pragma unroll
        for (int i = 0; i < KMAX; ++i)
            if (static_cast<uint32_t>(i) + k >= KMAX) out[static_cast<uint32_t>(i) + k - KMAX] = s[i];
    }
};

// Sorted insertion in memory (shared memory laid out slot-major so that a warp's threads hit
// distinct banks, or a thread's local array with stride 1).  Insertion shifts larger keys up
// by one and stops at the first smaller key.
struct MemSorted {
    uint64_t* base;
    uint32_t stride;
    uint32_t k;

    __device__ __forceinline__ uint64_t& at(uint32_t i) const { return base[static_cast<size_t>(i) * stride]; }
    __device__ __forceinline__ void init(uint32_t k_, uint64_t fill) {
        k = k_;
        for (uint32_t i = 0; i < k; ++i) at(i) = fill;
    }
    __device__ __forceinline__ uint64_t kth() const { return at(k - 1); }
    __device__ __forceinline__ void insert(uint64_t x) {
        uint32_t i = k - 1;
        while (i > 0) {
            const uint64_t prev = at(i - 1);
            if (prev <= x) break;
            at(i) = prev;
            --i;
        }
        at(i) = x;
    }
    __device__ __forceinline__ void emit(uint32_t, int32_t* __restrict__ idx, float* __restrict__ dist) const {
        for (uint32_t i = 0; i < k; ++i) {
            const uint64_t v = at(i);
            idx[i] = key_index(v);
            dist[i] = key_dist(v);
        }
    }
    __device__ __forceinline__ void emit_keys(uint32_t, uint64_t* __restrict__ out) const {
        for (uint32_t i = 0; i < k; ++i) out[i] = at(i);
    }
};

// Max-heap in memory, root at slot 0 (src/KnnTrees.cuh:154-189 keeps the same heap; this one
// never reads past slot k-1).  emit() heap-sorts the slots in place so rows come out ascending.
struct MemHeap {
    uint64_t* base;
    uint32_t stride;
    uint32_t k;

    __device__ __forceinline__ uint64_t& at(uint32_t i) const { return base[static_cast<size_t>(i) * stride]; }
    __device__ __forceinline__ void init(uint32_t k_, uint64_t fill) {
        k = k_;
        for (uint32_t i = 0; i < k; ++i) at(i) = fill;
    }
    __device__ __forceinline__ uint64_t kth() const { return at(0); }
    __device__ __forceinline__ void sift(uint64_t x, uint32_t n) {
        uint32_t pos = 0;
        for (;;) {
            const uint32_t l = 2 * pos + 1;
            if (l >= n) break;
            uint32_t big = l;
            uint64_t bv = at(l);
            if (l + 1 < n) {
                const uint64_t rv = at(l + 1);
                if (rv > bv) {
                    big = l + 1;
                    bv = rv;
                }
            }
            if (bv <= x) break;
            at(pos) = bv;
            pos = big;
        }
        at(pos) = x;
    }
    __device__ __forceinline__ void insert(uint64_t x) { sift(x, k); }
    __device__ __forceinline__ void sort_ascending() {
        for (uint32_t n = k; n > 1; --n) {
            const uint64_t top = at(0);
            const uint64_t last = at(n - 1);
            at(n - 1) = top;
            sift(last, n - 1);
        }
    }
    __device__ __forceinline__ void emit(uint32_t, int32_t* __restrict__ idx, float* __restrict__ dist) {
        sort_ascending();
        for (uint32_t i = 0; i < k; ++i) {
            const uint64_t v = at(i);
            idx[i] = key_index(v);
            dist[i] = key_dist(v);
        }
    }
    __device__ __forceinline__ void emit_keys(uint32_t, uint64_t* __restrict__ out) {
        sort_ascending();
        for (uint32_t i = 0; i < k; ++i) out[i] = at(i);
    }
};

// ---------------------------------------------------------------------------------------------
// Rigorous pruning bounds.  u = 2^-24 is float's unit roundoff.  For the dist2 above, with
// every term non-negative, the float result s and the exact value S of sum (a[d]-b[d])^2 over
// D dimensions satisfy  S (1 - (D+2)u) <= s <= S (1 + (D+2)u)  to first order; the margins
// below use (D+4) * 2u, twice that.
// ---------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ float rel_margin(uint32_t dims) {
    return static_cast<float>(dims + 4) * 1.1920928955078125e-07f;  // (D+4) * 2^-23
}

// Lower bound on the float dist2 from q to any point inside the ball (centre c, radius r),
// where r bounds the exact distance from c to each of its points.  Directed rounding keeps each
// step on the safe side.  `s` is the float dist2(q, c).
__device__ __forceinline__ float ball_bound(float s, float r, float margin) {
    const float s_lo = __fmul_rd(s, 1.0f - margin);       // <= exact |q-c|^2
    const float dq = __fsqrt_rd(s_lo);                     // <= exact |q-c|
    const float gap = __fsub_rd(dq, r);                    // <= exact |q-p| for p in the ball
    if (!(gap > 0.0f)) return 0.0f;
    const float b = __fmul_rd(gap, gap);                   // <= exact |q-p|^2
    return __fmul_rd(b, 1.0f - margin);                    // <= float dist2(q, p)
}

// Radius stored for a ball whose float dist2 from the centre to its farthest point is m:
// an upper bound on the exact distance.
__device__ __forceinline__ float ball_radius(float m, float margin) {
    return __fsqrt_ru(__fmul_ru(m, 1.0f + margin));
}

__host__ __device__ __forceinline__ uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

__host__ __device__ __forceinline__ uint32_t log2_ceil(uint32_t v) {
    uint32_t r = 1;
    uint64_t c = 2;
    while (c < v) {
        c *= 2;
        r += 1;
    }
    return r;
}

// Depth of node i in an implicit heap (root depth 0).
__device__ __forceinline__ uint32_t heap_depth(uint32_t node) { return 31u - __clz(node + 1u); }

// Position of the n-th (0-based) set bit of m (n < popc(m)), by halving on popcounts.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 16; w; w >>= 1) {
        const uint32_t c = __popc(m & ((1u << w) - 1u));
        if (n >= c) {
            n -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

}  // namespace knn
