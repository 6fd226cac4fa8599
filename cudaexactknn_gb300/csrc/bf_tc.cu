// Brute force with a BF16 tensor-core filter (tcgen05, sm_103a) and exact FP32 rescoring.
//
// The reference computes every pair's distance with SIMT FP32 (src/BruteForceGpu.cuh:9-31).
// For dims >= 16 the engine can instead compute G = q~ . p~ for all pairs as a BF16 GEMM with FP32
// accumulation on the 5th-generation tensor cores, and use
//     |q|^2 + |p|^2 - 2 G  +-  E(q, p)
// as a rigorous interval around each pair's distance.  The lower end filters candidates, the
// upper end maintains each query's running k-th bound T; every candidate is then rescored with
// the reference's own sequential FP32 sum, so the answer is exactly the plain brute force's.
//
// Error bound (u = 2^-8 is bf16's unit roundoff; q~, p~ are q, p rounded to bf16):
//   |q~_d p~_d - q_d p_d| <= (2u + u^2) |q_d p_d|,  sum |q_d p_d| <= |q| |p|  (Cauchy-Schwarz),
//   tensor-core FP32 accumulation of D products <= D 2^-20 sum |q~_d p~_d|  (8x the bound for
//   truncating every addition),
//   norms |q|^2, |p|^2 in float: relative error <= (D+1) 2^-24,
// so with S = exact sum (q_d - p_d)^2:
//   |(|q|^2 + |p|^2 - 2G) - S| <= c1 |q||p| + c2 (|q|^2 + |p|^2),
//   c1 = 2 (2u + u^2 + D 2^-20)(1 + 2^-7),  c2 = (D + 8) 2^-23.
// The float sequential sum S_f the engine reports satisfies S (1 - g) <= S_f <= S (1 + g) with
// g = (D + 4) 2^-23 (knn::rel_margin).  A point is a candidate when (lower bound)(1 - g) <= T; T is
// the k-th smallest (upper bound)(1 + g) seen so far, which is >= the final k-th S_f, so every
// point that can enter the top-k (ties included) is a candidate.
//
// Kernel shape: one CTA per 128 queries, 6 warps: warp 0 streams 256-point BF16 tiles into a
// 2-stage shared-memory ring with bulk asynchronous copies, warp 1 allocates tensor memory and
// issues tcgen05.mma (M=128, N=256, K=16 steps) into two TMEM accumulators of 256 columns,
// warps 2-5 read accumulator rows with tcgen05.ld (thread = query) and filter.  Operands are
// pre-packed in global memory in the exact shared-memory image of the K-major 128-byte-swizzle
// layout, so plain bulk copies (no tensor maps) land them ready for the MMA descriptors.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "knn_internal.h"
#include "tc_ptx.cuh"
#include "tracker.cuh"

namespace knn {

namespace {

using namespace tc;

constexpr uint32_t kTileM = 128;
constexpr uint32_t kTileN = 256;
constexpr uint32_t kEpiWarps = 4;
constexpr uint32_t kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kTmemCols = 512;  // two accumulators of kTileN fp32 columns

struct TcParams {
    const uint8_t* qimg;  // [qtiles][H][128 rows][128 B]
    const uint8_t* pimg;  // [ptiles][H][256 rows][128 B]
    const float2* qnorm;  // per query: {|q|^2, |q|}
    const float2* pnorm;  // per point: {|p|^2, |p|}
    uint32_t n, nq, ptiles;
    float c1, c2, g;
    float max_d2;
    const float* radii;   // per-query radius or null (indexed by query)
    const uint32_t* order;       // row -> query, or null
    const uint32_t* live_count;  // rows in use (device), or null for nq
    uint32_t k;
    uint32_t cap;
    uint32_t* cand;       // [nq][cap]
    uint32_t* cand_count; // [nq]
    int* error;
};

__device__ __forceinline__ uint32_t a_bytes(uint32_t h) { return h * kTileM * 128u; }
__device__ __forceinline__ uint32_t b_bytes(uint32_t h) { return h * kTileN * 128u; }

// Heap of this thread's k smallest upper bounds (max at slot 0), slot-major in shared memory.
struct BoundHeap {
    float* base;  // slot i at base[i * kTileM]
    uint32_t k;
    __device__ __forceinline__ float& at(uint32_t i) const { return base[i * kTileM]; }
    __device__ __forceinline__ void replace_top(float x) {
        uint32_t pos = 0;
        for (;;) {
            const uint32_t l = 2 * pos + 1;
            if (l >= k) break;
            uint32_t big = l;
            float bv = at(l);
            if (l + 1 < k && at(l + 1) > bv) {
                big = l + 1;
                bv = at(l + 1);
            }
            if (bv <= x) break;
            at(pos) = bv;
            pos = big;
        }
        at(pos) = x;
    }
};

template <uint32_t H>
__global__ void __launch_bounds__(kThreads, 1) tc_filter_kernel(const TcParams p) {
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the 128-byte swizzle atoms.
    const uint32_t raw = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* sA = smem;
    uint8_t* sB0 = sA + H * kTileM * 128u;
    uint8_t* sB1 = sB0 + H * kTileN * 128u;
    float2* sN = reinterpret_cast<float2*>(sB1 + H * kTileN * 128u);  // [2][kTileN] point norms
    float* heap_base = reinterpret_cast<float*>(sN + 2 * kTileN);
    uint64_t* bars = reinterpret_cast<uint64_t*>(heap_base + static_cast<size_t>(p.k) * kTileM);
    uint64_t* full = bars;         // [2] B stage loaded
    uint64_t* empty = bars + 2;    // [2] B stage consumed by the MMAs
    uint64_t* acc_full = bars + 4; // [2] accumulator ready
    uint64_t* acc_empty = bars + 6;// [2] accumulator drained by the epilogue
    uint64_t* a_full = bars + 8;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 9);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t live_rows = p.live_count ? *p.live_count : p.nq;
    if (blockIdx.x * kTileM >= live_rows) return;  // whole block idle: leave before any allocation
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(full + i, 1);
            mbar_init(empty + i, 1);
            mbar_init(acc_full + i, 1);
            mbar_init(acc_empty + i, kEpiWarps * 32);
        }
        mbar_init(a_full, 1);
        *abort = 0;
        mbar_fence_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t ptiles = p.ptiles;

    if (warp == 0) {
        if (lane == 0) {
            // Producer: the query tile once, then the point tiles through the 2-stage ring.
            mbar_expect_tx(a_full, a_bytes(H));
            bulk_copy_g2s(sA, p.qimg + static_cast<size_t>(blockIdx.x) * a_bytes(H), a_bytes(H), a_full);
            uint32_t issued = 0;
            constexpr uint32_t kNormBytes = kTileN * sizeof(float2);
            for (uint32_t t = 0; t < ptiles; ++t) {
                const uint32_t s = t & 1;
                // Stage s is free once the MMAs of tile t-2 are done (operands) and the epilogue
                // has drained tile t-2 (its norms).
                if (t >= 2 && (!mbar_wait(empty + s, ((t >> 1) - 1) & 1, abort) ||
                               !mbar_wait(acc_empty + s, ((t >> 1) - 1) & 1, abort))) {
                    *abort = 1;
                    break;
                }
                mbar_expect_tx(full + s, b_bytes(H) + kNormBytes);
                bulk_copy_g2s(s ? sB1 : sB0, p.pimg + static_cast<size_t>(t) * b_bytes(H), b_bytes(H), full + s);
                bulk_copy_g2s(sN + s * kTileN, p.pnorm + static_cast<size_t>(t) * kTileN, kNormBytes, full + s);
                ++issued;
            }
            if (*abort) {
                // Let copies already in flight land before the block can exit.
                mbar_wait(a_full, 0, abort);
                for (uint32_t t = issued >= 2 ? issued - 2 : 0; t < issued; ++t) {
                    volatile int never = 0;
                    mbar_wait(full + (t & 1), (t >> 1) & 1, &never);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer.
            constexpr uint32_t idesc = idesc_bf16(kTileM, kTileN);
            bool ok = mbar_wait(a_full, 0, abort);
            const uint32_t a0 = smem_addr(sA);
            for (uint32_t t = 0; ok && t < ptiles; ++t) {
                const uint32_t s = t & 1, b = t & 1;
                if (!mbar_wait(full + s, (t >> 1) & 1, abort)) {
                    ok = false;
                    break;
                }
                if (t >= 2 && !mbar_wait(acc_empty + b, ((t >> 1) - 1) & 1, abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t b0 = smem_addr(s ? sB1 : sB0);
#pragma unroll
                for (uint32_t h = 0; h < H; ++h)
#pragma unroll
                    for (uint32_t kk = 0; kk < 4; ++kk)
                        mma_bf16(tmem + b * kTileN, desc_sw128(a0 + h * kTileM * 128u + kk * 32u),
                                 desc_sw128(b0 + h * kTileN * 128u + kk * 32u), idesc, (h | kk) != 0);
                mma_commit(empty + s);
                mma_commit(acc_full + b);
            }
            if (!ok) *abort = 1;
        }
    } else {
        // Epilogue: thread = query row.  TMEM lanes 32*(warp%4) .. +31 belong to this warp.
        const uint32_t quarter = warp & 3;
        const uint32_t row = quarter * 32 + lane;
        const uint32_t q = blockIdx.x * kTileM + row;  // row of the batch (position in the list)
        const bool live = q < live_rows;
        const uint32_t qi = live ? (p.order ? p.order[q] : q) : 0u;
        const float2 qn = live ? p.qnorm[q] : make_float2(0.0f, 0.0f);
        const float seed = live ? (p.radii ? fminf(p.radii[qi], p.max_d2) : p.max_d2) : 0.0f;
        BoundHeap heap{heap_base + row, p.k};
        for (uint32_t i = 0; i < p.k; ++i) heap.at(i) = seed;
        float T = seed;
        const float one_m = __fsub_rd(1.0f, p.g), one_p = __fadd_ru(1.0f, p.g);
        const float c2_hi = __fadd_ru(1.0f, p.c2);
        const float c1q = __fmul_ru(p.c1, qn.y);
        // Candidate test as a threshold on G:  G >= alpha |p|^2 - beta |p| + gam, all rounded down.
        const float alpha = __fmul_rd(0.5f, 1.0f - p.c2);
        const float beta = __fmul_ru(0.5f * p.c1, qn.y);
        auto gamma_of = [&](float tb) {
            const float tp = __fdiv_ru(tb, one_m);  // T / (1 - g), rounded up
            return __fsub_rd(__fmul_rd(alpha, qn.x), __fmul_ru(0.5f, tp));
        };
        float gam = gamma_of(T);
        uint32_t count = 0;
        uint32_t* my_cand = p.cand + static_cast<size_t>(live ? q : 0) * p.cap;
        const uint32_t taddr_row = tmem + ((quarter * 32u) << 16);
        bool ok = true;
        for (uint32_t t = 0; t < ptiles; ++t) {
            const uint32_t b = t & 1;
            // The TMEM loads below are warp-collective: the whole warp proceeds or leaves.
            // acc_full: the MMAs are done; full: this tile's norms landed in shared memory
            // (already complete, waited on to observe the copy's writes).
            const bool got = mbar_wait(acc_full + b, (t >> 1) & 1, abort) && mbar_wait(full + b, (t >> 1) & 1, abort);
            if (!__all_sync(0xFFFFFFFFu, got)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const float2* pn = sN + b * kTileN;
            const uint32_t base = t * kTileN;
#pragma unroll 1
            for (uint32_t c = 0; c < kTileN / 32; ++c) {
                float v[32];
                tmem_ld32(taddr_row + b * kTileN + c * 32, v);
#pragma unroll
                for (uint32_t i = 0; i < 32; ++i) {
                    const uint32_t jl = c * 32 + i;
                    const float2 pp = pn[jl];
                    const float theta = __fmaf_rd(alpha, pp.x, __fmaf_rd(-beta, pp.y, gam));
                    if (live && v[i] >= theta && base + jl < p.n) {
                        if (count < p.cap) my_cand[count] = base + jl;
                        ++count;
                        // Upper bound of this pair's float distance.
                        const float s = __fadd_ru(qn.x, pp.x);
                        const float hi = __fmaf_ru(-2.0f, v[i], __fmaf_ru(c1q, pp.y, __fmul_ru(c2_hi, s)));
                        const float u = __fmul_ru(fmaxf(hi, 0.0f), one_p);
                        if (u < T) {
                            heap.replace_top(u);
                            T = heap.at(0);
                            gam = gamma_of(T);
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(acc_empty + b);
        }
        if (!ok) *abort = 1;
        if (live) p.cand_count[q] = ok ? count : 0xFFFFFFFFu;
    }
    tc_fence_before();
    __syncthreads();
    if (*abort && threadIdx.x == 0) atomicExch(p.error, 1);
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Exact rescoring: the reference's sequential FP32 distance for every candidate, top-k by key.
// Queries whose candidate list overflowed (or whose filter block aborted) are listed for the
// plain search instead.
template <int PS, int KMAX>
__global__ void __launch_bounds__(128) tc_rescore_kernel(const float* __restrict__ points, const float* __restrict__ queries,
                                                         uint32_t dims, uint32_t nq, const uint32_t* __restrict__ cand,
                                                         const uint32_t* __restrict__ cand_count, uint32_t cap, uint32_t k,
                                                         float max_d2, const float* __restrict__ radii,
                                                         const uint32_t* __restrict__ order,
                                                         const uint32_t* __restrict__ live_count,
                                                         int32_t* __restrict__ out_idx, float* __restrict__ out_dist,
                                                         uint32_t* __restrict__ retry, uint32_t* __restrict__ retry_count) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;  // row of the batch
    if (q >= (live_count ? *live_count : nq)) return;
    const uint32_t qi = order ? order[q] : q;
    const uint32_t cnt = cand_count[q];
    if (cnt > cap) {
        retry[atomicAdd(retry_count, 1u)] = qi;
        return;
    }
    float qv[PS];
#pragma unroll
    for (int d = 0; d < PS; ++d) qv[d] = static_cast<uint32_t>(d) < dims ? queries[static_cast<size_t>(qi) * dims + d] : 0.0f;
    Tracker<KMAX, false, false> tr;
    tr.init(k, radii ? fminf(radii[qi], max_d2) : max_d2, nullptr, 0);
    const uint32_t* c = cand + static_cast<size_t>(q) * cap;
    for (uint32_t i = 0; i < cnt; ++i) {
        const uint32_t j = c[i];
        const float d2 = dist2_vec4<PS>(qv, reinterpret_cast<const float4*>(points + static_cast<size_t>(j) * PS));
        tr.offer(make_key(d2, static_cast<int32_t>(j)));
    }
    tr.emit(k, out_idx + static_cast<size_t>(qi) * k, out_dist + static_cast<size_t>(qi) * k);
}

// Packs rows of float data ([rows][dims]) into the 128-byte-swizzle BF16 image of `tile`-row
// tiles with H 64-element halves, and writes {sum x^2, sqrt} per row.  Rows past `rows` and
// columns past `dims` are zero.
__global__ void tc_pack_kernel(const float* __restrict__ src, uint32_t rows, uint32_t dims, uint32_t src_stride,
                               uint32_t tile, uint32_t H, uint8_t* __restrict__ img, float2* __restrict__ norms,
                               uint32_t padded_rows, const uint32_t* __restrict__ order = nullptr,
                               const uint32_t* __restrict__ live_count = nullptr) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= padded_rows) return;
    const uint32_t t = r / tile, rr = r % tile;
    uint8_t* base = img + static_cast<size_t>(t) * H * tile * 128u;
    const bool valid = r < (live_count ? *live_count : rows);
    const uint32_t sr = valid ? (order ? order[r] : r) : 0u;  // source row
    float acc = 0.0f;
    for (uint32_t k = 0; k < 64 * H; ++k) {
        const float x = (valid && k < dims) ? src[static_cast<size_t>(sr) * src_stride + k] : 0.0f;
        acc = __fmaf_rn(x, x, acc);
        const __nv_bfloat16 b = __float2bfloat16_rn(x);
        *reinterpret_cast<__nv_bfloat16*>(base + sw128_offset(tile, rr, k)) = b;
    }
    norms[r] = make_float2(acc, sqrtf(acc));
}

// Self-test: one 128 x 256 x (64 H) tile through the same descriptors, written to global.
template <uint32_t H>
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const uint8_t* __restrict__ qimg,
                                                             const uint8_t* __restrict__ pimg, float* __restrict__ out,
                                                             int* __restrict__ error) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* sA = smem;
    uint8_t* sB = sA + H * kTileM * 128u;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + H * kTileN * 128u);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        *abort = 0;
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, 256);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, a_bytes(H) + b_bytes(H));
        bulk_copy_g2s(sA, qimg, a_bytes(H), bar);
        bulk_copy_g2s(sB, pimg, b_bytes(H), bar);
        if (mbar_wait(bar, 0, abort)) {
            tc_fence_after();
            constexpr uint32_t idesc = idesc_bf16(kTileM, kTileN);
            for (uint32_t h = 0; h < H; ++h)
                for (uint32_t kk = 0; kk < 4; ++kk)
                    mma_bf16(tmem, desc_sw128(smem_addr(sA) + h * kTileM * 128u + kk * 32u),
                             desc_sw128(smem_addr(sB) + h * kTileN * 128u + kk * 32u), idesc, (h | kk) != 0);
            mma_commit(bar + 1);
        } else {
            *abort = 1;
        }
    }
    __syncthreads();
    const bool ok = !*abort && mbar_wait(bar + 1, 0, abort);
    if (ok) {
        tc_fence_after();
        for (uint32_t c = 0; c < kTileN / 32; ++c) {
            float v[32];
            tmem_ld32(tmem + ((warp * 32u) << 16) + c * 32, v);
            for (uint32_t i = 0; i < 32; ++i) out[(warp * 32 + lane) * kTileN + c * 32 + i] = v[i];
        }
    } else if (threadIdx.x == 0) {
        atomicExch(error, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

size_t filter_smem(uint32_t H, uint32_t k) {
    return 1024 + H * kTileM * 128u + 2 * H * kTileN * 128u + 2 * kTileN * sizeof(float2) +
           static_cast<size_t>(k) * kTileM * 4 + 16 * 8;
}

// The filter allocates all 512 TMEM columns, so a second resident block on the same SM would
// wait inside tcgen05.alloc; asking for more than half the SM's shared memory keeps one block
// per SM.
size_t filter_launch_smem(uint32_t H, uint32_t k) { return std::max<size_t>(filter_smem(H, k), 120 * 1024); }

}  // namespace

bool tc_supported(uint32_t dims, uint32_t k) { return dims >= 1 && dims <= 128 && k <= 128 && filter_smem(dims <= 64 ? 1 : 2, k) <= 232448; }

// Prepares the BF16 point image and norms of a brute-force index (once).
int tc_prepare(knn_index* ix, cudaStream_t s) {
    if (ix->tc_ready) return KNN_OK;
    const uint32_t H = ix->dims <= 64 ? 1 : 2;
    const uint32_t ptiles = ceil_div(ix->n, kTileN);
    const uint32_t prows = ptiles * kTileN;
    KNN_TRY(ix->tc_img.alloc(static_cast<size_t>(ptiles) * H * kTileN * 128u));
    KNN_TRY(ix->tc_norm.alloc(static_cast<size_t>(prows) * sizeof(float2)));
    tc_pack_kernel<<<ceil_div(prows, 128), 128, 0, s>>>(ix->points.as<float>(), ix->n, ix->dims, ix->point_stride,
                                                        kTileN, H, ix->tc_img.as<uint8_t>(), ix->tc_norm.as<float2>(),
                                                        prows);
    KNN_LAUNCHED();
    ix->tc_ready = true;
    ix->device_bytes += ix->tc_img.bytes + ix->tc_norm.bytes;
    return KNN_OK;
}

template <int PS, int KMAX>
static int rescore(knn_index* ix, const QueryArgs& a, const uint32_t* cand, const uint32_t* cnt, uint32_t cap,
                   uint32_t* retry, uint32_t* retry_count, cudaStream_t s) {
    tc_rescore_kernel<PS, KMAX><<<ceil_div(a.count, 128), 128, 0, s>>>(
        ix->points.as<float>(), a.queries, ix->dims, a.count, cand, cnt, cap, a.k, a.max_d2, a.radii, a.order,
        a.count_dev, a.out_idx, a.out_dist, retry, retry_count);
    KNN_LAUNCHED();
    return KNN_OK;
}

template <int PS>
static int rescore_k(knn_index* ix, const QueryArgs& a, const uint32_t* cand, const uint32_t* cnt, uint32_t cap,
                     uint32_t* retry, uint32_t* retry_count, cudaStream_t s) {
    switch (k_class(a.k)) {
        case 8: return rescore<PS, 8>(ix, a, cand, cnt, cap, retry, retry_count, s);
        case 16: return rescore<PS, 16>(ix, a, cand, cnt, cap, retry, retry_count, s);
        case 32: return rescore<PS, 32>(ix, a, cand, cnt, cap, retry, retry_count, s);
        case 64: return rescore<PS, 64>(ix, a, cand, cnt, cap, retry, retry_count, s);
        default: return rescore<PS, 128>(ix, a, cand, cnt, cap, retry, retry_count, s);
    }
}

int bf_tc_query(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, cudaStream_t s) {
    const uint32_t H = ix->dims <= 64 ? 1 : 2;
    if (!tc_supported(ix->dims, a.k)) return fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: dims %u, k %u", ix->dims, a.k);
    KNN_TRY(tc_prepare(ix, s));
    const uint32_t nq = a.count;
    const uint32_t qtiles = ceil_div(nq, kTileM);
    const uint32_t qrows = qtiles * kTileM;
    const uint32_t cap = plan.tc_cap ? plan.tc_cap : 4096;
    const size_t qimg_bytes = static_cast<size_t>(qtiles) * H * kTileM * 128u;
    KNN_TRY(ix->tc_ws.reserve(carve_bytes({qimg_bytes, static_cast<size_t>(qrows) * 8, static_cast<size_t>(nq) * cap * 4,
                                           static_cast<size_t>(nq) * 4, static_cast<size_t>(nq) * 4, 256})));
    Carver c(ix->tc_ws.ptr);
    uint8_t* qimg = c.take<uint8_t>(qimg_bytes);
    float2* qnorm = c.take<float2>(qrows);
    uint32_t* cand = c.take<uint32_t>(static_cast<size_t>(nq) * cap);
    uint32_t* cnt = c.take<uint32_t>(nq);
    uint32_t* retry = c.take<uint32_t>(nq);
    uint32_t* small = c.take<uint32_t>(64);  // [0] retry count, [1] error flag
    KNN_TRY_CUDA(cudaMemsetAsync(small, 0, 64 * sizeof(uint32_t), s));
    tc_pack_kernel<<<ceil_div(qrows, 128), 128, 0, s>>>(a.queries, nq, ix->dims, ix->dims, kTileM, H, qimg, qnorm, qrows,
                                                        a.order, a.count_dev);
    KNN_LAUNCHED();

    TcParams p{};
    p.qimg = qimg;
    p.pimg = ix->tc_img.as<uint8_t>();
    p.qnorm = qnorm;
    p.pnorm = ix->tc_norm.as<float2>();
    p.n = ix->n;
    p.nq = nq;
    p.ptiles = ceil_div(ix->n, kTileN);
    const double u = 1.0 / 256.0, D = ix->dims;
    p.c1 = static_cast<float>(2.0 * (2.0 * u + u * u + D * std::ldexp(1.0, -20)) * (1.0 + 1.0 / 128.0));
    p.c2 = static_cast<float>((D + 8.0) * std::ldexp(1.0, -23));
    p.g = rel_margin(ix->dims);
    p.max_d2 = a.max_d2;
    p.radii = a.radii;
    p.order = a.order;
    p.live_count = a.count_dev;
    p.k = a.k;
    p.cap = cap;
    p.cand = cand;
    p.cand_count = cnt;
    p.error = reinterpret_cast<int*>(small + 1);
    const size_t smem = filter_launch_smem(H, a.k);
    auto kern = H == 1 ? tc_filter_kernel<1> : tc_filter_kernel<2>;
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern0, s));
    kern<<<qtiles, kThreads, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY_CUDA(cudaEventRecord(ix->timing.kern1, s));

    switch (round_up4(ix->dp)) {
        case 16: KNN_TRY(rescore_k<16>(ix, a, cand, cnt, cap, retry, small, s)); break;
        case 32: KNN_TRY(rescore_k<32>(ix, a, cand, cnt, cap, retry, small, s)); break;
        case 64: KNN_TRY(rescore_k<64>(ix, a, cand, cnt, cap, retry, small, s)); break;
        case 128: KNN_TRY(rescore_k<128>(ix, a, cand, cnt, cap, retry, small, s)); break;
        default: KNN_TRY(rescore_k<8>(ix, a, cand, cnt, cap, retry, small, s)); break;
    }
    // Queries whose candidates overflowed, or whose filter block gave up, take the plain path.
    QueryArgs again = a;
    again.order = retry;
    again.count_dev = small;
    QueryPlan plain = plan;
    plain.timing = false;
    plain.bf16 = false;
    return bf_query(ix, again, plain, s);
}

int tc_selftest(uint32_t dims, float* max_rel_err, uint32_t* bad) {
    const uint32_t H = dims <= 64 ? 1 : 2;
    const uint32_t qn = kTileM, pn = kTileN;
    std::vector<float> hq(static_cast<size_t>(qn) * dims), hp(static_cast<size_t>(pn) * dims);
    uint32_t st = 12345;
    auto rnd = [&]() {
        st = st * 1664525u + 1013904223u;
        return (static_cast<int>(st >> 9) % 2001 - 1000) / 250.0f;  // multiples of 1/250 in [-4, 4]
    };
    for (auto& v : hq) v = rnd();
    for (auto& v : hp) v = rnd();
    DevBuf buf;
    const size_t ab = static_cast<size_t>(H) * kTileM * 128u, bb = static_cast<size_t>(H) * kTileN * 128u;
    KNN_TRY(buf.alloc(carve_bytes({hq.size() * 4, hp.size() * 4, ab, bb, qn * 8ull, pn * 8ull, qn * pn * 4ull, 64})));
    Carver c(buf.ptr);
    float* dq = c.take<float>(hq.size());
    float* dp = c.take<float>(hp.size());
    uint8_t* qimg = c.take<uint8_t>(ab);
    uint8_t* pimg = c.take<uint8_t>(bb);
    float2* qnm = c.take<float2>(qn);
    float2* pnm = c.take<float2>(pn);
    float* out = c.take<float>(static_cast<size_t>(qn) * pn);
    int* err = c.take<int>(16);
    KNN_TRY_CUDA(cudaMemcpy(dq, hq.data(), hq.size() * 4, cudaMemcpyHostToDevice));
    KNN_TRY_CUDA(cudaMemcpy(dp, hp.data(), hp.size() * 4, cudaMemcpyHostToDevice));
    KNN_TRY_CUDA(cudaMemset(err, 0, 64));
    tc_pack_kernel<<<1, 128, 0>>>(dq, qn, dims, dims, kTileM, H, qimg, qnm, qn);
    tc_pack_kernel<<<2, 128, 0>>>(dp, pn, dims, dims, kTileN, H, pimg, pnm, pn);
    const size_t smem = 1024 + ab + bb + 64;
    auto kern = H == 1 ? tc_selftest_kernel<1> : tc_selftest_kernel<2>;
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    kern<<<1, 128, smem>>>(qimg, pimg, out, err);
    KNN_LAUNCHED_N(3);
    KNN_TRY_CUDA(cudaDeviceSynchronize());
    std::vector<float> ho(static_cast<size_t>(qn) * pn);
    int herr = 0;
    KNN_TRY_CUDA(cudaMemcpy(ho.data(), out, ho.size() * 4, cudaMemcpyDeviceToHost));
    KNN_TRY_CUDA(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
    if (herr) return fail(KNN_ERR_DEVICE_LIMIT, "tensor-core self-test kernel timed out");
    // Inputs are multiples of 1/250 with |x| <= 4, bf16-rounded; products and sums in double.
    auto bf = [](float x) {
        uint32_t u;
        std::memcpy(&u, &x, 4);
        const uint32_t lsb = (u >> 16) & 1u;
        u = (u + 0x7FFFu + lsb) & 0xFFFF0000u;
        float r;
        std::memcpy(&r, &u, 4);
        return r;
    };
    double worst = 0;
    uint32_t nbad = 0;
    for (uint32_t i = 0; i < qn; ++i)
        for (uint32_t j = 0; j < pn; ++j) {
            double ref = 0, mag = 0;
            for (uint32_t d = 0; d < dims; ++d) {
                const double t = static_cast<double>(bf(hq[i * dims + d])) * bf(hp[j * dims + d]);
                ref += t;
                mag += std::fabs(t);
            }
            const double e = std::fabs(ho[static_cast<size_t>(i) * pn + j] - ref) / std::max(mag, 1e-30);
            worst = std::max(worst, e);
            if (e > dims * std::ldexp(1.0, -20)) ++nbad;
        }
    *max_rel_err = static_cast<float>(worst);
    *bad = nbad;
    return KNN_OK;
}

}  // namespace knn
