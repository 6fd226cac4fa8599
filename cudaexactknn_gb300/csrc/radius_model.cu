// Learned search radius: a D -> 64 -> 64 -> 1 multilayer perceptron that predicts, from a
// query's coordinates, the logarithm of its k-th neighbour's squared distance.  The prediction
// plus a calibrated margin seeds each query's search radius (max_distance2); a query that finds
// fewer than k points inside its seeded radius is searched again without the seed, so answers
// stay exact and the plain search is both the fallback and the arbiter.
//
// Training runs on the GPU with the kernels below (forward + backward per sample, weight
// gradients as batch reductions in a fixed order, Adam), on targets produced by the engine's own
// exact search for sample queries.  Query-time inference runs on the tensor cores
// (mlp_infer_tc_kernel, FP16 operands, FP32 accumulation); the prediction API keeps the FP32
// kernel.  The reference has no counterpart: its pruning radius is the
// caller's single Query::maxDistance2 (src/KnnTrees.cuh:228, used at src/KdTreeGpu.cuh:211 and
// src/BallTreeGpu.cuh:48).
//
// Input encoding: the coordinates scaled to [0, 1]^D (per-dimension range of the training
// samples), followed by sin and cos of 32 fixed random projections 2 pi z . B (B ~ N(0, 4^2),
// seeded): E = D + 64 features.  Fourier features of this kind (Tancik et al., NeurIPS 2020) let a
// small ReLU network fit the narrow density peaks of clustered data; on raw coordinates the same
// 64-64 network learned nothing beyond the mean for a 64-cluster mixture.
//
// Parameter layout (floats): W1[64][E] b1[64] W2[64][64] b2[64] w3[64] b3 (trainable), then the
// fixed projection B[D][32], the scaling lo[D] inv_range[D], and the calibrated margin.

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "knn_internal.h"
#include "tc_ptx.cuh"

namespace knn {

constexpr uint32_t kHidden = 64;
constexpr uint32_t kFourier = 32;
constexpr float kFourierScale = 4.0f;

struct ModelLayout {
    uint32_t dims, feats;
    uint32_t w1, b1, w2, b2, w3, b3, proj, lo, inv_range, margin, total, trainable;
    __host__ __device__ explicit ModelLayout(uint32_t d) : dims(d), feats(d + 2 * kFourier) {
        w1 = 0;
        b1 = w1 + kHidden * feats;
        w2 = b1 + kHidden;
        b2 = w2 + kHidden * kHidden;
        w3 = b2 + kHidden;
        b3 = w3 + kHidden;
        trainable = b3 + 1;
        proj = trainable;
        lo = proj + d * kFourier;
        inv_range = lo + d;
        margin = inv_range + d;
        total = margin + 1;
    }
};

// Features of one input row: e[0..D) = scaled coordinates, e[D+f] = sin(2 pi z.B_f),
// e[D+32+f] = cos(2 pi z.B_f).
__device__ __forceinline__ void encode(const float* __restrict__ prm, const ModelLayout& L,
                                       const float* __restrict__ x, float* __restrict__ e) {
    for (uint32_t d = 0; d < L.dims; ++d) e[d] = (x[d] - prm[L.lo + d]) * prm[L.inv_range + d];
    for (uint32_t f = 0; f < kFourier; ++f) {
        float a = 0.0f;
        for (uint32_t d = 0; d < L.dims; ++d) a = fmaf(e[d], prm[L.proj + d * kFourier + f], a);
        float sv, cv;
        sincospif(2.0f * a, &sv, &cv);  // sin and cos of 2 pi a
        e[L.dims + f] = sv;
        e[L.dims + kFourier + f] = cv;
    }
}

namespace {

// Forward (and, with targets, backward) of one sample per thread.  Stores the activations and
// the back-propagated deltas for the gradient reductions.
__global__ void mlp_fwd_bwd_kernel(const float* __restrict__ prm, uint32_t dims, const float* __restrict__ x,
                                   const float* __restrict__ target, const uint32_t* __restrict__ rows,
                                   uint32_t batch, float* __restrict__ xn_out, float* __restrict__ h1_out,
                                   float* __restrict__ h2_out, float* __restrict__ d1_out,
                                   float* __restrict__ d2_out, float* __restrict__ dy_out,
                                   float* __restrict__ loss_out) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    const ModelLayout L(dims);
    const uint32_t r = rows ? rows[b] : b;
    float* xn = xn_out + static_cast<size_t>(b) * L.feats;  // the sample's features
    encode(prm, L, x + static_cast<size_t>(r) * dims, xn);
    float h1[kHidden], h2[kHidden];
    for (uint32_t i = 0; i < kHidden; ++i) {
        float a = prm[L.b1 + i];
        for (uint32_t d = 0; d < L.feats; ++d) a = fmaf(prm[L.w1 + i * L.feats + d], xn[d], a);
        h1[i] = fmaxf(a, 0.0f);
        h1_out[static_cast<size_t>(b) * kHidden + i] = h1[i];
    }
    float y = prm[L.b3];
    for (uint32_t i = 0; i < kHidden; ++i) {
        float a = prm[L.b2 + i];
        for (uint32_t j = 0; j < kHidden; ++j) a = fmaf(prm[L.w2 + i * kHidden + j], h1[j], a);
        h2[i] = fmaxf(a, 0.0f);
        h2_out[static_cast<size_t>(b) * kHidden + i] = h2[i];
        y = fmaf(prm[L.w3 + i], h2[i], y);
    }
    // Mean squared error on the log distance: loss = mean (y - t)^2.
    const float err = y - target[r];
    const float dy = 2.0f * err / static_cast<float>(batch);
    dy_out[b] = dy;
    loss_out[b] = err * err / static_cast<float>(batch);
    float d2[kHidden];
    for (uint32_t i = 0; i < kHidden; ++i) {
        d2[i] = h2[i] > 0.0f ? dy * prm[L.w3 + i] : 0.0f;
        d2_out[static_cast<size_t>(b) * kHidden + i] = d2[i];
    }
    for (uint32_t j = 0; j < kHidden; ++j) {
        float a = 0.0f;
        for (uint32_t i = 0; i < kHidden; ++i) a = fmaf(prm[L.w2 + i * kHidden + j], d2[i], a);
        d1_out[static_cast<size_t>(b) * kHidden + j] = h1[j] > 0.0f ? a : 0.0f;
    }
}

// One thread per trainable parameter: its gradient summed over the batch in sample order.
__global__ void mlp_grad_kernel(uint32_t dims, uint32_t batch, const float* __restrict__ xn,
                                const float* __restrict__ h1, const float* __restrict__ h2,
                                const float* __restrict__ d1, const float* __restrict__ d2,
                                const float* __restrict__ dy, float* __restrict__ grad) {
    const ModelLayout L(dims);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= L.trainable) return;
    float g = 0.0f;
    if (p < L.b1) {
        const uint32_t i = p / L.feats, d = p % L.feats;
        for (uint32_t b = 0; b < batch; ++b) g = fmaf(d1[b * kHidden + i], xn[b * L.feats + d], g);
    } else if (p < L.w2) {
        const uint32_t i = p - L.b1;
        for (uint32_t b = 0; b < batch; ++b) g += d1[b * kHidden + i];
    } else if (p < L.b2) {
        const uint32_t i = (p - L.w2) / kHidden, j = (p - L.w2) % kHidden;
        for (uint32_t b = 0; b < batch; ++b) g = fmaf(d2[b * kHidden + i], h1[b * kHidden + j], g);
    } else if (p < L.w3) {
        const uint32_t i = p - L.b2;
        for (uint32_t b = 0; b < batch; ++b) g += d2[b * kHidden + i];
    } else if (p < L.b3) {
        const uint32_t j = p - L.w3;
        for (uint32_t b = 0; b < batch; ++b) g = fmaf(dy[b], h2[b * kHidden + j], g);
    } else {
        for (uint32_t b = 0; b < batch; ++b) g += dy[b];
    }
    grad[p] = g;
}

// Adam (Kingma & Ba, 2015) with bias correction.
__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                            float* __restrict__ v, uint32_t n, float lr, float beta1, float beta2, float eps,
                            float corr1, float corr2) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float g = grad[p];
    const float mp = beta1 * m[p] + (1.0f - beta1) * g;
    const float vp = beta2 * v[p] + (1.0f - beta2) * g * g;
    m[p] = mp;
    v[p] = vp;
    prm[p] -= lr * (mp / corr1) / (sqrtf(vp / corr2) + eps);
}

// Seeded radius of each query, specialised on the padded input width: the parameters are
// staged in shared memory (every thread reads the same weights: broadcast float4 loads), the
// hidden activations stay in registers.
template <int DP>
__global__ void __launch_bounds__(256) mlp_infer_fast_kernel(const float* __restrict__ prm, uint32_t dims,
                                                             const float* __restrict__ x, uint32_t count,
                                                             float max_d2, const float* __restrict__ user_radii,
                                                             float* __restrict__ radii, float* __restrict__ raw) {
    extern __shared__ __align__(16) float sp[];
    const ModelLayout L(dims);
    // sp: the parameters as stored, then W1 transposed ([feature][hidden]) for float4 loads.
    float* w1t = sp + ((L.total + 3) & ~3u);
    for (uint32_t i = threadIdx.x; i < L.total; i += blockDim.x) sp[i] = prm[i];
    for (uint32_t i = threadIdx.x; i < kHidden * L.feats; i += blockDim.x) {
        const uint32_t h = i / L.feats, f = i % L.feats;
        w1t[f * kHidden + h] = prm[L.w1 + i];
    }
    __syncthreads();
    const float4* w1t4 = reinterpret_cast<const float4*>(w1t);
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    float z[DP];
#pragma unroll
    for (int d = 0; d < DP; ++d)
        z[d] = static_cast<uint32_t>(d) < dims ? (x[static_cast<size_t>(q) * dims + d] - sp[L.lo + d]) * sp[L.inv_range + d]
                                               : 0.0f;
    // First layer over the features, accumulated feature by feature.
    float h1[kHidden];
#pragma unroll
    for (int i = 0; i < static_cast<int>(kHidden); ++i) h1[i] = sp[L.b1 + i];
    auto add_feature = [&](uint32_t f, float v) {
#pragma unroll
        for (int i4 = 0; i4 < static_cast<int>(kHidden / 4); ++i4) {
            const float4 w = w1t4[f * (kHidden / 4) + i4];
            h1[4 * i4 + 0] = fmaf(w.x, v, h1[4 * i4 + 0]);
            h1[4 * i4 + 1] = fmaf(w.y, v, h1[4 * i4 + 1]);
            h1[4 * i4 + 2] = fmaf(w.z, v, h1[4 * i4 + 2]);
            h1[4 * i4 + 3] = fmaf(w.w, v, h1[4 * i4 + 3]);
        }
    };
#pragma unroll
    for (int d = 0; d < DP; ++d)
        if (static_cast<uint32_t>(d) < dims) add_feature(d, z[d]);
#pragma unroll 1
    for (uint32_t f = 0; f < kFourier; ++f) {
        float a = 0.0f;
#pragma unroll
        for (int d = 0; d < DP; ++d)
            if (static_cast<uint32_t>(d) < dims) a = fmaf(z[d], sp[L.proj + d * kFourier + f], a);
        float sv, cv;
        sincospif(2.0f * a, &sv, &cv);
        add_feature(dims + f, sv);
        add_feature(dims + kFourier + f, cv);
    }
#pragma unroll
    for (int i = 0; i < static_cast<int>(kHidden); ++i) h1[i] = fmaxf(h1[i], 0.0f);
    float y = sp[L.b3];
    const float4* w2 = reinterpret_cast<const float4*>(sp + L.w2);  // W2 starts at a multiple of 4 floats
    for (int i = 0; i < static_cast<int>(kHidden); ++i) {
        float a = sp[L.b2 + i];
#pragma unroll
        for (int j4 = 0; j4 < static_cast<int>(kHidden / 4); ++j4) {
            const float4 w = w2[i * (kHidden / 4) + j4];
            a = fmaf(w.x, h1[4 * j4 + 0], a);
            a = fmaf(w.y, h1[4 * j4 + 1], a);
            a = fmaf(w.z, h1[4 * j4 + 2], a);
            a = fmaf(w.w, h1[4 * j4 + 3], a);
        }
        y = fmaf(sp[L.w3 + i], fmaxf(a, 0.0f), y);
    }
    if (raw) raw[q] = y;
    if (radii) {
        const float cap = user_radii ? user_radii[q] : max_d2;
        radii[q] = fminf(__expf(fminf(y + sp[L.margin], 80.0f)), cap);
    }
}

// Seeded radius of each query: min(exp(prediction + margin), the caller's radius).
__global__ void mlp_infer_kernel(const float* __restrict__ prm, uint32_t dims, const float* __restrict__ x,
                                 uint32_t count, float max_d2, const float* __restrict__ user_radii,
                                 float* __restrict__ radii, float* __restrict__ raw) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const ModelLayout L(dims);
    float xn[kMaxDims + 2 * kFourier];
    encode(prm, L, x + static_cast<size_t>(q) * dims, xn);
    float h1[kHidden];
    for (uint32_t i = 0; i < kHidden; ++i) {
        float a = __ldg(prm + L.b1 + i);
        for (uint32_t d = 0; d < L.feats; ++d) a = fmaf(__ldg(prm + L.w1 + i * L.feats + d), xn[d], a);
        h1[i] = fmaxf(a, 0.0f);
    }
    float y = __ldg(prm + L.b3);
    for (uint32_t i = 0; i < kHidden; ++i) {
        float a = __ldg(prm + L.b2 + i);
#pragma unroll 16
        for (uint32_t j = 0; j < kHidden; ++j) a = fmaf(__ldg(prm + L.w2 + i * kHidden + j), h1[j], a);
        y = fmaf(__ldg(prm + L.w3 + i), fmaxf(a, 0.0f), y);
    }
    if (raw) raw[q] = y;
    if (radii) {
        const float cap = user_radii ? user_radii[q] : max_d2;
        const float r = __expf(fminf(y + __ldg(prm + L.margin), 80.0f));
        radii[q] = fminf(r, cap);
    }
}

// A query needs another search when its seeded radius was below the caller's and it found
// fewer than k points inside it.
__device__ __forceinline__ bool needs_retry(uint32_t q, const int32_t* out_idx, uint32_t k, const float* seeded,
                                            float max_d2, const float* user_radii) {
    const float cap = user_radii ? user_radii[q] : max_d2;
    return seeded[q] < cap && out_idx[static_cast<size_t>(q) * k + (k - 1)] < 0;
}

constexpr uint32_t kCompactThreads = 256;

__global__ void __launch_bounds__(kCompactThreads) retry_count_kernel(const uint32_t* __restrict__ order, uint32_t n,
                                                                      const int32_t* __restrict__ out_idx, uint32_t k,
                                                                      const float* __restrict__ seeded, float max_d2,
                                                                      const float* __restrict__ user_radii,
                                                                      uint32_t* __restrict__ bcnt) {
    __shared__ uint32_t warp_tot[kCompactThreads / 32];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    bool f = false;
    if (p < n) f = needs_retry(order ? order[p] : p, out_idx, k, seeded, max_d2, user_radii);
    const uint32_t c = __popc(__ballot_sync(0xFFFFFFFFu, f));
    if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x / 32] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < kCompactThreads / 32; ++w) t += warp_tot[w];
        bcnt[blockIdx.x] = t;
    }
}

// Writes the retry list in the given query order (stable compaction) and grows each listed
// query's radius: min(radius * grow, the caller's radius).
__global__ void __launch_bounds__(kCompactThreads) retry_scatter_kernel(
    const uint32_t* __restrict__ order, uint32_t n, const int32_t* __restrict__ out_idx, uint32_t k,
    float* __restrict__ seeded, float max_d2, const float* __restrict__ user_radii, const uint32_t* __restrict__ bpre,
    uint32_t nblk, float grow, uint32_t* __restrict__ list, uint32_t* __restrict__ list_count, DevCounters* counters) {
    __shared__ uint32_t warp_tot[kCompactThreads / 32];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x / 32;
    uint32_t q = 0;
    bool f = false;
    if (p < n) {
        q = order ? order[p] : p;
        f = needs_retry(q, out_idx, k, seeded, max_d2, user_radii);
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, f);
    if (lane == 0) warp_tot[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = bpre[blockIdx.x];
    for (uint32_t w = 0; w < warp; ++w) before += warp_tot[w];
    if (f) {
        list[before + __popc(bal & ((1u << lane) - 1u))] = q;
        const float cap = user_radii ? user_radii[q] : max_d2;
        seeded[q] = fminf(seeded[q] * grow, cap);
        if (counters) atomicAdd(&counters->fallback, 1ull);
    }
    if (blockIdx.x == nblk - 1 && threadIdx.x == 0) {
        uint32_t total = bpre[blockIdx.x];
        for (uint32_t w = 0; w < kCompactThreads / 32; ++w) total += warp_tot[w];
        *list_count = total;
    }
}

__global__ void kth_log_kernel(const float* __restrict__ dist, const int32_t* __restrict__ idx, uint32_t count,
                               uint32_t k, float* __restrict__ target) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const float d = dist[static_cast<size_t>(q) * k + (k - 1)];
    target[q] = logf(fmaxf(d, 1e-30f));
    (void)idx;
}

}  // namespace

size_t model_floats(uint32_t dims) { return ModelLayout(dims).total; }

// Forward + backward for `batch` samples with the given parameters; writes gradients and the
// summed loss (used by training and by the gradient check).
int model_gradients(const float* d_prm, uint32_t dims, const float* d_x, const float* d_t, const uint32_t* d_rows,
                    uint32_t batch, float* d_grad, float* d_loss_rows, DevBuf& scratch, cudaStream_t s) {
    const ModelLayout LL(dims);
    const size_t need = carve_bytes({static_cast<size_t>(batch) * LL.feats * 4, static_cast<size_t>(batch) * kHidden * 4,
                                     static_cast<size_t>(batch) * kHidden * 4, static_cast<size_t>(batch) * kHidden * 4,
                                     static_cast<size_t>(batch) * kHidden * 4, static_cast<size_t>(batch) * 4});
    KNN_TRY(scratch.reserve(need));
    Carver c(scratch.ptr);
    float* xn = c.take<float>(static_cast<size_t>(batch) * LL.feats);
    float* h1 = c.take<float>(static_cast<size_t>(batch) * kHidden);
    float* h2 = c.take<float>(static_cast<size_t>(batch) * kHidden);
    float* d1 = c.take<float>(static_cast<size_t>(batch) * kHidden);
    float* d2 = c.take<float>(static_cast<size_t>(batch) * kHidden);
    float* dy = c.take<float>(batch);
    mlp_fwd_bwd_kernel<<<ceil_div(batch, 128), 128, 0, s>>>(d_prm, dims, d_x, d_t, d_rows, batch, xn, h1, h2, d1,
                                                            d2, dy, d_loss_rows);
    const ModelLayout L(dims);
    mlp_grad_kernel<<<ceil_div(L.trainable, 128), 128, 0, s>>>(dims, batch, xn, h1, h2, d1, d2, dy, d_grad);
    KNN_LAUNCHED_N(2);
    return KNN_OK;
}

// ---- inference on the tensor cores ----------------------------------------------------------------
// Seeded radii for a query batch (the query path, and the training margin, so that the margin is
// measured on the same predictions): per 128-query tile, each thread builds its query's features
// (scaled coordinates, sin/cos of the Fourier projections), rounds them to FP16 and writes them to
// shared memory as the A operand (K-major, 128-byte swizzle); the hidden layers are tcgen05 GEMMs
// against W1 (64 x F) and W2 (64 x 64), packed to FP16 in shared memory once per block, with FP32
// accumulation in TMEM (columns 0-63 and 64-127); bias, ReLU and the output layer run in the
// epilogue.  The prediction only seeds a radius that the fallback rounds correct, so the 16-bit
// rounding changes no answer.  Blocks loop over tiles; every wait is bounded and a timeout leaves
// the caller's radius (the unseeded search) for the rest of the block's rows.
constexpr uint32_t kMlpRows = 128;
constexpr uint32_t kMlpFeatMax = 128;  // features per row this kernel takes (dims <= 64)

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// FP16 element (row, k) of a K-major 128-byte-swizzled image with `rows` rows.
__device__ __forceinline__ void put_half(uint8_t* img, uint32_t rows, uint32_t row, uint32_t k, float v) {
    *reinterpret_cast<__half*>(img + tc::sw_offset(128, rows, row, k)) = __float2half_rn(fminf(fmaxf(v, -65504.0f), 65504.0f));
}

__device__ __forceinline__ uint64_t mlp_desc(uint32_t base, uint32_t rows, uint32_t ks) {
    return tc::desc_sw(base + (ks / 4) * rows * 128u + (ks % 4) * 32u, 128);
}

template <int DP>
__global__ void __launch_bounds__(kMlpRows, 1) mlp_infer_tc_kernel(const float* __restrict__ prm, uint32_t dims,
                                                                   const float* __restrict__ x, uint32_t count,
                                                                   float max_d2, const float* __restrict__ user_radii,
                                                                   float* __restrict__ radii, float* __restrict__ raw) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_a = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw_a + 1023u) & ~1023u) - raw_a);
    uint8_t* sA1 = smem;                        // [128 rows][128 features] FP16, two 64-element blocks
    uint8_t* sW1 = sA1 + kMlpRows * 256;        // [64 hidden][128 features]
    uint8_t* sA2 = sW1 + kHidden * 256;         // [128 rows][64 hidden], one block
    uint8_t* sW2 = sA2 + kMlpRows * 128;        // [64][64]
    float* sb = reinterpret_cast<float*>(sW2 + kHidden * 128);  // b1[64], b2[64], w3[64]
    uint64_t* bar = reinterpret_cast<uint64_t*>(sb + 3 * kHidden);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const ModelLayout L(dims);
    const uint32_t t = threadIdx.x, warp = t / 32, lane = t % 32;
    // Weights to FP16 images (zero beyond the features), biases and the output layer.
    for (uint32_t e = t; e < kHidden * kMlpFeatMax; e += kMlpRows) {
        const uint32_t n = e / kMlpFeatMax, f = e % kMlpFeatMax;
        put_half(sW1, kHidden, n, f, f < L.feats ? prm[L.w1 + n * L.feats + f] : 0.0f);
    }
    for (uint32_t e = t; e < kHidden * kHidden; e += kMlpRows)
        put_half(sW2, kHidden, e / kHidden, e % kHidden, prm[L.w2 + e]);
    for (uint32_t e = t; e < kHidden; e += kMlpRows) {
        sb[e] = prm[L.b1 + e];
        sb[kHidden + e] = prm[L.b2 + e];
        sb[2 * kHidden + e] = prm[L.w3 + e];
    }
    if (t == 0) {
        mbar_init(bar, 1);
        *abort = 0;
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, 128);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_f16(kMlpRows, kHidden);
    const uint32_t k1 = (L.feats + 15) / 16;
    const float b3 = prm[L.b3], margin = prm[L.margin];
    uint32_t phase = 0, commits = 0;  // commits: thread 0's count
    for (uint32_t tile = blockIdx.x; tile * kMlpRows < count; tile += gridDim.x) {
        const uint32_t q = tile * kMlpRows + t;
        const bool live = q < count;
        // Features of this thread's row.
        float z[DP];
#pragma unroll
        for (int d = 0; d < DP; ++d)
            z[d] = (live && static_cast<uint32_t>(d) < dims)
                       ? (x[static_cast<size_t>(q) * dims + d] - prm[L.lo + d]) * prm[L.inv_range + d] : 0.0f;
#pragma unroll
        for (int d = 0; d < DP; ++d)
            if (static_cast<uint32_t>(d) < dims) put_half(sA1, kMlpRows, t, d, z[d]);
        for (uint32_t f = 0; f < kFourier; ++f) {
            float a = 0.0f;
#pragma unroll
            for (int d = 0; d < DP; ++d)
                if (static_cast<uint32_t>(d) < dims) a = fmaf(z[d], prm[L.proj + d * kFourier + f], a);
            float sv, cv;
            sincospif(2.0f * a, &sv, &cv);
            put_half(sA1, kMlpRows, t, dims + f, sv);
            put_half(sA1, kMlpRows, t, dims + kFourier + f, cv);
        }
        for (uint32_t f = L.feats; f < kMlpFeatMax; ++f) put_half(sA1, kMlpRows, t, f, 0.0f);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            for (uint32_t ks = 0; ks < k1; ++ks)
                mma_f16kind(tmem, mlp_desc(smem_addr(sA1), kMlpRows, ks), mlp_desc(smem_addr(sW1), kHidden, ks), idesc,
                            ks != 0);
            mma_commit(bar);
            ++commits;
        }
        bool ok = !*abort && mbar_wait(bar, phase, abort);
        phase ^= 1;
        float h[kHidden];
        if (__all_sync(0xFFFFFFFFu, ok)) {
            tc_fence_after();
            float v[32];
            tmem_ld32(tmem + ((warp * 32u) << 16), v);
#pragma unroll
            for (uint32_t i = 0; i < 32; ++i) h[i] = fmaxf(v[i] + sb[i], 0.0f);
            tmem_ld32(tmem + ((warp * 32u) << 16) + 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; ++i) h[32 + i] = fmaxf(v[i] + sb[32 + i], 0.0f);
        } else {
            ok = false;
            *abort = 1;
#pragma unroll
            for (uint32_t i = 0; i < kHidden; ++i) h[i] = 0.0f;
        }
#pragma unroll
        for (uint32_t i = 0; i < kHidden; ++i) put_half(sA2, kMlpRows, t, i, h[i]);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0 && !*abort) {
            tc_fence_after();
            for (uint32_t ks = 0; ks < kHidden / 16; ++ks)
                mma_f16kind(tmem + kHidden, mlp_desc(smem_addr(sA2), kMlpRows, ks), mlp_desc(smem_addr(sW2), kHidden, ks),
                            idesc, ks != 0);
            mma_commit(bar);
            ++commits;
        }
        __syncthreads();
        bool ok2 = !*abort && mbar_wait(bar, phase, abort);
        phase ^= 1;
        float y = b3;
        if (__all_sync(0xFFFFFFFFu, ok2)) {
            tc_fence_after();
            float v[32];
#pragma unroll
            for (uint32_t c = 0; c < 2; ++c) {
                tmem_ld32(tmem + ((warp * 32u) << 16) + kHidden + 32 * c, v);
#pragma unroll
                for (uint32_t i = 0; i < 32; ++i) y = fmaf(sb[2 * kHidden + 32 * c + i], fmaxf(v[i] + sb[kHidden + 32 * c + i], 0.0f), y);
            }
        } else {
            ok2 = false;
            *abort = 1;
        }
        if (live) {
            const float cap = user_radii ? user_radii[q] : max_d2;
            const bool good = ok && ok2;
            if (raw) raw[q] = good ? y : INFINITY;
            if (radii) radii[q] = good ? fminf(__expf(fminf(y + margin, 80.0f)), cap) : cap;
        }
        tc_fence_before();
        __syncthreads();  // every read of sA1, sA2 and TMEM is done before the next tile's writes
        if (*abort) break;
    }
    if (*abort && t == 0 && commits) {
        // The MMAs already issued finish before TMEM is released.
        volatile int never = 0;
        mbar_wait(bar, (commits - 1) & 1, &never);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

size_t mlp_tc_smem() { return 1024 + kMlpRows * 256 + kHidden * 256 + kMlpRows * 128 + kHidden * 128 + 3 * kHidden * 4 + 64; }

int model_predict(const float* d_prm, uint32_t dims, const float* d_x, uint32_t count, float max_d2,
                  const float* user_radii, float* d_radii, float* d_raw, cudaStream_t s, bool tensor_cores) {
    const ModelLayout L(dims);
    if (tensor_cores && L.feats <= kMlpFeatMax && count > 0) {
        const size_t smem = mlp_tc_smem();
        const uint32_t grid = std::min<uint32_t>(ceil_div(count, kMlpRows), 3u * static_cast<uint32_t>(sm_count()));
#define KNN_INFER_TC(D_)                                                                                           \
        if (dims <= D_) {                                                                                          \
            KNN_TRY_CUDA(cudaFuncSetAttribute(mlp_infer_tc_kernel<D_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                              static_cast<int>(smem)));                                            \
            mlp_infer_tc_kernel<D_><<<grid, kMlpRows, smem, s>>>(d_prm, dims, d_x, count, max_d2, user_radii,      \
                                                                 d_radii, d_raw);                                  \
            KNN_LAUNCHED();                                                                                        \
            return KNN_OK;                                                                                         \
        }
        KNN_INFER_TC(4)
        KNN_INFER_TC(8)
        KNN_INFER_TC(16)
        KNN_INFER_TC(32)
        KNN_INFER_TC(64)
#undef KNN_INFER_TC
    }
    const size_t smem = (static_cast<size_t>((L.total + 3) & ~3u) + kHidden * L.feats) * sizeof(float);
    const bool aligned = (L.w2 % 4) == 0;
#define KNN_INFER(D_)                                                                                     \
    if (aligned && dims <= D_) {                                                                          \
        KNN_TRY_CUDA(cudaFuncSetAttribute(mlp_infer_fast_kernel<D_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                          static_cast<int>(smem)));                                       \
        mlp_infer_fast_kernel<D_><<<ceil_div(count, 256), 256, smem, s>>>(d_prm, dims, d_x, count, max_d2, \
                                                                          user_radii, d_radii, d_raw);    \
        KNN_LAUNCHED();                                                                                   \
        return KNN_OK;                                                                                    \
    }
    KNN_INFER(4)
    KNN_INFER(8)
    KNN_INFER(16)
#undef KNN_INFER
    mlp_infer_kernel<<<ceil_div(count, 128), 128, 0, s>>>(d_prm, dims, d_x, count, max_d2, user_radii, d_radii,
                                                          d_raw);
    KNN_LAUNCHED();
    return KNN_OK;
}

size_t retry_scratch_bytes(uint32_t count) {
    return 2 * static_cast<size_t>(ceil_div(count, kCompactThreads)) * sizeof(uint32_t) + 512;
}

int model_retry_list(const uint32_t* order, const int32_t* out_idx, uint32_t count, uint32_t k, float* seeded,
                     float max_d2, const float* user_radii, float grow, uint32_t* list, uint32_t* list_count,
                     void* scratch, DevCounters* counters, cudaStream_t s) {
    const uint32_t nblk = ceil_div(count, kCompactThreads);
    uint32_t* bcnt = static_cast<uint32_t*>(scratch);
    uint32_t* bpre = bcnt + nblk;
    retry_count_kernel<<<nblk, kCompactThreads, 0, s>>>(order, count, out_idx, k, seeded, max_d2, user_radii, bcnt);
    KNN_LAUNCHED();
    KNN_TRY(scan_rows_exclusive(bcnt, bpre, 1, nblk, s));
    retry_scatter_kernel<<<nblk, kCompactThreads, 0, s>>>(order, count, out_idx, k, seeded, max_d2, user_radii, bpre,
                                                          nblk, grow, list, list_count, counters);
    KNN_LAUNCHED();
    return KNN_OK;
}

int model_train(knn_index* ix, const float* d_samples, uint32_t count, uint32_t k, const knn_train_opts& o,
                cudaStream_t s, knn_train_report* rep) {
    const uint32_t dims = ix->dims;
    const ModelLayout L(dims);
    cudaEvent_t e0, e1;
    KNN_TRY_CUDA(cudaEventCreate(&e0));
    KNN_TRY_CUDA(cudaEventCreate(&e1));
    KNN_TRY_CUDA(cudaEventRecord(e0, s));

    // 1. Exact k-th distances of the samples, from the engine's own plain search.
    DevBuf buf;
    const size_t ck = static_cast<size_t>(count) * k;
    const size_t pb = static_cast<size_t>(L.total) * 4;
    KNN_TRY(buf.alloc(carve_bytes({ck * 4, ck * 4, static_cast<size_t>(count) * 4, static_cast<size_t>(count) * 4,
                                   pb, pb, pb, pb, static_cast<size_t>(o.batch) * 4})));
    Carver c(buf.ptr);
    int32_t* idx = c.take<int32_t>(ck);
    float* dist = c.take<float>(ck);
    float* target = c.take<float>(count);
    uint32_t* rows = c.take<uint32_t>(count);
    float* prm = c.take<float>(L.total);
    float* grad = c.take<float>(L.total);
    float* m = c.take<float>(L.total);
    float* v = c.take<float>(L.total);
    float* loss_rows = c.take<float>(o.batch);
    QueryArgs qa{d_samples, count, INFINITY, nullptr, k, idx, dist, nullptr};
    QueryPlan plan;
    switch (ix->structure) {
        case KNN_BRUTE_FORCE: KNN_TRY(bf_query(ix, qa, plan, s)); break;
        case KNN_KD_TREE: KNN_TRY(kd_query(ix, qa, plan, s)); break;
        default: KNN_TRY(ball_query(ix, qa, plan, s)); break;
    }
    kth_log_kernel<<<ceil_div(count, 256), 256, 0, s>>>(dist, idx, count, k, target);
    KNN_LAUNCHED();

    // 2. Input normalisation and initial weights (seeded, He-style scaling), on the host.
    std::vector<float> hx(static_cast<size_t>(count) * dims), ht(count);
    KNN_TRY_CUDA(cudaMemcpyAsync(hx.data(), d_samples, hx.size() * 4, cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaMemcpyAsync(ht.data(), target, ht.size() * 4, cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    std::vector<float> hp(L.total, 0.0f);
    for (uint32_t d = 0; d < dims; ++d) {
        float lo = INFINITY, hi = -INFINITY;
        for (uint32_t i = 0; i < count; ++i) {
            lo = std::min(lo, hx[static_cast<size_t>(i) * dims + d]);
            hi = std::max(hi, hx[static_cast<size_t>(i) * dims + d]);
        }
        hp[L.lo + d] = lo;
        hp[L.inv_range + d] = hi > lo ? 1.0f / (hi - lo) : 1.0f;
    }
    double tmean = 0;
    for (float t : ht) tmean += t;
    tmean /= std::max(1u, count);
    std::mt19937 gen(o.seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    for (uint32_t i = 0; i < dims * kFourier; ++i) hp[L.proj + i] = nd(gen) * kFourierScale;
    for (uint32_t i = 0; i < kHidden * L.feats; ++i) hp[L.w1 + i] = nd(gen) * std::sqrt(2.0f / L.feats);
    for (uint32_t i = 0; i < kHidden * kHidden; ++i) hp[L.w2 + i] = nd(gen) * std::sqrt(2.0f / kHidden);
    for (uint32_t i = 0; i < kHidden; ++i) hp[L.w3 + i] = nd(gen) * std::sqrt(1.0f / kHidden);
    hp[L.b3] = static_cast<float>(tmean);
    KNN_TRY_CUDA(cudaMemcpyAsync(prm, hp.data(), hp.size() * 4, cudaMemcpyHostToDevice, s));
    KNN_TRY_CUDA(cudaMemsetAsync(m, 0, L.total * 4, s));
    KNN_TRY_CUDA(cudaMemsetAsync(v, 0, L.total * 4, s));

    // 3. Adam over shuffled minibatches.
    std::vector<uint32_t> perm(count);
    for (uint32_t i = 0; i < count; ++i) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), gen);
    KNN_TRY_CUDA(cudaMemcpyAsync(rows, perm.data(), count * 4, cudaMemcpyHostToDevice, s));
    DevBuf scratch;
    const uint32_t batch = std::min(o.batch, count);
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.0f, c2 = 1.0f;
    uint32_t offset = 0;
    for (uint32_t step = 0; step < o.steps; ++step) {
        if (offset + batch > count) offset = 0;
        KNN_TRY(model_gradients(prm, dims, d_samples, target, rows + offset, batch, grad, loss_rows, scratch, s));
        c1 *= b1;
        c2 *= b2;
        const float lr = o.lr * 0.5f * (1.0f + std::cos(3.14159265f * static_cast<float>(step) / o.steps));
        adam_kernel<<<ceil_div(L.trainable, 256), 256, 0, s>>>(prm, grad, m, v, L.trainable, lr, b1, b2, 1e-8f,
                                                              1.0f - c1, 1.0f - c2);
        KNN_LAUNCHED();
        offset += batch;
    }
    std::vector<float> hl(batch);
    KNN_TRY_CUDA(cudaMemcpyAsync(hl.data(), loss_rows, batch * 4, cudaMemcpyDeviceToHost, s));

    // 4. Margin: the `coverage` quantile of (target - prediction) over the samples.
    // (with the query path's tensor-core inference, so that the margin covers its predictions)
    KNN_TRY(model_predict(prm, dims, d_samples, count, INFINITY, nullptr, nullptr, dist, s, true));
    std::vector<float> pred(count);
    KNN_TRY_CUDA(cudaMemcpyAsync(pred.data(), dist, count * 4, cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    std::vector<float> resid(count);
    double sse = 0;
    for (uint32_t i = 0; i < count; ++i) {
        resid[i] = ht[i] - pred[i];
        sse += static_cast<double>(resid[i]) * resid[i];
    }
    std::vector<float> sorted = resid;
    const uint32_t qi = std::min<uint32_t>(count - 1, static_cast<uint32_t>(std::ceil(o.coverage * count)));
    std::nth_element(sorted.begin(), sorted.begin() + qi, sorted.end());
    const float margin = sorted[qi] + 1e-3f;
    KNN_TRY_CUDA(cudaMemcpyAsync(prm + L.margin, &margin, 4, cudaMemcpyHostToDevice, s));

    KNN_TRY(ix->model.alloc(L.total * 4));
    KNN_TRY_CUDA(cudaMemcpyAsync(ix->model.ptr, prm, L.total * 4, cudaMemcpyDeviceToDevice, s));
    KNN_TRY_CUDA(cudaEventRecord(e1, s));
    KNN_TRY_CUDA(cudaEventSynchronize(e1));
    ix->has_model = true;
    ix->model_k = k;
    ix->model_margin = margin;
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        KNN_TRY_CUDA(cudaEventElapsedTime(&rep->train_ms, e0, e1));
        double bl = 0;
        for (float l : hl) bl += l;
        rep->final_batch_loss = static_cast<float>(bl);
        rep->rmse = static_cast<float>(std::sqrt(sse / count));
        rep->margin = margin;
        uint32_t covered = 0;
        for (float r : resid) covered += r <= margin ? 1u : 0u;
        rep->coverage = static_cast<float>(covered) / count;
        rep->samples = count;
        rep->steps = o.steps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return KNN_OK;
}

}  // namespace knn
