// Exact kNN through a 16-bit tensor-core filter (tcgen05, sm_103a) with cell skipping and exact
// FP32 rescoring, for any index (brute force, k-d tree, ball tree).
//
// The reference computes every pair's distance with SIMT FP32 (src/BruteForceGpu.cuh:9-31) or
// walks a tree per query (src/KdTreeGpu.cuh:392-410, src/BallTreeGpu.cuh:630-648).  Here:
//
// Layout, once per index.  Up to 32 dims, the cells are the leaves of a tile-aligned partition
// tree (each node sends the first half of its tiles, by its widest dimension, to the left child),
// so every cell is a compact run of whole tiles with a tight axis-aligned box.  Beyond 32 dims,
// landmarks (every (n/L)-th point, L about n/1024; cells much wider than the median cell get a
// second landmark at their farthest point, twice) split the points into Voronoi cells.  The points
// are laid out cell by cell in tiles of 256 rows, each cell's last tile padded (tree cells have
// only the last tile of all partial).  Every cell gets a centre (the mean of its points) and a radius bounding the
// exact distance from the centre to each of its points.  The operand images hold every row, and
// every cell centre, scaled by s = 2^e (e >= 0, largest |coordinate| * s in [2^13, 2^14)) and
// rounded to FP16; data whose largest |coordinate| exceeds 2^14 uses BF16 with s = 1.
//
// Per query batch.  Each query goes to its cell (the leaf it descends to, or its nearest
// landmark's cell) and the batch is sorted by cell.  A run of 128 sorted queries (a query tile) has a home range: the cells of its queries,
// widened by whole cells to at least max(2k, 512) points.  One CTA per query tile, over a
// sequence of 256-row tiles:
//   phase 1   the home tiles: each query's running k-th upper bound T;
//   centres   the cell-centre tiles: per query and cell, a rigorous lower bound on the distance
//             from the query to any point of the cell (the GEMM bound below, less the radius);
//             a cell is kept when some query of the tile may need it;
//   phase 2   the tiles of every kept cell outside the home range.
// Per tile, warp 1 issues tcgen05.mma (M = 128 queries, N = 256 rows, K = 16 per step over the
// padded dims) into one of two TMEM accumulators, warp 0 streams the operand tile and its row data
// by bulk asynchronous copy, and warps 2-5 read accumulator rows (thread = query).  The exact
// rescoring then ranks the candidates by the reference's own sequential FP32 squared-difference
// sum, so every answer is the plain search's.  Queries whose candidates overflow the list, or that
// the 16-bit format cannot hold, take the plain search.
//
// GEMM bound.  q', p' are scaled FP32 vectors (exact: s is a power of two >= 1), u the format's
// unit roundoff (2^-11 FP16, 2^-8 BF16), delta the largest absolute rounding error of a value in
// the subnormal range (2^-14 for FP16, which also covers flushing to zero; negligible for BF16).
// With G the FP32-accumulated tensor-core sum of the rounded products:
//   |G - q'.p'| <= E = c1 |q'||p'| + c3 (|q'| + |p'|) + c4,
//   c1 = (2u + u^2 + D 2^-20 (1+u)^2)(1 + 2^-10),  c3 = 1.01 delta (1+u) sqrt(D),
//   c4 = 1.01 D delta^2 + 2 s^2 (D+4) 2^-149   (the last term: float distances in the subnormal range)
// (product rounding summed by Cauchy-Schwarz; FP32 accumulation of D products within D 2^-20 of
// their magnitude sum, 8x the bound for truncating every addition).  The float norms n = fl(|x'|^2)
// have relative error below gn = (D+4) 2^-23, so the exact scaled distance S' = s^2 S obeys
//   (1-gn)(n_q + n_p) - 2G - 2E  <=  S'  <=  (1+gn)(n_q + n_p) - 2G + 2E,
// and the engine's float distance S_f obeys S (1-g) <= S_f <= S (1+g), g = (D+4) 2^-23.
//
// Candidate test (point tiles).  With Pmax >= |p'| over the tile, a point can be among a query's k
// nearest (ties included) only if
//   G - a n_p  >=  a n_q - E(Pmax) - T' / (2 (1-g)),    a = (1-gn)/2,
// where T' is the k-th smallest upper bound (1+g)((1+gn)(n_q+n_p) - 2G + 2E(Pmax)) seen so far.
// The epilogue rounds the left side up (one FMA) and the right side down (once per tile and per
// change of T'), so the filter can only keep extra candidates.
//
// T' itself.  Each query thread buffers the upper bounds below its current T' as 16-bit codes
// relative to T' (code c stands for the float whose bits are bits(T') - c 2^13, never below the
// value it records; far values saturate, which only rounds them up).  Once a row holds k codes
// (the first time) or max(16, k/4) more than its last flush kept, its warp flushes: per query the
// largest code c with at least k codes >= c (bisection over its bits)
// gives the new T' (at least k recorded upper bounds lie at or below it) and the codes >= c stay,
// re-based by subtracting c (exact).  Any T' at or above the k-th smallest of some set of recorded
// upper bounds is correct; a lazily tightened one only keeps a few extra candidates, against a
// heap update per candidate (k up to 128 entries, one thread each) that serialised the epilogue.
// Where two blocks per SM still fit it (dims <= 32, or small k), T' is instead kept exact by a heap
// of the k smallest upper bounds per query (one update per candidate below T'): at a few candidates
// per query and tile that costs less than the flushes (C3's shape); with many, a flush every
// max(16, k/4) codes costs less than that many heap updates of up to 7 levels (C4's shape).
//
// Cell test (centre tiles).  For a cell of centre c' and radius R' (scaled), every point p' of it
// has |q' - p'| >= |q' - c'| - R', so no point of the cell can reach a query's k nearest when
//   S_lo = (1-gn)(n_q + n_c) - 2G - 2E(Cmax)  >  (R' + t)^2,   t >= sqrt((T' + c4) / (1 - g)).
// The left side is rounded down and the right side up.

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>
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
constexpr uint32_t kCellPoints = 1024;
constexpr uint32_t kMaxCells = 4096;
constexpr uint32_t kMaskWords = kMaxCells / 32;
constexpr uint32_t kBoxMaxDims = 32;  // the tree layout and its box test up to this many dims
constexpr uint32_t kRowData = 2 * kTileN;  // floats of row data per tile: norms, then (centres) radii
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kStage = 16;               // accumulator values staged per thread (half a chunk)
constexpr uint32_t kCodeShift = 13;           // a bound code's unit: 2^13 float bits (<= 2^-10 relative)
constexpr uint32_t kCentreBit = 0x80000000u;  // item code: a centre tile
constexpr uint32_t kBoundary = 0xFFFFFFFEu;   // item code: centre tiles done, mask next
constexpr uint32_t kEnd = 0xFFFFFFFDu;        // item code: no more items

// Operand image layout code (the template parameter H of the GEMM kernels): 1 or 2 = that many
// blocks of 64 elements in 128-byte rows (128-byte swizzle), for more than 32 dims; 32 or 64 = one
// block of 16 or 32 elements in 32- or 64-byte rows (32- or 64-byte swizzle), for up to 16 or 32
// dims, so that narrow data moves no zero padding.
__host__ __device__ constexpr uint32_t ly_row_bytes(uint32_t ly) { return ly >= 32 ? ly : 128u; }
__host__ __device__ constexpr uint32_t ly_blocks(uint32_t ly) { return ly >= 32 ? 1u : ly; }
__host__ __device__ constexpr uint32_t ly_elems(uint32_t ly) { return ly_blocks(ly) * ly_row_bytes(ly) / 2; }
__host__ __device__ __forceinline__ uint32_t a_bytes(uint32_t ly) { return ly_blocks(ly) * kTileM * ly_row_bytes(ly); }
__host__ __device__ __forceinline__ uint32_t b_bytes(uint32_t ly) { return ly_blocks(ly) * kTileN * ly_row_bytes(ly); }
// Descriptors of K step ks (16 elements) of a `rows`-row operand image at shared address base.
__device__ __forceinline__ uint64_t ly_desc(uint32_t ly, uint32_t base, uint32_t rows, uint32_t ks) {
    const uint32_t W = ly_row_bytes(ly), per = W / 32;
    return desc_sw(base + (ks / per) * rows * W + (ks % per) * 32u, W);
}

// Constants of the GEMM bound (scaled units).
struct Bounds {
    float c1, c3, c4;  // |G - q'.p'| <= c1 |q'||p'| + c3 (|q'| + |p'|) + c4
    float gn;          // relative error of the float norms
    float g;           // relative error of the engine's float distance
    float inv_one_m;   // >= 1 / (1 - g)
};

struct TcParams {
    const uint8_t* qimg;         // [qtiles][H][128 rows][128 B]
    const uint8_t* pimg;         // [ptiles][H][256 rows][128 B]
    const uint8_t* cimg;         // [ctiles][H][256 rows][128 B] cell centres
    const float* qnorm;          // per query row: n_q (NaN: not representable, plain search)
    const float* pnorm;          // per padded point row: n_p (+inf on padding rows)
    const float* cdata;          // per centre tile: 256 norms (+inf past the last cell), 256 radii
    const float* pmax;           // per point tile: >= |p'|
    const float* cmax;           // per centre tile: >= |c'|
    const uint32_t* cell_tile;   // [cells + 1] first point tile of each cell
    const uint32_t* qhome;       // per query tile: first tile, end tile, first cell, last cell
    const float* box;            // tree layout: per cell [2][BD] scaled box (minima, maxima)
    const float* queries;        // the caller's queries (for the box test)
    uint32_t dims;
    float scale;
    uint32_t cells, ctiles, nq, ksteps, idesc, idesc_half;  // instruction descriptors: N = 256, 128
    uint32_t qtiles;             // query tiles; blocks take the ones past gridDim.x from tile_counter
    uint32_t* tile_counter;      // zero before the launch
    Bounds b;
    float s2, max_d2;
    const float* radii;          // per query index, or null
    const float* seed;           // per query index: an upper bound on its k-th float distance
    const uint32_t* order;       // row -> query index
    const uint32_t* live_count;  // rows in use (device), or null for nq
    uint32_t k, cap;
    uint32_t codes;              // bound codes buffered per query row (a multiple of 16, >= k + 48)
    uint32_t* cand;              // [nq][cap] padded point rows
    float* cand_v;               // [nq][cap] their tensor-core sums G
    uint32_t* cand_count;        // [nq]; kNone = plain search
    float* final_t;              // [nq] the row's k-th upper bound T' after the last tile
    DevCounters* counters;
    int* error;
    uint32_t give_up;            // tests: the producer gives up after its first point-tile copy
};

// Heap of a thread's k smallest upper bounds (max at slot 0), slot-major in shared memory.
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

// A thread's buffered upper bounds: 16-bit codes relative to its bound T (see the header), four
// per 8-byte word, word-major in shared memory (word w of row `row` at base[w * kTileM + row]);
// slots at and past the thread's count hold 0.
__device__ __forceinline__ uint32_t bound_code(float T, float u) {  // 0 <= u < T
    return min((__float_as_uint(T) - __float_as_uint(u)) >> kCodeShift, 0xFFFFu);
}
__device__ __forceinline__ void put_code(uint16_t* codes, uint32_t row, uint32_t e, uint32_t code) {
    codes[((e >> 2) * kTileM + row) * 4 + (e & 3)] = static_cast<uint16_t>(code);
}
__device__ __forceinline__ uint32_t codes_at_least(uint2 w, uint32_t c) {
    return ((w.x & 0xFFFFu) >= c) + ((w.x >> 16) >= c) + ((w.y & 0xFFFFu) >= c) + ((w.y >> 16) >= c);
}

// The tile sequence of a query tile, identical for every role: home tiles [t0, t1), the centre
// tiles, then (after the mask is complete) the tiles of each kept cell outside [c0, c1].
struct TileSeq {
    uint32_t t0, t1, c0, c1, cells, ctiles;
    const uint32_t* mask;       // shared memory, kMaskWords words
    const uint32_t* cell_tile;  // global
    uint32_t stage = 0;         // 0 home, 1 centres, 2 kept cells
    uint32_t t = 0, tend = 0, word = 0, bits = 0;
    // Next item; *centre tells the kind.  Returns false at the end of stages 0-1 (the caller
    // then starts the next stage) and at the very end.
    __device__ __forceinline__ bool next(uint32_t* item, bool* centre) {
        if (stage == 0) {
            if (t < t1) {
                *item = t++;
                *centre = false;
                return true;
            }
            return false;
        }
        if (stage == 1) {
            if (t < ctiles) {
                *item = t++;
                *centre = true;
                return true;
            }
            return false;
        }
        while (t >= tend) {
            while (bits == 0) {
                if (++word >= kMaskWords || word * 32 >= cells) return false;
                bits = mask[word];
            }
            const uint32_t c = word * 32 + static_cast<uint32_t>(__ffs(bits) - 1);
            bits &= bits - 1u;
            if (c >= cells) return false;
            if (c >= c0 && c <= c1) continue;
            t = __ldg(cell_tile + c);
            tend = __ldg(cell_tile + c + 1);
        }
        *item = t++;
        *centre = false;
        return true;
    }
    __device__ __forceinline__ void begin(uint32_t st) {
        stage = st;
        if (st == 0) t = t0;
        if (st == 1) t = 0;
        if (st == 2) {
            t = tend = 0;
            word = 0;
            bits = mask[0];
        }
    }
};


// ACC accumulators of kTileN TMEM columns: 2 lets the MMAs of the next tile run while the
// epilogue drains this one (one block per SM); 1 leaves room for two blocks per SM, whose
// epilogues then hide each other's latencies.
// BD > 0 (tree layout): after the centre test, the kept cells are re-tested against the exact
// distance from each query to each cell's axis-aligned box (the query's BD scaled coordinates in
// registers).
// HEAP: T' from a heap of k bounds per query row (in the codes' place) instead of buffered codes.
template <uint32_t H, uint32_t ACC, uint32_t BD, bool HEAP>
__global__ void __launch_bounds__(kThreads, 1) tc_filter_kernel(const TcParams p) {
    constexpr uint32_t kCols = ACC * kTileN;
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the 128-byte swizzle atoms.
    const uint32_t raw = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* sA = smem;
    uint8_t* sB0 = sA + a_bytes(H);
    uint8_t* sB1 = sB0 + b_bytes(H);
    float* sN = reinterpret_cast<float*>(sB1 + b_bytes(H));       // [2][kRowData] row data
    uint2* sCodes = reinterpret_cast<uint2*>(sN + 2 * kRowData);       // [codes / 4][kTileM] bound codes
    uint32_t* sMask = reinterpret_cast<uint32_t*>(sCodes + static_cast<size_t>(p.codes / 4) * kTileM);  // [kMaskWords]
    uint32_t* sItem = sMask + kMaskWords;                              // [2] item code per stage
    float* sMeta = reinterpret_cast<float*>(sItem + 2);                // [2] its norm bound (Pmax/Cmax)
    float* sStage = sMeta + 2;                                         // [kStage][kTileM] staged sums
    uint64_t* bars = reinterpret_cast<uint64_t*>(sStage + kStage * kTileM);
    uint64_t* full = bars;            // [2] tile (operands + row data) landed
    uint64_t* empty = bars + 2;       // [2] operands consumed by the MMAs
    uint64_t* acc_full = bars + 4;    // [2] accumulator ready
    uint64_t* acc_empty = bars + 6;   // [2] accumulator and row data drained by the epilogue
    uint64_t* a_full = bars + 8;      // query tile landed
    uint64_t* mask_ready = bars + 9;  // kept-cell mask complete
    // One accumulator (ACC = 1): each item's MMAs run in two halves of 128 columns, the low half
    // signalled on acc_lo_full and handed back on acc_lo_empty, so that the next item's low half
    // is computed while the epilogue reads this item's high half.
    uint64_t* acc_lo_full = bars + 10;   // [2]
    uint64_t* acc_lo_empty = bars + 12;  // [2]
    uint64_t* a_empty = bars + 14;       // the MMAs of a query tile are done with its operand
    uint64_t* epi_bar = bars + 15;       // the epilogue warps' own barrier (bounded waits)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 16);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t live_rows = p.live_count ? *p.live_count : p.nq;
    // The block's first query tile; later ones come from tile_counter, taken by the producer and
    // passed to the other roles with each tile's end marker.
    const uint32_t qt0 = blockIdx.x;
    if (qt0 * kTileM >= live_rows) return;  // whole block idle: leave before any allocation
    for (uint32_t w = threadIdx.x; w < kMaskWords; w += blockDim.x) sMask[w] = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(full + i, 1);
            mbar_init(empty + i, 1);
            mbar_init(acc_full + i, 1);
            mbar_init(acc_empty + i, kEpiWarps * 32);
            mbar_init(acc_lo_full + i, 1);
            mbar_init(acc_lo_empty + i, kEpiWarps * 32);
        }
        mbar_init(a_full, 1);
        mbar_init(a_empty, 1);
        mbar_init(epi_bar, kEpiWarps * 32);
        mbar_init(mask_ready, kEpiWarps * 32);
        *abort = 0;
        mbar_fence_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // The producer walks the tile sequence and publishes each stage's item in shared memory
    // (sItem: tile index, kCentreBit for centre tiles, or a marker) before its arrival on `full`;
    // the MMA issuer and the epilogue take the items from there, in order.
    if (warp == 0) {
        if (lane == 0) {
            uint32_t issued = 0, data_tiles = 0, tiles = 0, a_loads = 0;
            auto stage_free = [&](uint32_t s) -> bool {
                // Stage s is free once the MMAs of item issued-2 are done (operands) and the
                // epilogue has drained it (row data).
                if (issued < 2) return true;
                const uint32_t par = ((issued >> 1) - 1) & 1;
                return mbar_wait(empty + s, par, abort) && mbar_wait(acc_empty + s, par, abort);
            };
            auto load = [&](uint32_t item, bool centre) -> bool {
                const uint32_t s = issued & 1;
                if (!stage_free(s)) return false;
                sItem[s] = item | (centre ? kCentreBit : 0u);
                sMeta[s] = centre ? __ldg(p.cmax + item) : __ldg(p.pmax + item);
                const uint32_t rd_bytes = (centre ? kRowData : kTileN) * sizeof(float);
                mbar_expect_tx(full + s, b_bytes(H) + rd_bytes);
                const uint8_t* img = centre ? p.cimg : p.pimg;
                const float* rd = centre ? p.cdata + static_cast<size_t>(item) * kRowData
                                         : p.pnorm + static_cast<size_t>(item) * kTileN;
                bulk_copy_g2s(s ? sB1 : sB0, img + static_cast<size_t>(item) * b_bytes(H), b_bytes(H), full + s);
                bulk_copy_g2s(sN + s * kRowData, rd, rd_bytes, full + s);
                ++issued;
                data_tiles += centre ? 0u : 1u;
                return true;
            };
            // A marker item; `meta` travels in the stage's sMeta slot (the next tile, for kEnd).
            auto marker = [&](uint32_t code, uint32_t meta) -> bool {
                const uint32_t s = issued & 1;
                if (!stage_free(s)) return false;
                sItem[s] = code;
                sMeta[s] = __uint_as_float(meta);
                mbar_arrive(full + s);
                ++issued;
                return true;
            };
            bool ok = true;
            for (uint32_t qt = qt0;;) {
                // The query tile's operand, once the MMAs of the block's previous tile are done.
                if (tiles > 0 && !mbar_wait(a_empty, (tiles - 1) & 1, abort)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(a_full, a_bytes(H));
                bulk_copy_g2s(sA, p.qimg + static_cast<size_t>(qt) * a_bytes(H), a_bytes(H), a_full);
                ++a_loads;
                // (The kept-cell mask of the previous tile was read to the end; the epilogue writes
                // this tile's only after the centre items below.)
                if (tiles > 0)
                    for (uint32_t w = 0; w < kMaskWords; ++w) sMask[w] = 0;
                TileSeq seq;
                seq.t0 = p.qhome[4 * qt];
                seq.t1 = p.qhome[4 * qt + 1];
                seq.c0 = p.qhome[4 * qt + 2];
                seq.c1 = p.qhome[4 * qt + 3];
                seq.cells = p.cells;
                seq.ctiles = p.ctiles;
                seq.mask = sMask;
                seq.cell_tile = p.cell_tile;
                uint32_t item;
                bool centre;
                for (uint32_t st = 0; ok && st < 3; ++st) {
                    if (st == 2) ok = marker(kBoundary, 0) && mbar_wait(mask_ready, tiles & 1, abort) && !*abort;
                    seq.begin(st);
                    while (ok && seq.next(&item, &centre)) {
                        ok = load(item, centre);
                        if (p.give_up) ok = false;  // tests: as if the next wait had run out
                    }
                }
                uint32_t next = kNone;
                if (ok) {
                    const uint32_t t = gridDim.x + atomicAdd(p.tile_counter, 1u);
                    if (t < p.qtiles && t * kTileM < live_rows) next = t;
                }
                ok = ok && marker(kEnd, next);
                ++tiles;
                if (!ok || next == kNone) break;
                qt = next;
            }
            if (!ok) {
                *abort = 1;
                // Let copies in flight land before the block can exit.
                volatile int never = 0;
                if (a_loads) mbar_wait(a_full, (a_loads - 1) & 1, &never);
                for (uint32_t i = issued >= 2 ? issued - 2 : 0; i < issued; ++i)
                    mbar_wait(full + (i & 1), (i >> 1) & 1, &never);
            }
            if (p.counters && data_tiles) atomicAdd(&p.counters->leaves, static_cast<unsigned long long>(data_tiles));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: one accumulator per item; markers pass through.
            const uint32_t a0 = smem_addr(sA);
            uint32_t i = 0, tiles = 0, next = kNone;
            uint64_t* drain_bar = nullptr;  // the last commit's barrier and phase
            uint32_t drain_par = 0;
            bool ok = true;
            for (;;) {
            ok = mbar_wait(a_full, tiles & 1, abort);
            while (ok) {
                const uint32_t s = i & 1;
                // The accumulator this item writes is free once the epilogue has drained the item
                // that used it last: item i-2 (two accumulators) or i-1 (one).
                const uint32_t prev = i - ACC;
                if (!mbar_wait(full + s, (i >> 1) & 1, abort) ||
                    (ACC == 2 && i >= ACC && !mbar_wait(acc_empty + (prev & 1), (prev >> 1) & 1, abort))) {
                    ok = false;
                    break;
                }
                const uint32_t code = sItem[s];
                if (code == kBoundary || code == kEnd) {
                    if (code == kEnd) {
                        next = __float_as_uint(sMeta[s]);  // read before the stage is handed back
                        mma_commit(a_empty);  // the query operand is free once this tile's MMAs are done
                    }
                    mbar_arrive(empty + s);
                    if constexpr (ACC == 1) mbar_arrive(acc_lo_full + s);
                    mbar_arrive(acc_full + s);
                } else if constexpr (ACC == 2) {
                    tc_fence_after();
                    const uint32_t b0 = smem_addr(s ? sB1 : sB0);
                    for (uint32_t ks = 0; ks < p.ksteps; ++ks)
                        mma_f16kind(tmem + s * kTileN, ly_desc(H, a0, kTileM, ks), ly_desc(H, b0, kTileN, ks), p.idesc,
                                    ks != 0);
                    mma_commit(empty + s);
                    mma_commit(acc_full + s);
                    drain_bar = acc_full + s;
                    drain_par = (i >> 1) & 1;
                } else {
                    // Low half (rows 0-127 of the point tile into columns 0-127) once the previous
                    // item's low half is drained, then the high half once it is drained too.
                    const uint32_t b0 = smem_addr(s ? sB1 : sB0);
                    const uint32_t hb = b0 + 128u * ly_row_bytes(H);
                    if (i >= 1 && !mbar_wait(acc_lo_empty + (prev & 1), (prev >> 1) & 1, abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    for (uint32_t ks = 0; ks < p.ksteps; ++ks)
                        mma_f16kind(tmem, ly_desc(H, a0, kTileM, ks), ly_desc(H, b0, kTileN, ks), p.idesc_half, ks != 0);
                    mma_commit(acc_lo_full + s);
                    drain_bar = acc_lo_full + s;
                    drain_par = (i >> 1) & 1;
                    if (i >= 1 && !mbar_wait(acc_empty + (prev & 1), (prev >> 1) & 1, abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    for (uint32_t ks = 0; ks < p.ksteps; ++ks)
                        mma_f16kind(tmem + 128u, ly_desc(H, a0, kTileM, ks), ly_desc(H, hb, kTileN, ks), p.idesc_half,
                                    ks != 0);
                    mma_commit(empty + s);
                    mma_commit(acc_full + s);
                    drain_bar = acc_full + s;
                }
                ++i;
                if (code == kEnd) break;
            }
            if (!ok) break;
            ++tiles;
            if (next == kNone) break;
            }
            if (!ok) {
                *abort = 1;
                // The MMAs already issued finish before TMEM is released.
                volatile int never = 0;
                if (drain_bar) mbar_wait(drain_bar, drain_par, &never);
            }
        }
    } else {
        // Epilogue: thread = query row.  TMEM lanes 32*(warp%4) .. +31 belong to this warp.
        const uint32_t quarter = warp & 3;
        const uint32_t row = quarter * 32 + lane;
        uint32_t i = 0;  // items taken, over all of the block's tiles
        // The four epilogue warps meet here (an mbarrier with the kernel's bounded wait rather than
        // a named barrier, so that a warp that gives up cannot leave the others waiting forever).
        uint32_t epi_phase = 0;
        auto epi_sync = [&]() {
            mbar_arrive(epi_bar);
            mbar_wait(epi_bar, epi_phase & 1, abort);
            ++epi_phase;
        };
        for (uint32_t qt = qt0;;) {
        const uint32_t r = qt * kTileM + row;  // row of the sorted batch
        const bool live = r < live_rows;
        const uint32_t qi = live ? p.order[r] : 0u;
        const float nq = live ? p.qnorm[r] : 0.0f;
        const bool good = live && nq <= FLT_MAX;  // NaN or +inf: not representable
        const Bounds& b = p.b;
        float qb[BD > 0 ? BD : 1];
#pragma unroll
        for (uint32_t d = 0; d < (BD > 0 ? BD : 1); ++d)
            qb[d] = (BD > 0 && good && d < p.dims) ? p.queries[static_cast<size_t>(qi) * p.dims + d] * p.scale : 0.0f;
        const float r2 = fminf(p.radii ? fminf(p.radii[qi], p.max_d2) : p.max_d2, p.seed[qi]);
        const float seed = good ? __fmul_ru(r2, p.s2) : 0.0f;
        // (The seed bounds the k-th distance by itself; the buffer starts empty.)
        float T = seed;
        uint16_t* codes16 = reinterpret_cast<uint16_t*>(sCodes);
        // (Heap mode: the heap's k slots in the codes' place.)
        BoundHeap heap{reinterpret_cast<float*>(sCodes) + row, p.k};
        if constexpr (HEAP) {
            for (uint32_t x = 0; x < p.k; ++x) heap.at(x) = seed;
        } else {
            for (uint32_t w = 0; w < p.codes / 4; ++w) sCodes[w * kTileM + row] = make_uint2(0u, 0u);
        }
        uint32_t nb = 0;  // codes this row buffers
        uint32_t umax = 0;  // while T is infinite: the largest value buffered (its bits)
        bool home = true;  // no centre tile of this query tile seen yet
        // A flush is due once a row buffers this many codes: k for the first one (the seed is
        // usually loose), then max(16, k/4) more than a flush kept (a stale bound admits extra
        // candidates), within the room that leaves for one more chunk.
        uint32_t due = p.k;
        const uint32_t step = max(16u, p.k / 4);
        const float qup = good ? __fsqrt_ru(__fmul_ru(nq, __fadd_ru(1.0f, b.gn))) : 0.0f;  // >= |q'|
        const float one_m_gn = __fsub_rd(1.0f, b.gn);
        const float a = __fmul_rd(0.5f, one_m_gn);
        const float a_q = __fmul_rd(a, nq);
        const float up_n = __fadd_ru(1.0f, b.gn);
        const float up_g = __fadd_ru(1.0f, b.g);
        const float c1q = __fmul_ru(b.c1, qup);
        auto bound_e = [&](float pm) { return __fadd_ru(__fmaf_ru(c1q, pm, __fmul_ru(b.c3, __fadd_ru(qup, pm))), b.c4); };
        float E = 0.0f, theta0 = 0.0f, theta = INFINITY;
        auto set_theta = [&]() {
            const float tp = __fmul_ru(T, b.inv_one_m);  // >= T / (1 - g)
            theta = good ? fmaxf(__fsub_rd(theta0, __fmul_ru(0.5f, tp)), -FLT_MAX) : INFINITY;
        };
        // Tightens T from the buffered codes (warp-collective; every lane runs the same passes).
        auto flush = [&]() {
            if constexpr (HEAP) return;  // the heap's bound is always exact
            const bool finite = T <= FLT_MAX;
            if (__all_sync(0xFFFFFFFFu, nb < p.k)) return;
            const uint32_t words = (nb + 3) / 4;
            // Words in steps of four (codes is a multiple of 16; words past a row's count hold 0).
            const uint32_t wmax = (__reduce_max_sync(0xFFFFFFFFu, words) + 3) & ~3u;
            uint32_t top = 0;
            for (uint32_t w = 0; w < wmax; ++w) {
                const uint2 v = sCodes[w * kTileM + row];
                top = max(top, max(max(v.x & 0xFFFFu, v.x >> 16), max(v.y & 0xFFFFu, v.y >> 16)));
            }
            top = __reduce_max_sync(0xFFFFFFFFu, finite ? top : 0u);
            // The largest code c with at least k codes >= c, bit by bit from the top one present.
            uint32_t cstar = 0;
            for (int bit = top ? 31 - __clz(top) : -1; bit >= 0; --bit) {
                const uint32_t cand = cstar | (1u << bit);
                uint32_t n0 = 0, n1 = 0, n2 = 0, n3 = 0;
                for (uint32_t w = 0; w < wmax; w += 4) {
                    const uint2 v0 = sCodes[(w + 0) * kTileM + row], v1 = sCodes[(w + 1) * kTileM + row];
                    const uint2 v2 = sCodes[(w + 2) * kTileM + row], v3 = sCodes[(w + 3) * kTileM + row];
                    n0 += codes_at_least(v0, cand);
                    n1 += codes_at_least(v1, cand);
                    n2 += codes_at_least(v2, cand);
                    n3 += codes_at_least(v3, cand);
                }
                if ((n0 + n1) + (n2 + n3) >= p.k) cstar = cand;
            }
            if (!finite) {
                // An infinite bound carries no codes: the largest value buffered (at least k of
                // them lie at or below it) becomes T, and the buffer starts again.
                if (nb >= p.k) {
                    for (uint32_t w = 0; w < words; ++w) sCodes[w * kTileM + row] = make_uint2(0u, 0u);
                    nb = 0;
                    T = __uint_as_float(umax);
                    set_theta();
                }
            } else {
                // Keep the codes >= cstar, re-based to the new T (their values are unchanged); with
                // cstar = 0 (T stays) the codes 0, values within one unit of T, make room.
                const uint32_t keep = max(cstar, 1u);
                uint32_t kept = 0;
                for (uint32_t w = 0; w < words; ++w) {
                    const uint2 v = sCodes[w * kTileM + row];
                    const uint32_t cc[4] = {v.x & 0xFFFFu, v.x >> 16, v.y & 0xFFFFu, v.y >> 16};
#pragma unroll
                    for (uint32_t e = 0; e < 4; ++e)
                        if (cc[e] >= keep) put_code(codes16, row, kept++, cc[e] - cstar);
                }
                for (uint32_t e = kept; e < 4 * words; ++e) put_code(codes16, row, e, 0u);
                nb = kept;
                due = max(p.k, min(kept + step, p.codes - 32));
                if (cstar) {
                    T = __uint_as_float(__float_as_uint(T) - (cstar << kCodeShift));
                    set_theta();
                }
            }
        };
        uint32_t count = 0;
        uint32_t* my_cand = p.cand + static_cast<size_t>(live ? r : 0) * p.cap;
        float* my_v = p.cand_v + static_cast<size_t>(live ? r : 0) * p.cap;
        const uint32_t taddr_row = tmem + ((quarter * 32u) << 16);
        // Takes the next item (waits for its accumulator and row data); false on failure.
        auto take = [&](uint32_t* code) -> bool {
            const uint32_t s = i & 1;
            // The TMEM loads that follow are warp-collective: the whole warp proceeds or leaves.
            const bool got =
                mbar_wait((ACC == 1 ? acc_lo_full : acc_full) + s, (i >> 1) & 1, abort) && mbar_wait(full + s, (i >> 1) & 1, abort);
            if (!__all_sync(0xFFFFFFFFu, got)) return false;
            tc_fence_after();
            *code = sItem[s];
            return true;
        };
        // Hands the item's accumulator (and, with one accumulator, its low half when `marker`: a
        // marker has no half-way point) and row data back.
        auto release = [&](bool marker) {
            tc_fence_before();
            if (ACC == 1 && marker) mbar_arrive(acc_lo_empty + (i & 1));
            mbar_arrive(acc_empty + (i & 1));
            ++i;
        };
        // One accumulator: the low 128 columns are read; hand them back and wait for the high half.
        auto half_way = [&]() {
            tc_fence_before();
            mbar_arrive(acc_lo_empty + (i & 1));
            const bool got = mbar_wait(acc_full + (i & 1), (i >> 1) & 1, abort);
            if (!__all_sync(0xFFFFFFFFu, got)) *abort = 1;  // the next take() leaves
            tc_fence_after();
        };
        auto process = [&](uint32_t item, bool centre) {
            if (centre && home) {
                flush();  // the cell test with the tightest bound the home tiles give
                home = false;
            }
            const uint32_t s = i & 1;
            const float meta = sMeta[s];
            const float* rd = sN + s * kRowData;
            const uint32_t tcol = taddr_row + (ACC == 2 ? s * kTileN : 0u);
            // Chunks of 32 accumulator columns; the TMEM load of chunk c+1 is in flight while
            // chunk c is processed.
            uint32_t ra[32], rb[32];
            tmem_ld32_async(tcol, ra);
            tmem_wait_ld(ra);
            if (centre) {
                // Cell test: keep cell c when S_lo(q, c) <= (R_c + t)^2 for some query.
                const float Ec = bound_e(meta);
                const float base = __fsub_rd(__fmul_rd(one_m_gn, nq), __fmul_ru(2.0f, Ec));
                const float t2 = __fmul_ru(__fadd_ru(T, b.c4), b.inv_one_m);
                const float tq = __fsqrt_ru(t2);
                const float tq2 = __fmul_ru(tq, tq);
                const float tq_2 = __fmul_ru(2.0f, tq);
                auto chunk = [&](const uint32_t (&r)[32], uint32_t c) {
                    uint32_t bits = 0;
#pragma unroll
                    for (uint32_t j = 0; j < 32; ++j) {
                        const float cn = rd[c * 32 + j], cr = rd[kTileN + c * 32 + j];
                        const float s_lo = __fmaf_rd(-2.0f, __uint_as_float(r[j]), __fmaf_rd(one_m_gn, cn, base));
                        const float y = __fmaf_ru(cr, __fadd_ru(cr, tq_2), tq2);
                        bits |= !(s_lo > y) ? (1u << j) : 0u;
                    }
                    bits = __reduce_or_sync(0xFFFFFFFFu, good ? bits : 0u);
                    const uint32_t w = item * (kTileN / 32) + c;
                    if (lane == 0 && bits && w < kMaskWords) atomicOr(sMask + w, bits);
                };
                // (The TMEM loads and waits are warp-collective: the warp reconverges before each.)
#pragma unroll 1
                for (uint32_t c = 0; c < kTileN / 32; c += 2) {
                    tmem_ld32_async(tcol + (c + 1) * 32, rb);
                    chunk(ra, c);
                    __syncwarp();
                    tmem_wait_ld(rb);
                    if (c + 2 < kTileN / 32) {
                        if (ACC == 1 && c + 2 == kTileN / 64) half_way();
                        tmem_ld32_async(tcol + (c + 2) * 32, ra);
                    }
                    chunk(rb, c + 1);
                    __syncwarp();
                    if (c + 2 < kTileN / 32) tmem_wait_ld(ra);
                }
            } else {
                E = bound_e(meta);
                theta0 = __fsub_rd(a_q, E);
                set_theta();
                const float E2 = __fmul_ru(2.0f, E);
                const float4* pn4 = reinterpret_cast<const float4*>(rd);
                const uint32_t base = item * kTileN;
                float* stage = sStage + row;  // slot x at stage[x * kTileM]
                auto chunk = [&](const uint32_t (&r)[32], uint32_t c) {
                    // The hit mask of all 32 columns first, branch-free, in four independent
                    // partial masks; then, per half of 16 columns with hits, each lane walks its
                    // own hits (lanes side by side), recording candidates and their distance
                    // upper bounds.  A hit is tested again against the current theta first (theta
                    // only rises as T falls; testing against an older, lower theta only keeps
                    // extra candidates).
                    uint32_t mp[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                    for (uint32_t j4 = 0; j4 < 8; ++j4) {
                        const float4 n4 = pn4[c * 8 + j4];
                        const float nn[4] = {n4.x, n4.y, n4.z, n4.w};
#pragma unroll
                        for (uint32_t e = 0; e < 4; ++e) {
                            const uint32_t j = j4 * 4 + e;
                            mp[e] |= (__fmaf_ru(-a, nn[e], __uint_as_float(r[j])) >= theta) ? (1u << j) : 0u;
                        }
                    }
                    const uint32_t mask = (mp[0] | mp[1]) | (mp[2] | mp[3]);
                    if (mask == 0) return;
#pragma unroll
                    for (uint32_t half = 0; half < 2; ++half) {
                        uint32_t m = (mask >> (16 * half)) & 0xFFFFu;
                        if (m == 0) continue;
                        // This lane's 16 sums go to shared memory so that its hits can be taken
                        // bit by bit (registers cannot be indexed at run time).
#pragma unroll
                        for (uint32_t jj = 0; jj < 16; ++jj) stage[jj * kTileM] = __uint_as_float(r[half * 16 + jj]);
                        while (m) {
                            const uint32_t jj = static_cast<uint32_t>(__ffs(m) - 1);
                            m &= m - 1u;
                            const uint32_t j = half * 16 + jj;
                            const float vj = stage[jj * kTileM];
                            const float nj = rd[c * 32 + j];
                            if (!(__fmaf_ru(-a, nj, vj) >= theta)) continue;
                            if (count < p.cap) {
                                my_cand[count] = base + c * 32 + j;
                                my_v[count] = vj;
                            }
                            ++count;
                            // Upper bound of this pair's float distance (scaled).
                            const float hi = __fmaf_ru(-2.0f, vj, __fadd_ru(E2, __fmul_ru(up_n, __fadd_ru(nq, nj))));
                            const float u = __fmul_ru(fmaxf(hi, 0.0f), up_g);
                            if (u < T) {
                                if constexpr (HEAP) {
                                    heap.replace_top(u);
                                    T = heap.at(0);
                                    set_theta();
                                } else if (nb < p.codes) {
                                    put_code(codes16, row, nb++, bound_code(T, u));
                                    if (!(T <= FLT_MAX)) umax = max(umax, __float_as_uint(u));
                                }
                            }
                        }
                    }
                };
                // Buffered codes: a flush once some row of the warp is due (which also leaves room
                // for the next chunk's 32 columns).
                auto maybe_flush = [&]() {
                    if constexpr (!HEAP)
                        if (__any_sync(0xFFFFFFFFu, nb >= due)) flush();
                };
                // (The TMEM loads and waits are warp-collective: the warp reconverges before each.)
#pragma unroll 1
                for (uint32_t c = 0; c < kTileN / 32; c += 2) {
                    tmem_ld32_async(tcol + (c + 1) * 32, rb);
                    chunk(ra, c);
                    __syncwarp();
                    maybe_flush();
                    tmem_wait_ld(rb);
                    if (c + 2 < kTileN / 32) {
                        if (ACC == 1 && c + 2 == kTileN / 64) half_way();
                        tmem_ld32_async(tcol + (c + 2) * 32, ra);
                    }
                    chunk(rb, c + 1);
                    __syncwarp();
                    maybe_flush();
                    if (c + 2 < kTileN / 32) tmem_wait_ld(ra);
                }
            }
        };
        // Items until the end marker; at the boundary marker (every centre tile done) the
        // epilogue warps complete the kept-cell mask and release the producer into phase 2.  A
        // warp that fails still joins that barrier (once) before it leaves.
        bool ok = true, boundary_done = false;
        uint32_t next = kNone;
        auto boundary = [&]() {
            epi_sync();
            mbar_arrive(mask_ready);
            boundary_done = true;
        };
        for (;;) {
            uint32_t code = 0;
            if (!take(&code)) {
                ok = false;
                break;
            }
            if (code == kEnd) {
                flush();  // the final bound, for the rescoring
                next = __float_as_uint(sMeta[i & 1]);
                release(true);
                break;
            }
            if (code == kBoundary) {
                release(true);
                if constexpr (BD > 0) {
                    // Box test of every cell the centre test kept: each query's exact distance to
                    // the cell's box, lower-bounded with directed rounding; a cell stays when some
                    // query may need it.
                    epi_sync();  // the centre test's mask is complete
                    uint32_t* sNeed = reinterpret_cast<uint32_t*>(sStage);  // [kEpiWarps][kMaskWords]
                    const uint32_t ew = warp - 2, mwords = (p.cells + 31) / 32;
                    const float one_m_g = __fsub_rd(1.0f, b.g);
                    // Squared distance from the query to cell c's box, rounded down (16-byte loads,
                    // the same address in every lane).
                    auto box_d2 = [&](uint32_t c) {
                        const float4* bx = reinterpret_cast<const float4*>(p.box + static_cast<size_t>(c) * 2 * BD);
                        float acc = 0.0f;
#pragma unroll
                        for (uint32_t v = 0; v < BD / 4; ++v) {
                            const float4 lo4 = __ldg(bx + v), hi4 = __ldg(bx + BD / 4 + v);
                            const float lo[4] = {lo4.x, lo4.y, lo4.z, lo4.w}, hi[4] = {hi4.x, hi4.y, hi4.z, hi4.w};
#pragma unroll
                            for (uint32_t e = 0; e < 4; ++e) {
                                const float q = qb[4 * v + e];
                                const float gap = fmaxf(fmaxf(__fsub_rd(lo[e], q), __fsub_rd(q, hi[e])), 0.0f);
                                acc = __fmaf_rd(gap, gap, acc);
                            }
                        }
                        return acc;
                    };
                    for (uint32_t w = 0; w < mwords; ++w) {
                        uint32_t bits = good ? sMask[w] : 0u, need = 0;
                        // Two cells at a time at 16 dims (their loads and sums are independent;
                        // at 32 dims the second box would not fit the register budget).
                        while (bits) {
                            const uint32_t b0 = static_cast<uint32_t>(__ffs(bits) - 1);
                            bits &= bits - 1u;
                            const bool two = BD <= 16 && bits != 0;
                            const uint32_t b1 = two ? static_cast<uint32_t>(__ffs(bits) - 1) : b0;
                            if (two) bits &= bits - 1u;
                            const float d0 = box_d2(w * 32 + b0);
                            const float d1 = two ? box_d2(w * 32 + b1) : d0;
                            if (!(__fsub_rd(__fmul_rd(d0, one_m_g), b.c4) > T)) need |= 1u << b0;
                            if (!(__fsub_rd(__fmul_rd(d1, one_m_g), b.c4) > T)) need |= 1u << b1;
                        }
                        need = __reduce_or_sync(0xFFFFFFFFu, need);
                        if (lane == 0) sNeed[ew * kMaskWords + w] = need;
                    }
                    epi_sync();
                    for (uint32_t w = threadIdx.x - 64; w < mwords; w += kEpiWarps * 32)
                        sMask[w] &= sNeed[w] | sNeed[kMaskWords + w] | sNeed[2 * kMaskWords + w] | sNeed[3 * kMaskWords + w];
                }
                boundary();
                continue;
            }
            process(code & ~kCentreBit, (code & kCentreBit) != 0);
            release(false);
        }
        if (!ok) *abort = 1;
        if (!boundary_done) boundary();
        if (live) {
            p.cand_count[r] = (ok && good) ? count : kNone;
            p.final_t[r] = (ok && good) ? T : INFINITY;
        }
        if (!ok || next == kNone) break;
        qt = next;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*abort && threadIdx.x == 0) {
        atomicExch(p.error, 1);
        if (p.counters) atomicAdd(&p.counters->give_ups, 1);
    }
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, kCols);
    }
}

// Exact rescoring: the reference's sequential FP32 distance for every candidate, top-k by key.
// A candidate is skipped, without reading its row, when its GEMM lower bound already exceeds the
// row's final k-th upper bound T' (then its float distance exceeds the k-th one).  Rows whose
// candidate list overflowed (or whose block gave up, or that the 16-bit format could not hold) are
// listed for the plain search.
struct RescoreArgs {
    const float* pts;         // FP32 points per padded row (stride PS)
    const uint32_t* ids;      // point index per padded row
    const float* pnorm;       // scaled norm per padded row
    const float* pmax;        // per point tile
    const float* queries;
    uint32_t dims, nq, cap, k;
    float max_d2;
    const float* radii;
    const uint32_t* order;       // row -> query index
    const uint32_t* live_count;  // rows in use (device), or null for nq
    uint32_t* cand;           // per row: candidate positions (compacted in place by the rescoring)
    const float* cand_v;
    const uint32_t* cand_count;
    const float* qnorm;       // per row: scaled norm of the query
    const float* final_t;     // per row: T'
    Bounds b;
    int32_t* out_idx;
    float* out_dist;
    uint32_t* retry;
    uint32_t* retry_count;
    float* retry_r2;          // per query index: the radius its plain search may use
    float inv_s2;             // 1 / s^2
    DevCounters* counters;
    uint32_t buf;             // keys buffered per warp (rescore_buf(k))
    uint32_t warp_bytes;      // shared memory per warp
};

constexpr uint32_t kRescoreWarps = 4;  // most warps per block (one row each)

// Staging of candidate rows in shared memory: each warp copies the rows of 32 candidates at a time
// with coalesced 16-byte copies (one row of PS floats = kV lanes' worth), into slots of an odd
// number of 16-byte units so that lane l reading slot l with 16-byte loads hits distinct banks.
template <int PS>
struct RescoreShape {
    static constexpr uint32_t kV = PS / 4;                       // 16-byte units per row
    static constexpr uint32_t kSlot = (kV % 2) ? kV : kV + 1;    // 16-byte units per staged row
    static constexpr uint32_t kRowsPerCopy = 32 / kV;            // rows one warp-wide copy moves
    static constexpr uint32_t kStageBytes = 32 * kSlot * 16;     // 32 candidates
};

// Keys buffered per warp before a sort-and-trim: room for k kept keys plus one step of 32.
inline uint32_t rescore_buf(uint32_t k) {
    uint32_t b = 64;
    while (b < k + 32) b <<= 1;
    return b;
}

// Sorts buf[0, n) ascending (n a power of two) with the lanes of one warp.
__device__ __forceinline__ void warp_bitonic(uint64_t* buf, uint32_t n, uint32_t lane) {
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = lane; i < n / 2; i += 32) {
                const uint32_t lo = 2 * stride * (i / stride) + (i % stride);
                const uint32_t hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t x = buf[lo], y = buf[hi];
                if ((x > y) == up) {
                    buf[lo] = y;
                    buf[hi] = x;
                }
            }
            __syncwarp();
        }
    }
}

// The reference's sequential FP32 squared-difference sum of a query and a point row, both in shared
// memory (zero padded to PS: the padding adds fma(0, 0, acc) = acc).
template <int PS>
__device__ __forceinline__ float dist2_smem(const float4* __restrict__ q4, const float4* __restrict__ p4) {
    float acc = 0.0f;
#pragma unroll
    for (int v = 0; v < PS / 4; ++v) {
        const float4 q = q4[v], x = p4[v];
        float t = __fsub_rn(q.x, x.x);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q.y, x.y);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q.z, x.z);
        acc = __fmaf_rn(t, t, acc);
        t = __fsub_rn(q.w, x.w);
        acc = __fmaf_rn(t, t, acc);
    }
    return acc;
}

// One warp per row.  Phase 1 tests every candidate's GEMM lower bound and compacts the ones that
// must be rescored.  Phase 2 takes them 32 per step, one per lane: the warp copies their rows into
// one of two shared-memory stages (the copies of step j + 1 are in flight while step j is scored),
// each lane sums its own row in dimension order and the keys go to the warp's buffer; a full
// buffer is sorted and trimmed to the k smallest keys.
template <int PS, int S>
__global__ void __launch_bounds__(32 * kRescoreWarps) tc_rescore_kernel(const RescoreArgs a) {
    using Sh = RescoreShape<PS>;
    extern __shared__ __align__(16) uint8_t rs_smem[];
    const uint32_t lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const uint32_t r = blockIdx.x * (blockDim.x / 32) + w;  // row of the sorted batch
    if (r >= (a.live_count ? *a.live_count : a.nq)) return;  // warp-uniform
    uint8_t* mine = rs_smem + static_cast<size_t>(w) * a.warp_bytes;
    float4* stage = reinterpret_cast<float4*>(mine);                                   // [2][32][kSlot]
    float4* sq = reinterpret_cast<float4*>(mine + S * Sh::kStageBytes);               // [PS / 4]
    uint64_t* buf = reinterpret_cast<uint64_t*>(mine + S * Sh::kStageBytes + PS * 4);  // [a.buf]
    const uint32_t qi = a.order[r];
    const uint32_t cnt = a.cand_count[r];
    if (cnt > a.cap) {
        if (lane == 0) {
            // The plain search of this query may stop at the filter's final k-th upper bound:
            // at least k points lie within it, so the answer is unchanged.
            const float user = a.radii ? fminf(a.radii[qi], a.max_d2) : a.max_d2;
            a.retry_r2[qi] = fminf(user, __fmul_ru(a.final_t[r], a.inv_s2));
            a.retry[atomicAdd(a.retry_count, 1u)] = qi;
            if (a.counters) atomicAdd(&a.counters->fallback, 1ull);
        }
        return;
    }
    // The query, zero padded, in shared memory: every lane reads it (broadcast).
    float* sqf = reinterpret_cast<float*>(sq);
    for (uint32_t d = lane; d < static_cast<uint32_t>(PS); d += 32)
        sqf[d] = d < a.dims ? a.queries[static_cast<size_t>(qi) * a.dims + d] : 0.0f;
    const float r2 = a.radii ? fminf(a.radii[qi], a.max_d2) : a.max_d2;
    const uint64_t limit = make_key(r2, -1);  // the key an unfilled slot holds
    const Bounds& b = a.b;
    const float nq = a.qnorm[r];
    const float qup = __fsqrt_ru(__fmul_ru(nq, __fadd_ru(1.0f, b.gn)));
    const float one_m_gn = __fsub_rd(1.0f, b.gn);
    const float one_m_g = __fsub_rd(1.0f, b.g);
    const float c1q = __fmul_ru(b.c1, qup);
    const float tfin = a.final_t[r];
    uint32_t* c = a.cand + static_cast<size_t>(r) * a.cap;
    const float* cv = a.cand_v + static_cast<size_t>(r) * a.cap;
    // Phase 1: keep the candidates whose GEMM lower bound (s^2 times a lower bound of the pair's
    // float distance) does not exceed T', compacted in place at the front of the list.  Four
    // groups of 32 per pass, their loads independent.
    uint32_t kept = 0;
    for (uint32_t i0 = 0; i0 < cnt; i0 += 128) {
        uint32_t pos[4];
        float v[4], pm[4], pn[4];
#pragma unroll
        for (uint32_t u = 0; u < 4; ++u) {
            const uint32_t i = i0 + 32 * u + lane;
            pos[u] = i < cnt ? c[i] : 0u;
            v[u] = i < cnt ? cv[i] : 0.0f;
        }
#pragma unroll
        for (uint32_t u = 0; u < 4; ++u) {
            pm[u] = __ldg(a.pmax + pos[u] / kTileN);
            pn[u] = __ldg(a.pnorm + pos[u]);
        }
#pragma unroll
        for (uint32_t u = 0; u < 4; ++u) {
            const float E = __fadd_ru(__fmaf_ru(c1q, pm[u], __fmul_ru(b.c3, __fadd_ru(qup, pm[u]))), b.c4);
            const float lo = __fsub_rd(__fmaf_rd(-2.0f, v[u], __fmul_rd(one_m_gn, __fadd_rd(nq, pn[u]))),
                                       __fmul_ru(2.0f, E));
            const bool keep = i0 + 32 * u + lane < cnt && !(__fmul_rd(__fsub_rd(lo, b.c4), one_m_g) > tfin);
            // The ballot orders every lane's loads of this pass before any lane's store below.
            const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, keep);
            if (keep) c[kept + __popc(ballot & ((1u << lane) - 1u))] = pos[u];
            kept += __popc(ballot);
        }
    }
    __syncwarp();  // the compacted list and the query are visible to every lane
    // Phase 2: the kept rows, 32 per step, staged in shared memory and summed one per lane.
    auto stage_rows = [&](uint32_t st, uint32_t mask, uint32_t pos) {
        float4* dst = stage + st * 32 * Sh::kSlot;
        const uint32_t sub = lane / Sh::kV, v = lane % Sh::kV;
#pragma unroll 4
        for (uint32_t g = 0; g < 32; g += Sh::kRowsPerCopy) {
            uint32_t grp;
            if constexpr (Sh::kRowsPerCopy == 32) grp = mask;
            else grp = (mask >> g) & ((1u << Sh::kRowsPerCopy) - 1u);
            if (grp == 0) continue;  // warp-uniform
            const uint32_t slot = g + sub;
            const uint32_t src = __shfl_sync(0xFFFFFFFFu, pos, slot);
            if ((mask >> slot) & 1u) cp_async16(dst + slot * Sh::kSlot + v, a.pts + static_cast<size_t>(src) * PS + 4 * v);
        }
        cp_async_commit();
    };
    const uint32_t steps = (kept + 31) / 32;
    uint32_t m = 0;  // keys in the buffer
    bool need_c = lane < kept;
    uint32_t pos_c = need_c ? c[lane] : 0u;
    uint32_t id_c = need_c ? a.ids[pos_c] : 0u;
    // Appends this lane's key (if below the limit) to the warp's buffer, sorting and trimming it
    // to the k smallest first when it could overflow.
    auto append = [&](uint64_t key) {
        if (m + 32 > a.buf) {
            // Sort and keep the k smallest (the rest cannot be in the answer).
            uint32_t n2 = 1;
            while (n2 < m) n2 <<= 1;
            for (uint32_t t = m + lane; t < n2; t += 32) buf[t] = ~0ull;
            __syncwarp();
            warp_bitonic(buf, n2, lane);
            m = min(m, a.k);
        }
        const bool take = key < limit;
        const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, take);
        if (take) buf[m + __popc(ballot & ((1u << lane) - 1u))] = key;
        m += __popc(ballot);
        __syncwarp();  // the stage is read before the next copies overwrite it
    };
    if constexpr (S == 2) {
        // Two stages: the copies of step j + 1 are in flight while step j is summed.
        if (steps) stage_rows(0, __ballot_sync(0xFFFFFFFFu, need_c), pos_c);
        for (uint32_t j = 0; j < steps; ++j) {
            uint32_t pos_n = 0, id_n = 0;
            bool need_n = false;
            if (j + 1 < steps) {
                need_n = 32 * (j + 1) + lane < kept;
                if (need_n) {
                    pos_n = c[32 * (j + 1) + lane];
                    id_n = a.ids[pos_n];
                }
                stage_rows((j + 1) & 1, __ballot_sync(0xFFFFFFFFu, need_n), pos_n);
            } else {
                cp_async_commit();  // an empty group: the wait below always leaves the newest one
            }
            cp_async_wait<1>();
            __syncwarp();  // every lane's copies of step j have landed
            uint64_t key = ~0ull;
            if (need_c) key = make_key(dist2_smem<PS>(sq, stage + (j & 1) * 32 * Sh::kSlot + lane * Sh::kSlot),
                                       static_cast<int32_t>(id_c));
            append(key);
            pos_c = pos_n;
            id_c = id_n;
            need_c = need_n;
        }
    } else {
        // One stage (wide rows): more warps per SM hide the copies instead.
        for (uint32_t j = 0; j < steps; ++j) {
            if (j) {
                need_c = 32 * j + lane < kept;
                pos_c = need_c ? c[32 * j + lane] : 0u;
                id_c = need_c ? a.ids[pos_c] : 0u;
            }
            stage_rows(0, __ballot_sync(0xFFFFFFFFu, need_c), pos_c);
            cp_async_wait<0>();
            __syncwarp();
            uint64_t key = ~0ull;
            if (need_c) key = make_key(dist2_smem<PS>(sq, stage + lane * Sh::kSlot), static_cast<int32_t>(id_c));
            append(key);
        }
    }
    cp_async_wait<0>();
    uint32_t n2 = 1;
    while (n2 < m) n2 <<= 1;
    for (uint32_t t = m + lane; t < n2; t += 32) buf[t] = ~0ull;
    __syncwarp();
    if (m > 1) warp_bitonic(buf, n2, lane);
    for (uint32_t t = lane; t < a.k; t += 32) {
        const uint64_t key = t < m ? buf[t] : limit;
        a.out_idx[static_cast<size_t>(qi) * a.k + t] = t < m ? key_index(key) : -1;
        a.out_dist[static_cast<size_t>(qi) * a.k + t] = t < m ? key_dist(key) : r2;
    }
    if (a.counters && lane == 0) {
        atomicAdd(&a.counters->nodes, static_cast<unsigned long long>(kept));
        atomicAdd(&a.counters->points, static_cast<unsigned long long>(cnt));
    }
}

// Exhaustive search for the queries the filter could not settle (listed in `retry`, count on the
// device), split over at least kExhChunks blocks per query (more when few queries would leave most
// of the grid idle; the same count in both kernels): each block scans its share of the point rows
// with the reference's sequential FP32 distance, appends keys below the query's radius to a shared
// buffer that is sorted and trimmed to the k smallest whenever it fills (the radius then tightens
// to the k-th key), and writes its k smallest; a second kernel merges the chunks per query.
constexpr uint32_t kExhThreads = 256;
constexpr uint32_t kExhBuf = 2048;
constexpr uint32_t kExhRound = 4;    // points per thread between buffer checks
constexpr uint32_t kExhChunks = 8;      // blocks per query, at least
constexpr uint32_t kExhMaxChunks = 64;  // and at most

// More chunks only while each keeps at least kExhMinRows rows: the merge sorts chunks x k keys.
constexpr uint32_t kExhMinRows = 8192;
__host__ __device__ __forceinline__ uint32_t exh_chunks(uint32_t nretry, uint32_t blocks, uint32_t prows) {
    return nretry ? max(kExhChunks, min(min(kExhMaxChunks, blocks / nretry), prows / kExhMinRows)) : kExhChunks;
}

__device__ __forceinline__ void block_bitonic(uint64_t* buf, uint32_t n) {
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < n / 2; i += blockDim.x) {
                const uint32_t lo = 2 * stride * (i / stride) + (i % stride);
                const uint32_t hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t x = buf[lo], y = buf[hi];
                if ((x > y) == up) {
                    buf[lo] = y;
                    buf[hi] = x;
                }
            }
            __syncthreads();
        }
    }
}

// Sorts buf[0, *fill) (padding to a power of two), keeps the k smallest and lowers *limit below
// the k-th key.  Called by the whole block.
__device__ __forceinline__ void block_trim(uint64_t* buf, uint32_t* fill, uint64_t* limit, uint32_t k) {
    uint32_t n2 = 1;
    while (n2 < *fill) n2 <<= 1;
    for (uint32_t j = *fill + threadIdx.x; j < n2; j += blockDim.x) buf[j] = ~0ull;
    __syncthreads();
    block_bitonic(buf, n2);
    if (threadIdx.x == 0) {
        if (*fill >= k) *limit = min(*limit, buf[k - 1] + 1);  // keys above the k-th cannot enter
        *fill = min(*fill, k);
    }
    __syncthreads();
}

template <int PS>
__global__ void __launch_bounds__(kExhThreads) tc_exhaustive_kernel(const float* __restrict__ pts,
                                                                    const uint32_t* __restrict__ ids,
                                                                    const float* __restrict__ pnorm, uint32_t prows,
                                                                    const float* __restrict__ queries, uint32_t dims,
                                                                    uint32_t k, const uint32_t* __restrict__ retry,
                                                                    const uint32_t* __restrict__ retry_count,
                                                                    const float* __restrict__ retry_r2,
                                                                    uint64_t* __restrict__ xkeys) {
    __shared__ uint64_t buf[kExhBuf];
    __shared__ uint32_t fill;
    __shared__ uint64_t limit;
    const uint32_t nretry = *retry_count;
    const uint32_t chunks = exh_chunks(nretry, gridDim.x, prows);
    const uint32_t items = nretry * chunks;
    const uint32_t csize = (prows + chunks - 1) / chunks;
    for (uint32_t item = blockIdx.x; item < items; item += gridDim.x) {
        const uint32_t e = item / chunks, ch = item % chunks;
        const uint32_t qi = retry[e];
        float qv[PS];
#pragma unroll
        for (int d = 0; d < PS; ++d) qv[d] = static_cast<uint32_t>(d) < dims ? queries[static_cast<size_t>(qi) * dims + d] : 0.0f;
        if (threadIdx.x == 0) {
            fill = 0;
            limit = make_key(retry_r2[qi], -1);
        }
        __syncthreads();
        const uint32_t lo = ch * csize, hi = min(prows, lo + csize);
        for (uint32_t base = lo; base < hi; base += kExhThreads * kExhRound) {
            const uint64_t lim = limit;
#pragma unroll
            for (uint32_t u = 0; u < kExhRound; ++u) {
                const uint32_t pos = base + u * kExhThreads + threadIdx.x;
                if (pos < hi && pnorm[pos] <= FLT_MAX) {
                    const float d2 = dist2_vec4<PS>(qv, reinterpret_cast<const float4*>(pts + static_cast<size_t>(pos) * PS));
                    const uint64_t key = make_key(d2, static_cast<int32_t>(ids[pos]));
                    if (key < lim) buf[atomicAdd(&fill, 1u)] = key;
                }
            }
            __syncthreads();
            if (fill + kExhThreads * kExhRound > kExhBuf) block_trim(buf, &fill, &limit, k);
        }
        block_trim(buf, &fill, &limit, k);
        uint64_t* out = xkeys + (static_cast<size_t>(e) * chunks + ch) * k;
        for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) out[j] = j < fill ? buf[j] : ~0ull;
        __syncthreads();
    }
}

// Merges the partial lists of each retried query and writes its row (launched on the same grid as
// the scan, so that both count the same chunks; shared memory: the next power of two at or above
// kExhMaxChunks k keys).
__global__ void __launch_bounds__(kExhThreads) tc_exhaustive_merge_kernel(uint32_t k, uint32_t prows,
                                                                          const uint32_t* __restrict__ retry,
                                                                          const uint32_t* __restrict__ retry_count,
                                                                          const float* __restrict__ retry_r2,
                                                                          const uint64_t* __restrict__ xkeys,
                                                                          int32_t* __restrict__ out_idx,
                                                                          float* __restrict__ out_dist) {
    extern __shared__ uint64_t xbuf[];
    uint64_t* buf = xbuf;
    const uint32_t nretry = *retry_count;
    const uint32_t m = exh_chunks(nretry, gridDim.x, prows) * k;
    uint32_t n2 = 1;
    while (n2 < m) n2 <<= 1;
    for (uint32_t e = blockIdx.x; e < nretry; e += gridDim.x) {
        const uint32_t qi = retry[e];
        const float r2 = retry_r2[qi];
        for (uint32_t j = threadIdx.x; j < n2; j += blockDim.x)
            buf[j] = j < m ? xkeys[static_cast<size_t>(e) * m + j] : ~0ull;
        __syncthreads();
        block_bitonic(buf, n2);
        const uint64_t limit = make_key(r2, -1);
        for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) {
            const bool have = buf[j] < limit;
            out_idx[static_cast<size_t>(qi) * k + j] = have ? key_index(buf[j]) : -1;
            out_dist[static_cast<size_t>(qi) * k + j] = have ? key_dist(buf[j]) : r2;
        }
        __syncthreads();
    }
}

// One thread per padded row: gathers source row row_of[r] (identity when row_of is null; rows
// past the live count or mapped to kNone are padding), scales it by `scale`, rounds it to FP16 or
// BF16 into the 128-byte-swizzle image of `tile_rows`-row tiles with H 64-element halves, and
// writes the float norm of the scaled row (padding: pad_norm; not representable: NaN, and
// *bad is set).  Optionally keeps an unscaled FP32 copy (zero padded) and the row's point index.
__global__ void tc_pack_kernel(const float* __restrict__ src, uint32_t src_stride, uint32_t dims,
                               const uint32_t* __restrict__ row_of, uint32_t rows, const uint32_t* __restrict__ live_count,
                               uint32_t tile_rows, uint32_t H, bool f16, float scale, uint8_t* __restrict__ img,
                               float* __restrict__ norm, float pad_norm, float* __restrict__ copy, uint32_t copy_stride,
                               const uint32_t* __restrict__ src_ids, uint32_t* __restrict__ ids, uint32_t padded_rows,
                               int* __restrict__ bad) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= padded_rows) return;
    const uint32_t t = r / tile_rows, rr = r % tile_rows;
    uint8_t* base = img + static_cast<size_t>(t) * ly_blocks(H) * tile_rows * ly_row_bytes(H);
    const bool live = r < (live_count ? *live_count : rows);
    const uint32_t sr = live ? (row_of ? row_of[r] : r) : kNone;
    const bool valid = sr != kNone;
    float acc = 0.0f;
    bool inf = false;
    for (uint32_t k = 0; k < ly_elems(H); ++k) {
        const float x = (valid && k < dims) ? src[static_cast<size_t>(sr) * src_stride + k] : 0.0f;
        const float xs = x * scale;  // exact: scale is a power of two and the result stays finite
        acc = __fmaf_rn(xs, xs, acc);
        uint16_t bits;
        if (f16) {
            const __half h = __float2half_rn(xs);
            inf |= __hisinf(h) != 0 || __hisnan(h);
            bits = __half_as_ushort(h);
        } else {
            const __nv_bfloat16 h = __float2bfloat16_rn(xs);
            const float back = __bfloat162float(h);
            inf |= !(fabsf(back) <= FLT_MAX);
            bits = __bfloat16_as_ushort(h);
        }
        *reinterpret_cast<uint16_t*>(base + sw_offset(ly_row_bytes(H), tile_rows, rr, k)) = bits;
        if (copy && k < copy_stride) copy[static_cast<size_t>(r) * copy_stride + k] = x;
    }
    const bool ok = !inf && acc <= FLT_MAX;
    norm[r] = valid ? (ok ? acc : __int_as_float(0x7fc00000)) : pad_norm;
    if (valid && !ok && bad) atomicExch(bad, 1);
    if (ids) ids[r] = valid ? (src_ids ? src_ids[sr] : sr) : kNone;
}

// Nearest landmark (float distance, lowest index on ties) of each row; rows past the live count
// get key `cells`.  keys/vals are indexed by row; vals = the source row.  With `cell_far` (per
// cell: float squared distance from the landmark to its farthest point) and `cell_start`, also
// writes seed[source row]: an upper bound on the float distance from the row to its k-th
// nearest point, (|x - l| + r)^2 over the landmark's own cell when that holds >= k points, else
// +inf (rounded up, margins g for the float distances and 2^-120 for subnormal ones).
template <int DP>
__global__ void __launch_bounds__(128) tc_assign_kernel(const float* __restrict__ src, uint32_t stride, uint32_t dims,
                                                        uint32_t rows, const uint32_t* __restrict__ order,
                                                        const uint32_t* __restrict__ live_count,
                                                        const float* __restrict__ land, uint32_t ps, uint32_t cells,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                        const float* __restrict__ cell_far,
                                                        const uint32_t* __restrict__ cell_start, uint32_t k,
                                                        float* __restrict__ seed) {
    constexpr uint32_t kChunk = 64;
    __shared__ float sl[kChunk * DP];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = r < rows && r < (live_count ? *live_count : rows);
    const uint32_t row = live ? (order ? order[r] : r) : 0u;
    float q[DP];
#pragma unroll
    for (int d = 0; d < DP; ++d) q[d] = (live && static_cast<uint32_t>(d) < dims) ? src[static_cast<size_t>(row) * stride + d] : 0.0f;
    float best = INFINITY;
    uint32_t bi = 0;
    for (uint32_t c0 = 0; c0 < cells; c0 += kChunk) {
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < kChunk * DP; e += blockDim.x) {
            const uint32_t j = e / DP, d = e % DP;
            sl[e] = c0 + j < cells ? land[static_cast<size_t>(c0 + j) * ps + d] : 0.0f;
        }
        __syncthreads();
        const uint32_t jn = min(kChunk, cells - c0);
        // Two landmarks at a time, four partial sums each (the assignment may pick any landmark,
        // and the seed's error margin holds for any summation order).
        auto consider = [&](float acc, uint32_t j) {
            if (acc < best) {
                best = acc;
                bi = c0 + j;
            }
        };
        uint32_t j = 0;
        for (; j + 1 < jn; j += 2) {
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, b0 = 0.0f, b1 = 0.0f, b2 = 0.0f, b3 = 0.0f;
#pragma unroll
            for (int d = 0; d < DP; ++d) {
                const float t = __fsub_rn(q[d], sl[j * DP + d]), u = __fsub_rn(q[d], sl[(j + 1) * DP + d]);
                switch (d & 3) {
                    case 0: a0 = __fmaf_rn(t, t, a0); b0 = __fmaf_rn(u, u, b0); break;
                    case 1: a1 = __fmaf_rn(t, t, a1); b1 = __fmaf_rn(u, u, b1); break;
                    case 2: a2 = __fmaf_rn(t, t, a2); b2 = __fmaf_rn(u, u, b2); break;
                    default: a3 = __fmaf_rn(t, t, a3); b3 = __fmaf_rn(u, u, b3); break;
                }
            }
            consider((a0 + a1) + (a2 + a3), j);
            consider((b0 + b1) + (b2 + b3), j + 1);
        }
        if (j < jn) {
            float acc = 0.0f;
#pragma unroll
            for (int d = 0; d < DP; ++d) {
                const float t = __fsub_rn(q[d], sl[j * DP + d]);
                acc = __fmaf_rn(t, t, acc);
            }
            consider(acc, j);
        }
    }
    if (r < rows) {
        keys[r] = live ? bi : cells;
        vals[r] = row;
        if (seed && live) {
            float t = INFINITY;
            if (best <= FLT_MAX && cell_start[bi + 1] - cell_start[bi] >= k) {
                const float g = rel_margin(dims);
                const float inv = __frcp_ru(__fsub_rd(1.0f, g));  // >= 1 / (1 - g)
                const float a = __fsqrt_ru(__fmul_ru(best, inv));  // >= exact |x - l|
                const float b = __fsqrt_ru(__fmul_ru(cell_far[bi], inv));
                // Plus 2^-120 for float distances whose terms fall in the subnormal range.
                t = __fadd_ru(__fmul_ru(__fmul_ru(__fadd_ru(a, b), __fadd_ru(a, b)), __fadd_ru(1.0f, g)), 0x1p-120f);
            }
            seed[row] = t;
        }
    }
}

// Farthest row of each cell from its landmark, as (distance bits << 32) | row.
__global__ void tc_cell_far_kernel(const float* __restrict__ src, uint32_t stride, uint32_t dims,
                                   const uint32_t* __restrict__ cell, uint32_t rows, const float* __restrict__ land,
                                   uint32_t ps, unsigned long long* __restrict__ far) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint32_t c = cell[r];
    const float* x = src + static_cast<size_t>(r) * stride;
    const float* l = land + static_cast<size_t>(c) * ps;
    float acc = 0.0f;
    for (uint32_t d = 0; d < dims; ++d) {
        const float t = __fsub_rn(x[d], l[d]);
        acc = __fmaf_rn(t, t, acc);
    }
    atomicMax(far + c, (static_cast<unsigned long long>(__float_as_uint(acc)) << 32) | r);
}

// Padded position of each sorted point row: cell c's rows fill tiles cell_tile[c].. in order.
__global__ void tc_place_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n,
                                const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ cell_tile,
                                uint32_t* __restrict__ row_of) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = keys[i];
    row_of[static_cast<size_t>(cell_tile[c]) * kTileN + (i - cell_start[c])] = vals[i];
}

// Home range of each query tile: the cells of its (cell-sorted) queries, widened by whole
// neighbouring cells until they hold at least `min_points` points; written as first tile, end
// tile, first cell, last cell.
__global__ void tc_home_kernel(const uint32_t* __restrict__ cell_sorted, const uint32_t* __restrict__ live_count,
                               uint32_t nq, const uint32_t* __restrict__ cell_start,
                               const uint32_t* __restrict__ cell_tile, uint32_t cells, uint32_t min_points,
                               uint32_t qtiles, uint32_t* __restrict__ home) {
    const uint32_t qt = blockIdx.x * blockDim.x + threadIdx.x;
    if (qt >= qtiles) return;
    const uint32_t live = live_count ? *live_count : nq;
    const uint32_t first = qt * kTileM;
    if (first >= live) {
        home[4 * qt] = home[4 * qt + 1] = home[4 * qt + 2] = home[4 * qt + 3] = 0;
        return;
    }
    const uint32_t last = min(first + kTileM - 1, live - 1);
    uint32_t c0 = min(cell_sorted[first], cells - 1), c1 = min(cell_sorted[last], cells - 1);
    while (cell_start[c1 + 1] - cell_start[c0] < min_points && (c0 > 0 || c1 + 1 < cells)) {
        if (c0 > 0) --c0;
        if (c1 + 1 < cells && cell_start[c1 + 1] - cell_start[c0] < min_points) ++c1;
    }
    home[4 * qt] = cell_tile[c0];
    home[4 * qt + 1] = cell_tile[c1 + 1];
    home[4 * qt + 2] = c0;
    home[4 * qt + 3] = c1;
}

// One warp per cell, over its padded rows (valid: finite norm), in scaled coordinates (x * scale,
// exact): centre = the mean of its rows; radius = an upper bound on the exact distance from the
// centre to each of them (relative margin for normal-range rounding plus 2^-64 for subnormal
// rounding).
__global__ void tc_cell_ball_kernel(const float* __restrict__ pts, uint32_t ps, uint32_t dims, float scale,
                                    const float* __restrict__ norm, const uint32_t* __restrict__ cell_tile,
                                    uint32_t cells, float margin, float* __restrict__ centre,
                                    float* __restrict__ radius) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (c >= cells) return;
    const uint32_t r0 = cell_tile[c] * kTileN, r1 = cell_tile[c + 1] * kTileN;
    float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t cnt = 0;
    for (uint32_t r = r0; r < r1; ++r) {
        if (!(norm[r] <= FLT_MAX)) continue;
        ++cnt;
#pragma unroll
        for (uint32_t m = 0; m < 4; ++m) {
            const uint32_t d = lane + 32 * m;
            if (d < dims) sum[m] += pts[static_cast<size_t>(r) * ps + d] * scale;
        }
    }
    float cc[4];
#pragma unroll
    for (uint32_t m = 0; m < 4; ++m) {
        const uint32_t d = lane + 32 * m;
        cc[m] = (cnt && d < dims) ? sum[m] / static_cast<float>(cnt) : 0.0f;
        if (d < ps) centre[static_cast<size_t>(c) * ps + d] = cc[m];
    }
    float far = 0.0f;
    for (uint32_t r = r0; r < r1; ++r) {
        if (!(norm[r] <= FLT_MAX)) continue;
        float part = 0.0f;
#pragma unroll
        for (uint32_t m = 0; m < 4; ++m) {
            const uint32_t d = lane + 32 * m;
            if (d < dims) {
                const float e = __fsub_rn(cc[m], pts[static_cast<size_t>(r) * ps + d] * scale);
                part = __fmaf_rn(e, e, part);
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
        far = fmaxf(far, part);
    }
    if (lane == 0) radius[c] = cnt ? __fadd_ru(ball_radius(far, margin), 0x1p-64f) : 0.0f;
}

// Per tile of 256 rows: an upper bound on the norms of its rows (finite entries only).
__global__ void tc_tile_max_kernel(const float* __restrict__ norm, uint32_t tiles, float gn, float* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    float m = 0.0f;
    for (uint32_t r = 0; r < kTileN; ++r) {
        const float v = norm[static_cast<size_t>(t) * kTileN + r];
        if (v <= FLT_MAX) m = fmaxf(m, v);
    }
    out[t] = __fsqrt_ru(__fmul_ru(m, __fadd_ru(1.0f, gn)));
}

// Row data of the centre tiles: 256 norms then 256 radii per tile.
__global__ void tc_cdata_kernel(const float* __restrict__ cnorm, const float* __restrict__ radius, uint32_t cells,
                                uint32_t ctiles, float* __restrict__ cdata) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ctiles * kTileN) return;
    const uint32_t t = i / kTileN, j = i % kTileN;
    cdata[static_cast<size_t>(t) * kRowData + j] = i < cells ? cnorm[i] : INFINITY;
    cdata[static_cast<size_t>(t) * kRowData + kTileN + j] = i < cells ? radius[i] : 0.0f;
}

// ---- tree layout (dims <= kBoxMaxDims): a tile-aligned partition tree --------------------------
// Every node of m points covering t = ceil(m / 256) tiles sends its first ceil(t/2) * 256 points,
// in the order of their coordinate along the node's widest dimension, to its left child; nodes of
// one tile are leaves (cells).  The leaves are axis-aligned, compact tiles of 256 points (the last
// one possibly partial), and the shape depends on n alone.

__device__ __forceinline__ uint32_t order_key(float x) {
    const uint32_t u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float order_val(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Segment of each position: the last segment start <= i (starts ascending, starts[0] = 0).
__global__ void kp_segment_kernel(const uint32_t* __restrict__ starts, uint32_t nseg, uint32_t n,
                                  uint32_t* __restrict__ seg_of) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t lo = 0, hi = nseg;  // starts[lo] <= i < starts[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (starts[mid] <= i) lo = mid;
        else hi = mid;
    }
    seg_of[i] = lo;
}

// Per split segment and dimension, the range of its points' coordinates (orderable keys).
__global__ void kp_range_kernel(const float* __restrict__ src, uint32_t stride, uint32_t dims,
                                const uint32_t* __restrict__ order, const uint32_t* __restrict__ seg_of,
                                const uint8_t* __restrict__ split, uint32_t n, uint32_t* __restrict__ range) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t sg = seg_of[i];
    if (!split[sg]) return;
    const float* x = src + static_cast<size_t>(order[i]) * stride;
    for (uint32_t d = 0; d < dims; ++d) {
        const uint32_t key = order_key(x[d]);
        atomicMin(range + (static_cast<size_t>(sg) * dims + d) * 2, key);
        atomicMax(range + (static_cast<size_t>(sg) * dims + d) * 2 + 1, key);
    }
}

// Widest dimension of each split segment (lowest on ties).
__global__ void kp_dim_kernel(const uint32_t* __restrict__ range, const uint8_t* __restrict__ split, uint32_t nseg,
                              uint32_t dims, uint32_t* __restrict__ seg_dim) {
    const uint32_t sg = blockIdx.x * blockDim.x + threadIdx.x;
    if (sg >= nseg || !split[sg]) return;
    uint32_t best = 0;
    float width = -1.0f;
    for (uint32_t d = 0; d < dims; ++d) {
        const float w = order_val(range[(static_cast<size_t>(sg) * dims + d) * 2 + 1]) -
                        order_val(range[(static_cast<size_t>(sg) * dims + d) * 2]);
        if (w > width) {
            width = w;
            best = d;
        }
    }
    seg_dim[sg] = best;
}

__global__ void kp_key_kernel(const float* __restrict__ src, uint32_t stride, const uint32_t* __restrict__ order,
                              const uint32_t* __restrict__ seg_of, const uint8_t* __restrict__ split,
                              const uint32_t* __restrict__ seg_dim, uint32_t n, uint32_t* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t sg = seg_of[i];
    keys[i] = split[sg] ? order_key(src[static_cast<size_t>(order[i]) * stride + seg_dim[sg]]) : 0u;
    vals[i] = i;
}

__global__ void kp_segkey_kernel(const uint32_t* __restrict__ seg_of, const uint32_t* __restrict__ vals, uint32_t n,
                                 uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = seg_of[vals[i]];
}

__global__ void kp_gather_kernel(const uint32_t* __restrict__ order, const uint32_t* __restrict__ vals, uint32_t n,
                                 uint32_t* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = order[vals[i]];
}

// Split record of each split segment: its dimension and the coordinate of its last left point.
__global__ void kp_node_kernel(const float* __restrict__ src, uint32_t stride, const uint32_t* __restrict__ order,
                               const uint32_t* __restrict__ starts, const uint32_t* __restrict__ left,
                               const uint32_t* __restrict__ node, const uint8_t* __restrict__ split,
                               const uint32_t* __restrict__ seg_dim, uint32_t nseg, int32_t* __restrict__ node_dim,
                               float* __restrict__ node_val) {
    const uint32_t sg = blockIdx.x * blockDim.x + threadIdx.x;
    if (sg >= nseg || !split[sg]) return;
    node_dim[node[sg]] = static_cast<int32_t>(seg_dim[sg]);
    node_val[node[sg]] = src[static_cast<size_t>(order[starts[sg] + left[sg] - 1]) * stride + seg_dim[sg]];
}

// Axis-aligned box of each cell's rows in scaled coordinates (exact: the scale is a power of two),
// [cells][2][bd]: minima then maxima, zero past `dims`.
__global__ void tc_box_kernel(const float* __restrict__ pts, uint32_t ps, uint32_t dims, float scale,
                              const float* __restrict__ norm, const uint32_t* __restrict__ cell_tile, uint32_t cells,
                              uint32_t bd, float* __restrict__ box) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (c >= cells || lane >= bd) return;
    float lo = INFINITY, hi = -INFINITY;
    for (uint32_t r = cell_tile[c] * kTileN; r < cell_tile[c + 1] * kTileN; ++r) {
        if (!(norm[r] <= FLT_MAX) || lane >= dims) continue;
        const float x = pts[static_cast<size_t>(r) * ps + lane] * scale;
        lo = fminf(lo, x);
        hi = fmaxf(hi, x);
    }
    if (lane >= dims || lo > hi) lo = hi = 0.0f;
    box[static_cast<size_t>(c) * 2 * bd + lane] = lo;
    box[static_cast<size_t>(c) * 2 * bd + bd + lane] = hi;
}

// Leaf cell each query descends to; rows past the live count get key `cells`.  vals = the
// query index; seed[query] = an upper bound on its k-th float distance from its own cell's ball
// (centre c', radius R, scaled): ((|q' - c'| + R)^2 (1 + g) + slack) / s^2, when the cell holds
// >= k points, else +inf.
template <int DP>
__global__ void __launch_bounds__(128) kp_descend_kernel(const float* __restrict__ queries, uint32_t dims,
                                                         uint32_t rows, const uint32_t* __restrict__ order,
                                                         const uint32_t* __restrict__ live_count,
                                                         const int32_t* __restrict__ node_dim,
                                                         const float* __restrict__ node_val,
                                                         const int32_t* __restrict__ node_leaf, uint32_t cells,
                                                         const float* __restrict__ centre, uint32_t ps,
                                                         const float* __restrict__ radius,
                                                         const uint32_t* __restrict__ cell_start, uint32_t k,
                                                         float scale, uint32_t* __restrict__ keys,
                                                         uint32_t* __restrict__ vals, float* __restrict__ seed) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const bool live = r < (live_count ? *live_count : rows);
    const uint32_t qi = live ? (order ? order[r] : r) : 0u;
    uint32_t key = cells;
    if (live) {
        float q[DP];
#pragma unroll
        for (int d = 0; d < DP; ++d) q[d] = static_cast<uint32_t>(d) < dims ? queries[static_cast<size_t>(qi) * dims + d] : 0.0f;
        uint32_t nd = 0;
        for (int depth = 0; depth < 32 && node_leaf[nd] < 0; ++depth)
            nd = pick<DP>(q, static_cast<uint32_t>(node_dim[nd])) <= node_val[nd] ? 2 * nd + 1 : 2 * nd + 2;
        const uint32_t c = node_leaf[nd] >= 0 ? min(static_cast<uint32_t>(node_leaf[nd]), cells - 1) : 0u;
        key = c;
        float t = INFINITY;
        if (cell_start[c + 1] - cell_start[c] >= k) {
            float acc = 0.0f;
#pragma unroll
            for (int d = 0; d < DP; ++d) {
                const float e = __fsub_rn(q[d] * scale, centre[static_cast<size_t>(c) * ps + d]);
                acc = __fmaf_rn(e, e, acc);
            }
            const float g = rel_margin(dims);
            const float a = __fsqrt_ru(__fmul_ru(acc, __frcp_ru(__fsub_rd(1.0f, g))));  // >= exact |q' - c'|
            const float u = __fadd_ru(a, radius[c]);
            const float t_scaled = __fadd_ru(__fmul_ru(__fmul_ru(u, u), __fadd_ru(1.0f, g)), 0x1p-120f);
            t = __fmul_ru(t_scaled, 1.0f / (scale * scale));
        }
        seed[qi] = t;
    }
    keys[r] = key;
    vals[r] = qi;
}

// Squared float distances between all pairs of landmarks ([cells][cells]).
__global__ void tc_pair_d2_kernel(const float* __restrict__ land, uint32_t ps, uint32_t dims, uint32_t cells,
                                  float* __restrict__ out) {
    const uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (e >= static_cast<uint64_t>(cells) * cells) return;
    const float* a = land + (e / cells) * ps;
    const float* b = land + (e % cells) * ps;
    float acc = 0.0f;
    for (uint32_t d = 0; d < dims; ++d) {
        const float t = __fsub_rn(a[d], b[d]);
        acc = __fmaf_rn(t, t, acc);
    }
    out[e] = acc;
}

// out[j][0..ps) = src row rows[j], zero padded past `dims`.
__global__ void tc_gather_rows_kernel(const float* __restrict__ src, uint32_t stride, uint32_t dims,
                                      const uint32_t* __restrict__ rows, uint32_t count, uint32_t ps,
                                      float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count * ps) return;
    const uint32_t j = i / ps, d = i % ps;
    out[i] = d < dims ? src[static_cast<size_t>(rows[j]) * stride + d] : 0.0f;
}

// Largest |coordinate| over the rows (as float bits; NaN compares largest).
__global__ void tc_absmax_kernel(const float* __restrict__ src, uint32_t stride, uint32_t dims, uint32_t rows,
                                 uint32_t* __restrict__ out) {
    uint32_t m = 0;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < static_cast<size_t>(rows) * dims;
         e += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const size_t r = e / dims, d = e % dims;
        m = max(m, __float_as_uint(src[r * stride + d]) & 0x7FFFFFFFu);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if (threadIdx.x % 32 == 0) atomicMax(out, m);
}

// Dense copy of a tree's occupied leaf slots (slot order): coordinates (zero padded to ps) and ids.
__global__ void tc_gather_slots_kernel(const float* __restrict__ leaf, uint32_t leaf_stride, uint32_t id_at,
                                       const uint32_t* __restrict__ slots, uint32_t n, uint32_t dims, uint32_t ps,
                                       float* __restrict__ dense, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* s = leaf + static_cast<size_t>(slots[i]) * leaf_stride;
    for (uint32_t d = 0; d < ps; ++d) dense[static_cast<size_t>(i) * ps + d] = d < dims ? s[d] : 0.0f;
    ids[i] = static_cast<uint32_t>(__float_as_int(s[id_at]));
}

__global__ void tc_slot_keys_kernel(const float* __restrict__ leaf, uint32_t leaf_stride, uint32_t id_at, uint32_t slots,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots) return;
    keys[i] = __float_as_int(leaf[static_cast<size_t>(i) * leaf_stride + id_at]) >= 0 ? 0u : 1u;
    vals[i] = i;
}

// Self-test: one 128 x 256 tile over the layout's whole K extent through the same descriptors,
// written to global.
template <uint32_t H>
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const uint8_t* __restrict__ qimg,
                                                             const uint8_t* __restrict__ pimg, uint32_t idesc,
                                                             float* __restrict__ out, int* __restrict__ error) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* sA = smem;
    uint8_t* sB = sA + a_bytes(H);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + b_bytes(H));
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
            for (uint32_t ks = 0; ks < ly_elems(H) / 16; ++ks)
                mma_f16kind(tmem, ly_desc(H, smem_addr(sA), kTileM, ks), ly_desc(H, smem_addr(sB), kTileN, ks), idesc,
                            ks != 0);
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

// Shared memory of the filter apart from its bound codes.
size_t filter_fixed_smem(uint32_t H) {
    return 1024 + a_bytes(H) + 2 * b_bytes(H) + 2 * kRowData * sizeof(float) + kMaskWords * sizeof(uint32_t) + 16 +
           kStage * kTileM * 4 + 16 * 8 + 8;
}

// The heap mode's k floats per query row, where two blocks per SM still fit them.
bool filter_heap_fits(uint32_t H, uint32_t k) {
    return 2 * (filter_fixed_smem(H) + static_cast<size_t>((2 * k + 15) & ~15u) * kTileM * 2 + 1024) <= 228 * 1024;
}

// Bound codes buffered per query row: 4 (k + 32), when two blocks per SM then still fit; else
// as many as one block's shared memory leaves, up to that (a flush makes room for the next chunk's
// 32 columns above the k codes it keeps, so fewer than k + 48 leave too little room).  In heap
// mode, the codes' bytes hold the heap and the pending list instead.
uint32_t filter_codes(uint32_t H, uint32_t k, bool heap = false) {
    if (heap) return (2 * k + 15) & ~15u;
    const uint32_t want = (4 * (k + 32) + 15) & ~15u;
    const size_t fixed = filter_fixed_smem(H);
    if (2 * (fixed + static_cast<size_t>(want) * kTileM * 2 + 1024) <= 228 * 1024) return want;
    const size_t room = fixed < 232448 ? 232448 - fixed : 0;
    return std::min<uint32_t>(want, static_cast<uint32_t>(room / (kTileM * 2)) & ~15u);
}

size_t filter_smem(uint32_t H, uint32_t k, bool heap = false) {
    return filter_fixed_smem(H) + static_cast<size_t>(filter_codes(H, k, heap)) * kTileM * 2;
}

// The filter allocates all 512 TMEM columns, so a second resident block on the same SM would
// wait inside tcgen05.alloc; asking for more than half the SM's shared memory keeps one block
// per SM.
// One accumulator (two blocks per SM) when two blocks' shared memory fits an SM.
uint32_t accumulators(uint32_t H, uint32_t k, bool heap) {
    return 2 * (filter_smem(H, k, heap) + 1024) <= 228 * 1024 ? 1u : 2u;
}

// A block allocates ACC x 256 TMEM columns of the SM's 512, so more resident blocks than
// 512 / (ACC x 256) would wait inside tcgen05.alloc: the shared memory asked for caps them at one
// block per SM (two accumulators) or two (one accumulator).
size_t filter_launch_smem(uint32_t H, uint32_t k, bool heap) {
    return std::max<size_t>(filter_smem(H, k, heap), accumulators(H, k, heap) == 2 ? 120 * 1024 : 80 * 1024);
}

// Layout code of the operand images for `dims` dimensions (see ly_row_bytes).
uint32_t halves(uint32_t dims) { return dims <= 16 ? 32u : dims <= 32 ? 64u : dims <= 64 ? 1u : 2u; }

Bounds make_bounds(uint32_t dims, bool f16, float scale) {
    const double u = f16 ? std::ldexp(1.0, -11) : std::ldexp(1.0, -8);
    const double delta = f16 ? std::ldexp(1.0, -14) : std::ldexp(1.0, -100);
    const double D = dims;
    Bounds b{};
    b.c1 = static_cast<float>((2 * u + u * u + D * std::ldexp(1.0, -20) * (1 + u) * (1 + u)) * (1 + std::ldexp(1.0, -10)));
    b.c3 = static_cast<float>(1.01 * delta * (1 + u) * std::sqrt(D));
    // Plus the float distance's absolute error when its terms fall in the subnormal range,
    // (D + 4) 2^-149 unscaled, twice over, in scaled units.
    const double s2 = static_cast<double>(scale) * scale;
    b.c4 = static_cast<float>(1.01 * D * delta * delta + 2.0 * s2 * (D + 4) * std::ldexp(1.0, -149));
    b.gn = rel_margin(dims);
    b.g = rel_margin(dims);
    float inv = static_cast<float>(1.0 / (1.0 - static_cast<double>(b.g)));
    if (static_cast<double>(inv) < 1.0 / (1.0 - static_cast<double>(b.g))) inv = std::nextafter(inv, INFINITY);
    b.inv_one_m = inv;
    return b;
}

// Cell of each query at query time (landmark layout): the nearest landmark by the 16-bit GEMM,
// one CTA per 128 rows.  Thread 0 streams the rows' operand tile and every landmark tile (with its
// 256 scaled norms) through a two-stage ring and issues the MMAs; all four warps read the
// accumulator (thread = row) and keep the column of least n_l - 2G.  Any cell is a correct choice
// (every later bound holds for any assignment); the nearest landmark's cell is the one whose
// points lie around the query.  The seed is then (|x - l| + far_l)^2 over that cell when it holds
// >= k points, from the row's float distance to the landmark (rounded up, margins g for the float
// distances and 2^-120 for subnormal ones).
// Rows past the live count get key `cells`.  Every wait is bounded; a timeout sets *error and the
// rows keep the best cell seen so far, with no seed.
template <uint32_t H>
__global__ void __launch_bounds__(128, 1) tc_assign_mma_kernel(
    const uint8_t* __restrict__ qimg, const uint8_t* __restrict__ limg, const float* __restrict__ lnorm,
    uint32_t ctiles, uint32_t cells, uint32_t idesc, uint32_t rows, const uint32_t* __restrict__ order,
    const uint32_t* __restrict__ live_count, const float* __restrict__ queries, uint32_t dims,
    const float* __restrict__ land, uint32_t ps, const float* __restrict__ cell_far,
    const uint32_t* __restrict__ cell_start, uint32_t k, uint32_t* __restrict__ keys,
    uint32_t* __restrict__ vals, float* __restrict__ seed, int* __restrict__ error) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* sA = smem;
    uint8_t* sB = sA + a_bytes(H);                                              // [2] landmark tiles
    float* sN = reinterpret_cast<float*>(sB + 2 * b_bytes(H));                 // [2][kTileN] norms
    uint64_t* bar = reinterpret_cast<uint64_t*>(sN + 2 * kTileN);               // [0..1] loads, [2] MMA
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 3);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t tile = blockIdx.x;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        mbar_init(bar + 2, 1);
        *abort = 0;
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, kTileN);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    uint32_t loads_issued = 0, loads_done = 0, commits = 0;  // thread 0's counts
    auto load_centres = [&](uint32_t t) {  // thread 0
        const uint32_t st = t & 1;
        ++loads_issued;
        mbar_expect_tx(bar + st, b_bytes(H) + kTileN * 4 + (t == 0 ? a_bytes(H) : 0u));
        if (t == 0) bulk_copy_g2s(sA, qimg + static_cast<size_t>(tile) * a_bytes(H), a_bytes(H), bar);
        bulk_copy_g2s(sB + st * b_bytes(H), limg + static_cast<size_t>(t) * b_bytes(H), b_bytes(H), bar + st);
        bulk_copy_g2s(sN + st * kTileN, lnorm + static_cast<size_t>(t) * kTileN, kTileN * 4, bar + st);
    };
    if (threadIdx.x == 0) {
        load_centres(0);
        if (ctiles > 1) load_centres(1);
    }
    float best = INFINITY;
    uint32_t bi = 0;
    for (uint32_t t = 0; t < ctiles; ++t) {
        const uint32_t st = t & 1;
        if (threadIdx.x == 0) {
            if (!*abort && mbar_wait(bar + st, (t >> 1) & 1u, abort)) {
                ++loads_done;
                tc_fence_after();
                for (uint32_t ks = 0; ks < ly_elems(H) / 16; ++ks)
                    mma_f16kind(tmem, ly_desc(H, smem_addr(sA), kTileM, ks),
                                ly_desc(H, smem_addr(sB + st * b_bytes(H)), kTileN, ks), idesc, ks != 0);
                mma_commit(bar + 2);
                ++commits;
            } else {
                *abort = 1;
            }
        }
        __syncthreads();
        const bool failed = *abort || !mbar_wait(bar + 2, t & 1u, abort);
        if (__syncthreads_or(failed)) {  // every thread leaves the loop at the same tile
            if (threadIdx.x == 0) *abort = 1;
            break;
        }
        tc_fence_after();
        const float* nrm = sN + st * kTileN;
        for (uint32_t c = 0; c < kTileN / 32; ++c) {
            float v[32];
            tmem_ld32(tmem + ((warp * 32u) << 16) + c * 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; ++i) {
                const float d = __fmaf_rn(-2.0f, v[i], nrm[c * 32 + i]);
                if (d < best) {
                    best = d;
                    bi = t * kTileN + c * 32 + i;
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // the accumulator and stage st are free
        if (threadIdx.x == 0 && t + 2 < ctiles) load_centres(t + 2);
    }
    __syncthreads();
    const bool aborted = *abort != 0;
    if (aborted && threadIdx.x == 0) {
        atomicExch(error, 1);
        // Let the copies and MMAs still in flight land before the block's memory is released.
        volatile int never = 0;
        for (uint32_t i = loads_done; i < loads_issued; ++i) mbar_wait(bar + (i & 1), (i >> 1) & 1u, &never);
        if (commits) mbar_wait(bar + 2, (commits - 1) & 1u, &never);
    }
    // Every row gets a valid cell, also after a timeout (any cell is correct).
    const uint32_t r = tile * kTileM + warp * 32 + lane;
    if (r < rows) {
        const bool live = r < (live_count ? *live_count : rows);
        const uint32_t qi = live ? (order ? order[r] : r) : 0u;
        const uint32_t c = min(bi, cells - 1);
        keys[r] = live ? c : cells;
        vals[r] = qi;
        if (live && seed) {
            float t = INFINITY;
            if (!aborted && cell_start[c + 1] - cell_start[c] >= k) {
                float acc = 0.0f;
                for (uint32_t d = 0; d < dims; ++d) {
                    const float e = __fsub_rn(queries[static_cast<size_t>(qi) * dims + d], land[static_cast<size_t>(c) * ps + d]);
                    acc = __fmaf_rn(e, e, acc);
                }
                if (acc <= FLT_MAX) {
                    const float g = rel_margin(dims);
                    const float inv = __frcp_ru(__fsub_rd(1.0f, g));  // >= 1 / (1 - g)
                    const float a = __fsqrt_ru(__fmul_ru(acc, inv));   // >= exact |x - l|
                    const float b = __fsqrt_ru(__fmul_ru(cell_far[c], inv));
                    t = __fadd_ru(__fmul_ru(__fmul_ru(__fadd_ru(a, b), __fadd_ru(a, b)), __fadd_ru(1.0f, g)), 0x1p-120f);
                }
            }
            seed[qi] = t;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTileN);
    }
}

size_t assign_mma_smem(uint32_t H) { return 1024 + a_bytes(H) + 2 * b_bytes(H) + 2 * kTileN * 4 + 64; }

int launch_assign(uint32_t dp, const float* src, uint32_t stride, uint32_t dims, uint32_t rows, const uint32_t* order,
                  const uint32_t* live_count, const float* land, uint32_t ps, uint32_t cells, uint32_t* keys,
                  uint32_t* vals, cudaStream_t s, const float* cell_far = nullptr, const uint32_t* cell_start = nullptr,
                  uint32_t k = 0, float* seed = nullptr) {
    const uint32_t grid = ceil_div(rows, 128);
#define KNN_ASSIGN(D_)                                                                                         \
    case D_:                                                                                                   \
        tc_assign_kernel<D_><<<grid, 128, 0, s>>>(src, stride, dims, rows, order, live_count, land, ps, cells, \
                                                   keys, vals, cell_far, cell_start, k, seed);                 \
        break;
    switch (dp) {
        KNN_ASSIGN(1) KNN_ASSIGN(2) KNN_ASSIGN(3) KNN_ASSIGN(4) KNN_ASSIGN(8) KNN_ASSIGN(16) KNN_ASSIGN(32)
        KNN_ASSIGN(64) KNN_ASSIGN(128)
        default: return fail(KNN_ERR_UNSUPPORTED, "dims");
    }
#undef KNN_ASSIGN
    KNN_LAUNCHED();
    return KNN_OK;
}

int launch_descend(uint32_t dp, const float* queries, uint32_t dims, uint32_t rows, const uint32_t* order,
                   const uint32_t* live_count, const knn_index::TensorCoreState& T, uint32_t k, uint32_t* keys,
                   uint32_t* vals, float* seed, cudaStream_t s) {
    const uint32_t grid = ceil_div(rows, 128);
#define KNN_DESCEND(D_)                                                                                               \
    case D_:                                                                                                          \
        kp_descend_kernel<D_><<<grid, 128, 0, s>>>(queries, dims, rows, order, live_count, T.node_dim.as<int32_t>(),  \
                                                    T.node_val.as<float>(), T.node_leaf.as<int32_t>(), T.cells,        \
                                                    T.ccentre.as<float>(), T.ps, T.cradius.as<float>(),                \
                                                    T.cell_start.as<uint32_t>(), k, T.scale, keys, vals, seed);        \
        break;
    switch (dp) {
        KNN_DESCEND(1) KNN_DESCEND(2) KNN_DESCEND(3) KNN_DESCEND(4) KNN_DESCEND(8) KNN_DESCEND(16) KNN_DESCEND(32)
        default: return fail(KNN_ERR_UNSUPPORTED, "tree layout beyond %u dims", kBoxMaxDims);
    }
#undef KNN_DESCEND
    KNN_LAUNCHED();
    return KNN_OK;
}

}  // namespace

bool tc_supported(uint32_t dims, uint32_t k) {
    return dims >= 1 && dims <= kMaxDims && k >= 1 && k <= kMaxK && filter_codes(halves(dims), k) >= k + 48 &&
           filter_smem(halves(dims), k) <= 232448;
}

// Builds the cells, operand images, norms, FP32 copy, ids and cell balls of an index (once).
int tc_prepare(knn_index* ix, cudaStream_t s) {
    auto& T = ix->tc;
    if (T.ready) return T.usable ? KNN_OK : fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: coordinates out of range");
    const Range range("tensor-core filter layout");
    const uint32_t n = ix->n, dims = ix->dims, ps = round_up4(ix->dp), H = halves(dims);
    // Dense source rows: the brute-force points, or a tree's occupied leaf slots in slot order.
    DevBuf dense_buf;
    const float* src = nullptr;
    uint32_t stride = 0;
    const uint32_t* src_ids = nullptr;
    if (ix->structure == KNN_BRUTE_FORCE) {
        src = ix->points.as<float>();
        stride = ix->point_stride;
    } else {
        const uint32_t slots = (1u << ix->node_depth) * ix->leaf_slots;
        DevBuf tmp;
        KNN_TRY(tmp.alloc(carve_bytes({slots * 4ull, slots * 4ull, slots * 4ull, slots * 4ull, radix_sort_temp_bytes(slots)})));
        Carver c(tmp.ptr);
        uint32_t* k0 = c.take<uint32_t>(slots);
        uint32_t* v0 = c.take<uint32_t>(slots);
        uint32_t* k1 = c.take<uint32_t>(slots);
        uint32_t* v1 = c.take<uint32_t>(slots);
        void* st = c.take<uint8_t>(radix_sort_temp_bytes(slots));
        tc_slot_keys_kernel<<<ceil_div(slots, 256), 256, 0, s>>>(ix->leaf.as<float>(), ix->leaf_stride, ix->leaf_id_at,
                                                                 slots, k0, v0);
        KNN_LAUNCHED();
        bool alt = false;
        KNN_TRY(radix_sort_pairs(k0, v0, k1, v1, slots, 1, st, s, &alt));
        KNN_TRY(dense_buf.alloc(carve_bytes({static_cast<size_t>(n) * ps * 4, n * 4ull})));
        Carver dc(dense_buf.ptr);
        float* dense = dc.take<float>(static_cast<size_t>(n) * ps);
        uint32_t* ids = dc.take<uint32_t>(n);
        tc_gather_slots_kernel<<<ceil_div(n, 128), 128, 0, s>>>(ix->leaf.as<float>(), ix->leaf_stride, ix->leaf_id_at,
                                                                alt ? v1 : v0, n, dims, ps, dense, ids);
        KNN_LAUNCHED();
        KNN_TRY_CUDA(cudaStreamSynchronize(s));
        src = dense;
        stride = ps;
        src_ids = ids;
    }

    // Scale: largest |coordinate| * 2^e in [2^13, 2^14) with e >= 0, else BF16.
    DevBuf small;
    KNN_TRY(small.alloc(256));
    KNN_TRY_CUDA(cudaMemsetAsync(small.ptr, 0, 256, s));
    const uint32_t am_grid = static_cast<uint32_t>(
        std::max<uint64_t>(1, std::min<uint64_t>((static_cast<uint64_t>(n) * dims + 255) / 256, 4ull * sm_count())));
    tc_absmax_kernel<<<am_grid, 256, 0, s>>>(src, stride, dims, n, small.as<uint32_t>());
    KNN_LAUNCHED();
    uint32_t mbits = 0;
    KNN_TRY_CUDA(cudaMemcpyAsync(&mbits, small.ptr, 4, cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    float M;
    std::memcpy(&M, &mbits, 4);
    T.ready = true;
    T.usable = false;
    if (!(M <= FLT_MAX)) return fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: non-finite coordinates");
    T.f16 = M <= 16384.0f;
    int e = 0;
    if (T.f16 && M > 0.0f)
        while (e < 60 && std::ldexp(static_cast<double>(M), e + 1) < 16384.0) ++e;
    T.scale = T.f16 ? std::ldexp(1.0f, e) : 1.0f;
    T.ps = ps;

    // Cells: the leaves of a partition tree at low dims (axis-aligned, tight boxes), landmark cells
    // otherwise (boxes say little in many dims; the centre test does the work).
    T.tree = dims <= kBoxMaxDims;
    uint32_t cells = 0;
    std::vector<uint32_t> cell_start, cell_tile;
    DevBuf rowmap;
    if (T.tree) {
        {
            struct Node {
                uint32_t start = 0, size = 0, depth = 0;
                int32_t leaf = -1;
                bool used = false;
            };
            std::vector<Node> shape(1);
            shape[0] = Node{0, n, 0, -1, true};
            uint32_t max_depth = 0;
            // Leaves of up to `lt` tiles, so that there are at most kMaxCells of them.
            const uint32_t lt = std::max(1u, ceil_div(ceil_div(n, kTileN), kMaxCells));
            for (std::vector<uint32_t> work{0}; !work.empty();) {
                const uint32_t id = work.back();
                work.pop_back();
                const Node nd = shape[id];
                const uint32_t t = ceil_div(nd.size, kTileN);
                if (t <= lt) {
                    shape[id].leaf = 0;  // numbered in position order below
                    continue;
                }
                max_depth = std::max(max_depth, nd.depth);
                const uint32_t left = (t + 1) / 2 * kTileN;
                if (shape.size() < 2 * static_cast<size_t>(id) + 3) shape.resize(2 * static_cast<size_t>(id) + 3);
                shape[2 * id + 1] = Node{nd.start, left, nd.depth + 1, -1, true};
                shape[2 * id + 2] = Node{nd.start + left, nd.size - left, nd.depth + 1, -1, true};
                work.push_back(2 * id + 1);
                work.push_back(2 * id + 2);
            }
            const uint32_t nodes = static_cast<uint32_t>(shape.size());
            std::vector<uint32_t> leaves;
            for (uint32_t i = 0; i < nodes; ++i)
                if (shape[i].used && shape[i].leaf >= 0) leaves.push_back(i);
            std::sort(leaves.begin(), leaves.end(), [&](uint32_t x, uint32_t y) { return shape[x].start < shape[y].start; });
            for (uint32_t c = 0; c < leaves.size(); ++c) shape[leaves[c]].leaf = static_cast<int32_t>(c);
            KNN_TRY(T.node_dim.alloc(nodes * 4ull));
            KNN_TRY(T.node_val.alloc(nodes * 4ull));
            KNN_TRY(T.node_leaf.alloc(nodes * 4ull));
            KNN_TRY_CUDA(cudaMemsetAsync(T.node_dim.ptr, 0, nodes * 4ull, s));
            KNN_TRY_CUDA(cudaMemsetAsync(T.node_val.ptr, 0, nodes * 4ull, s));
            std::vector<int32_t> leaf(nodes, 0);
            for (uint32_t i = 0; i < nodes; ++i) leaf[i] = shape[i].used ? shape[i].leaf : 0;
            KNN_TRY_CUDA(cudaMemcpyAsync(T.node_leaf.ptr, leaf.data(), nodes * 4ull, cudaMemcpyHostToDevice, s));
            DevBuf tb;
            KNN_TRY(tb.alloc(carve_bytes({n * 4ull, n * 4ull, n * 4ull, n * 4ull, n * 4ull, n * 4ull, n * 4ull,
                                          radix_sort_temp_bytes(n), nodes * 4ull, nodes * 4ull, nodes * 4ull, nodes * 1ull,
                                          nodes * 4ull, static_cast<size_t>(nodes) * dims * 8})));
            Carver tc_(tb.ptr);
            uint32_t* order = tc_.take<uint32_t>(n);
            uint32_t* order_alt = tc_.take<uint32_t>(n);
            uint32_t* seg_of = tc_.take<uint32_t>(n);
            uint32_t* q0 = tc_.take<uint32_t>(n);
            uint32_t* w0 = tc_.take<uint32_t>(n);
            uint32_t* q1 = tc_.take<uint32_t>(n);
            uint32_t* w1 = tc_.take<uint32_t>(n);
            void* tst = tc_.take<uint8_t>(radix_sort_temp_bytes(n));
            uint32_t* d_starts = tc_.take<uint32_t>(nodes);
            uint32_t* d_left = tc_.take<uint32_t>(nodes);
            uint32_t* d_node = tc_.take<uint32_t>(nodes);
            uint8_t* d_split = tc_.take<uint8_t>(nodes);
            uint32_t* seg_dim = tc_.take<uint32_t>(nodes);
            uint32_t* range = tc_.take<uint32_t>(static_cast<size_t>(nodes) * dims * 2);
            {
                std::vector<uint32_t> iota(n);
                std::iota(iota.begin(), iota.end(), 0u);
                KNN_TRY_CUDA(cudaMemcpyAsync(order, iota.data(), n * 4ull, cudaMemcpyHostToDevice, s));
                KNN_TRY_CUDA(cudaStreamSynchronize(s));
            }
            for (uint32_t depth = 0; leaves.size() > 1 && depth <= max_depth; ++depth) {
                // Frontier in position order: the nodes of this depth and the shallower leaves.
                std::vector<uint32_t> ids;
                for (uint32_t i = 0; i < nodes; ++i)
                    if (shape[i].used && (shape[i].depth == depth || (shape[i].leaf >= 0 && shape[i].depth < depth)))
                        ids.push_back(i);
                std::sort(ids.begin(), ids.end(), [&](uint32_t x, uint32_t y) { return shape[x].start < shape[y].start; });
                const uint32_t nseg = static_cast<uint32_t>(ids.size());
                std::vector<uint32_t> starts(nseg), left(nseg);
                std::vector<uint8_t> split(nseg);
                for (uint32_t j = 0; j < nseg; ++j) {
                    const Node& nd = shape[ids[j]];
                    starts[j] = nd.start;
                    split[j] = nd.leaf < 0 && nd.depth == depth;
                    left[j] = split[j] ? (ceil_div(nd.size, kTileN) + 1) / 2 * kTileN : 0u;
                }
                KNN_TRY_CUDA(cudaMemcpyAsync(d_starts, starts.data(), nseg * 4ull, cudaMemcpyHostToDevice, s));
                KNN_TRY_CUDA(cudaMemcpyAsync(d_left, left.data(), nseg * 4ull, cudaMemcpyHostToDevice, s));
                KNN_TRY_CUDA(cudaMemcpyAsync(d_node, ids.data(), nseg * 4ull, cudaMemcpyHostToDevice, s));
                KNN_TRY_CUDA(cudaMemcpyAsync(d_split, split.data(), nseg, cudaMemcpyHostToDevice, s));
                kp_segment_kernel<<<ceil_div(n, 256), 256, 0, s>>>(d_starts, nseg, n, seg_of);
                KNN_LAUNCHED();
                // Range per segment and dimension: minima start at all ones, maxima at zero.
                std::vector<uint32_t> init(static_cast<size_t>(nseg) * dims * 2);
                for (size_t e = 0; e < init.size(); ++e) init[e] = (e % 2 == 0) ? 0xFFFFFFFFu : 0u;
                KNN_TRY_CUDA(cudaMemcpyAsync(range, init.data(), init.size() * 4, cudaMemcpyHostToDevice, s));
                kp_range_kernel<<<ceil_div(n, 128), 128, 0, s>>>(src, stride, dims, order, seg_of, d_split, n, range);
                KNN_LAUNCHED();
                kp_dim_kernel<<<ceil_div(nseg, 128), 128, 0, s>>>(range, d_split, nseg, dims, seg_dim);
                KNN_LAUNCHED();
                // Positions by (segment, coordinate along its widest dimension): coordinate first,
                // then segment (stable).
                kp_key_kernel<<<ceil_div(n, 256), 256, 0, s>>>(src, stride, order, seg_of, d_split, seg_dim, n, q0, w0);
                KNN_LAUNCHED();
                bool alt = false;
                KNN_TRY(radix_sort_pairs(q0, w0, q1, w1, n, 32, tst, s, &alt));
                uint32_t* ka = alt ? q1 : q0;
                uint32_t* va = alt ? w1 : w0;
                uint32_t* kb = alt ? q0 : q1;
                uint32_t* vb = alt ? w0 : w1;
                kp_segkey_kernel<<<ceil_div(n, 256), 256, 0, s>>>(seg_of, va, n, ka);
                KNN_LAUNCHED();
                bool alt2 = false;
                KNN_TRY(radix_sort_pairs(ka, va, kb, vb, n, static_cast<int>(log2_ceil(nseg + 1)), tst, s, &alt2));
                kp_gather_kernel<<<ceil_div(n, 256), 256, 0, s>>>(order, alt2 ? vb : va, n, order_alt);
                KNN_LAUNCHED();
                std::swap(order, order_alt);
                kp_node_kernel<<<ceil_div(nseg, 128), 128, 0, s>>>(src, stride, order, d_starts, d_left, d_node, d_split,
                                                                   seg_dim, nseg, T.node_dim.as<int32_t>(),
                                                                   T.node_val.as<float>());
                KNN_LAUNCHED();
                KNN_TRY_CUDA(cudaStreamSynchronize(s));  // the host vectors above are reused next level
            }
            cells = static_cast<uint32_t>(leaves.size());
            cell_start.resize(cells + 1);
            cell_tile.resize(cells + 1);
            for (uint32_t c = 0; c < cells; ++c) {
                cell_start[c] = shape[leaves[c]].start;
                cell_tile[c] = shape[leaves[c]].start / kTileN;
            }
            cell_start[cells] = n;
            cell_tile[cells] = ceil_div(n, kTileN);
            KNN_TRY(T.cell_start.alloc((cells + 1) * 4ull));
            KNN_TRY(T.cell_tile.alloc((cells + 1) * 4ull));
            KNN_TRY_CUDA(cudaMemcpyAsync(T.cell_start.ptr, cell_start.data(), (cells + 1) * 4ull, cudaMemcpyHostToDevice, s));
            KNN_TRY_CUDA(cudaMemcpyAsync(T.cell_tile.ptr, cell_tile.data(), (cells + 1) * 4ull, cudaMemcpyHostToDevice, s));
            const uint32_t prows = cell_tile[cells] * kTileN;
            KNN_TRY(rowmap.alloc(prows * 4ull));
            KNN_TRY_CUDA(cudaMemsetAsync(rowmap.ptr, 0xFF, prows * 4ull, s));
            KNN_TRY_CUDA(cudaMemcpyAsync(rowmap.ptr, order, n * 4ull, cudaMemcpyDeviceToDevice, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));
        }

    } else {
        // Landmarks: every (n/L)-th point; then, up to three times, a landmark at the farthest point
        // of each cell whose farthest squared distance exceeds 4x the 25th percentile over cells (a
        // cell holding two clusters is split); finally the landmarks in the order of a greedy
        // nearest-neighbour chain, so that consecutive cells lie near each other.
        std::vector<uint32_t> lrows;
        {
            const uint32_t L0 = std::max(1u, std::min(kMaxCells / 2, n / kCellPoints));
            for (uint32_t j = 0; j < L0; ++j) lrows.push_back(static_cast<uint32_t>(static_cast<uint64_t>(j) * n / L0));
        }
        DevBuf sortb;
        KNN_TRY(sortb.alloc(carve_bytes({n * 4ull, n * 4ull, n * 4ull, n * 4ull, radix_sort_temp_bytes(n), kMaxCells * 8ull,
                                         kMaxCells * 4ull})));
        Carver sc(sortb.ptr);
        uint32_t* k0 = sc.take<uint32_t>(n);
        uint32_t* v0 = sc.take<uint32_t>(n);
        uint32_t* k1 = sc.take<uint32_t>(n);
        uint32_t* v1 = sc.take<uint32_t>(n);
        void* st = sc.take<uint8_t>(radix_sort_temp_bytes(n));
        unsigned long long* far = sc.take<unsigned long long>(kMaxCells);
        uint32_t* lr = sc.take<uint32_t>(kMaxCells);
        KNN_TRY(T.land.alloc(static_cast<size_t>(kMaxCells) * ps * 4));
        auto place_landmarks = [&]() -> int {
            const uint32_t cells = static_cast<uint32_t>(lrows.size());
            KNN_TRY_CUDA(cudaMemcpyAsync(lr, lrows.data(), cells * 4ull, cudaMemcpyHostToDevice, s));
            tc_gather_rows_kernel<<<ceil_div(cells * ps, 256), 256, 0, s>>>(src, stride, dims, lr, cells, ps,
                                                                           T.land.as<float>());
            KNN_LAUNCHED();
            KNN_TRY(launch_assign(ix->dp, src, stride, dims, n, nullptr, nullptr, T.land.as<float>(), ps, cells, k0, v0, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));  // lrows is reused
            return KNN_OK;
        };
        for (int round = 0;; ++round) {
            const uint32_t cells = static_cast<uint32_t>(lrows.size());
            KNN_TRY(place_landmarks());
            if (round == 3 || cells >= kMaxCells) break;
            KNN_TRY_CUDA(cudaMemsetAsync(far, 0, cells * 8ull, s));
            tc_cell_far_kernel<<<ceil_div(n, 256), 256, 0, s>>>(src, stride, dims, k0, n, T.land.as<float>(), ps, far);
            KNN_LAUNCHED();
            std::vector<unsigned long long> hfar(cells);
            KNN_TRY_CUDA(cudaMemcpyAsync(hfar.data(), far, cells * 8ull, cudaMemcpyDeviceToHost, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));
            std::vector<float> d2;
            for (auto f : hfar) {
                float v;
                const uint32_t bits = static_cast<uint32_t>(f >> 32);
                std::memcpy(&v, &bits, 4);
                if (f) d2.push_back(v);
            }
            if (d2.empty()) break;
            std::vector<float> sorted = d2;
            std::nth_element(sorted.begin(), sorted.begin() + sorted.size() / 4, sorted.end());
            const float q25 = sorted[sorted.size() / 4];
            uint32_t added = 0;
            for (uint32_t c = 0; c < cells && lrows.size() < kMaxCells; ++c) {
                if (!hfar[c]) continue;
                float v;
                const uint32_t bits = static_cast<uint32_t>(hfar[c] >> 32);
                std::memcpy(&v, &bits, 4);
                if (v > 4.0f * q25 && v > 0.0f) {
                    lrows.push_back(static_cast<uint32_t>(hfar[c] & 0xFFFFFFFFu));
                    ++added;
                }
            }
            if (!added) break;
        }
        cells = static_cast<uint32_t>(lrows.size());
        if (cells > 2) {
            DevBuf pd;
            KNN_TRY(pd.alloc(static_cast<size_t>(cells) * cells * 4));
            tc_pair_d2_kernel<<<static_cast<uint32_t>((static_cast<uint64_t>(cells) * cells + 255) / 256), 256, 0, s>>>(
                T.land.as<float>(), ps, dims, cells, pd.as<float>());
            KNN_LAUNCHED();
            std::vector<float> hd(static_cast<size_t>(cells) * cells);
            KNN_TRY_CUDA(cudaMemcpyAsync(hd.data(), pd.ptr, hd.size() * 4, cudaMemcpyDeviceToHost, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));
            std::vector<uint8_t> seen(cells, 0);
            std::vector<uint32_t> chain{0};
            seen[0] = 1;
            for (uint32_t step = 1; step < cells; ++step) {
                const float* row = hd.data() + static_cast<size_t>(chain.back()) * cells;
                uint32_t best = kNone;
                for (uint32_t j = 0; j < cells; ++j)
                    if (!seen[j] && (best == kNone || row[j] < row[best])) best = j;
                seen[best] = 1;
                chain.push_back(best);
            }
            std::vector<uint32_t> reordered(cells);
            for (uint32_t i = 0; i < cells; ++i) reordered[i] = lrows[chain[i]];
            lrows.swap(reordered);
            KNN_TRY(place_landmarks());
        }

        // Farthest squared distance from each final landmark to its cell's points (query seeds).
        KNN_TRY_CUDA(cudaMemsetAsync(far, 0, cells * 8ull, s));
        tc_cell_far_kernel<<<ceil_div(n, 256), 256, 0, s>>>(src, stride, dims, k0, n, T.land.as<float>(), ps, far);
        KNN_LAUNCHED();
        {
            std::vector<unsigned long long> hfar(cells);
            KNN_TRY_CUDA(cudaMemcpyAsync(hfar.data(), far, cells * 8ull, cudaMemcpyDeviceToHost, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));
            std::vector<float> cf(cells);
            for (uint32_t c = 0; c < cells; ++c) {
                const uint32_t bits = static_cast<uint32_t>(hfar[c] >> 32);
                std::memcpy(&cf[c], &bits, 4);
            }
            KNN_TRY(T.cell_far.alloc(cells * 4ull));
            KNN_TRY_CUDA(cudaMemcpyAsync(T.cell_far.ptr, cf.data(), cells * 4ull, cudaMemcpyHostToDevice, s));
            KNN_TRY_CUDA(cudaStreamSynchronize(s));
        }
        // The landmarks as a 16-bit operand image with their scaled norms (+inf on padding), for
        // the query-time assignment GEMM.
        {
            const uint32_t ltiles = ceil_div(cells, kTileN);
            KNN_TRY(T.limg.alloc(static_cast<size_t>(ltiles) * b_bytes(H)));
            KNN_TRY(T.lnorm.alloc(static_cast<size_t>(ltiles) * kTileN * 4));
            tc_pack_kernel<<<ceil_div(ltiles * kTileN, 128), 128, 0, s>>>(T.land.as<float>(), ps, dims, nullptr, cells,
                                                                          nullptr, kTileN, H, T.f16, T.scale,
                                                                          T.limg.as<uint8_t>(), T.lnorm.as<float>(),
                                                                          INFINITY, nullptr, 0, nullptr, nullptr,
                                                                          ltiles * kTileN, nullptr);
            KNN_LAUNCHED();
        }


        // Points by cell (stable), each cell's rows filling whole tiles.
        bool alt = false;
        KNN_TRY(radix_sort_pairs(k0, v0, k1, v1, n, static_cast<int>(log2_ceil(cells + 1)), st, s, &alt));
        const uint32_t* keys = alt ? k1 : k0;
        const uint32_t* vals = alt ? v1 : v0;
        std::vector<uint32_t> hkeys(n);
        KNN_TRY_CUDA(cudaMemcpyAsync(hkeys.data(), keys, n * 4ull, cudaMemcpyDeviceToHost, s));
        KNN_TRY_CUDA(cudaStreamSynchronize(s));
        cell_start.assign(cells + 1, 0);
        cell_tile.assign(cells + 1, 0);
        for (uint32_t i = 0; i < n; ++i) cell_start[hkeys[i] + 1]++;
        for (uint32_t c = 0; c < cells; ++c) {
            cell_tile[c + 1] = cell_tile[c] + ceil_div(cell_start[c + 1], kTileN);
            cell_start[c + 1] += cell_start[c];
        }
        const uint32_t prows = cell_tile[cells] * kTileN;
        KNN_TRY(T.cell_start.alloc((cells + 1) * 4ull));
        KNN_TRY(T.cell_tile.alloc((cells + 1) * 4ull));
        KNN_TRY(rowmap.alloc(prows * 4ull));
        KNN_TRY_CUDA(cudaMemcpyAsync(T.cell_start.ptr, cell_start.data(), (cells + 1) * 4ull, cudaMemcpyHostToDevice, s));
        KNN_TRY_CUDA(cudaMemcpyAsync(T.cell_tile.ptr, cell_tile.data(), (cells + 1) * 4ull, cudaMemcpyHostToDevice, s));
        KNN_TRY_CUDA(cudaMemsetAsync(rowmap.ptr, 0xFF, prows * 4ull, s));
        tc_place_kernel<<<ceil_div(n, 256), 256, 0, s>>>(keys, vals, n, T.cell_start.as<uint32_t>(),
                                                         T.cell_tile.as<uint32_t>(), rowmap.as<uint32_t>());
        KNN_LAUNCHED();


    }
    const uint32_t ptiles = cell_tile[cells];
    const uint32_t prows = ptiles * kTileN;
    const uint32_t ctiles = ceil_div(cells, kTileN);
    T.cells = cells;
    T.ptiles = ptiles;
    T.ctiles = ctiles;

    // Point operand image, norms, FP32 copy, ids, per-tile norm bounds.
    KNN_TRY(T.img.alloc(static_cast<size_t>(ptiles) * b_bytes(H)));
    KNN_TRY(T.norm.alloc(prows * 4ull));
    KNN_TRY(T.pts.alloc(static_cast<size_t>(prows) * ps * 4));
    KNN_TRY(T.ids.alloc(prows * 4ull));
    KNN_TRY(T.pmax.alloc(ptiles * 4ull));
    tc_pack_kernel<<<ceil_div(prows, 128), 128, 0, s>>>(src, stride, dims, rowmap.as<uint32_t>(), prows, nullptr, kTileN,
                                                        H, T.f16, T.scale, T.img.as<uint8_t>(), T.norm.as<float>(),
                                                        INFINITY, T.pts.as<float>(), ps, src_ids, T.ids.as<uint32_t>(),
                                                        prows, small.as<int>() + 1);
    KNN_LAUNCHED();
    tc_tile_max_kernel<<<ceil_div(ptiles, 128), 128, 0, s>>>(T.norm.as<float>(), ptiles, rel_margin(dims),
                                                             T.pmax.as<float>());
    KNN_LAUNCHED();

    // Cell centres and radii (scaled), their operand image and row data; tree cells' boxes.
    DevBuf cb;
    KNN_TRY(cb.alloc(ctiles * kTileN * 4ull));
    KNN_TRY(T.ccentre.alloc(static_cast<size_t>(cells) * ps * 4));
    KNN_TRY(T.cradius.alloc(cells * 4ull));
    float* centre = T.ccentre.as<float>();
    float* radius = T.cradius.as<float>();
    float* cnorm = cb.as<float>();
    if (T.tree) {
        T.bd = dims <= 16 ? 16u : 32u;
        KNN_TRY(T.box.alloc(static_cast<size_t>(cells) * 2 * T.bd * 4));
        tc_box_kernel<<<ceil_div(cells * 32, 128), 128, 0, s>>>(T.pts.as<float>(), ps, dims, T.scale, T.norm.as<float>(),
                                                                T.cell_tile.as<uint32_t>(), cells, T.bd, T.box.as<float>());
        KNN_LAUNCHED();
    }
    tc_cell_ball_kernel<<<ceil_div(cells * 32, 128), 128, 0, s>>>(T.pts.as<float>(), ps, dims, T.scale, T.norm.as<float>(),
                                                                  T.cell_tile.as<uint32_t>(), cells, rel_margin(dims),
                                                                  centre, radius);
    KNN_LAUNCHED();
    KNN_TRY(T.cimg.alloc(static_cast<size_t>(ctiles) * b_bytes(H)));
    KNN_TRY(T.cdata.alloc(static_cast<size_t>(ctiles) * kRowData * 4));
    KNN_TRY(T.cmax.alloc(ctiles * 4ull));
    tc_pack_kernel<<<ceil_div(ctiles * kTileN, 128), 128, 0, s>>>(centre, ps, dims, nullptr, cells, nullptr, kTileN, H,
                                                                  T.f16, 1.0f, T.cimg.as<uint8_t>(), cnorm, INFINITY,
                                                                  nullptr, 0, nullptr, nullptr, ctiles * kTileN,
                                                                  small.as<int>() + 1);
    KNN_LAUNCHED();
    tc_cdata_kernel<<<ceil_div(ctiles * kTileN, 256), 256, 0, s>>>(cnorm, radius, cells, ctiles, T.cdata.as<float>());
    KNN_LAUNCHED();
    tc_tile_max_kernel<<<ceil_div(ctiles, 128), 128, 0, s>>>(cnorm, ctiles, rel_margin(dims), T.cmax.as<float>());
    KNN_LAUNCHED();
    int bad = 0;
    KNN_TRY_CUDA(cudaMemcpyAsync(&bad, small.as<int>() + 1, 4, cudaMemcpyDeviceToHost, s));
    KNN_TRY_CUDA(cudaStreamSynchronize(s));
    if (bad) return fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: a point's norm is not finite");
    T.usable = true;
    ix->device_bytes += T.img.bytes + T.norm.bytes + T.pts.bytes + T.ids.bytes + T.pmax.bytes + T.cimg.bytes +
                        T.cdata.bytes + T.cmax.bytes + T.land.bytes + T.cell_tile.bytes + T.cell_start.bytes +
                        T.cell_far.bytes + T.limg.bytes + T.lnorm.bytes + T.node_dim.bytes + T.node_val.bytes + T.node_leaf.bytes + T.ccentre.bytes +
                        T.cradius.bytes + T.box.bytes;
    return KNN_OK;
}

template <int PS>
static int rescore(RescoreArgs ra, uint32_t count, cudaStream_t s) {
    // Rows of 128 floats: one stage per warp (about 19 KB with the buffer), one warp per block, so
    // that ~11 warps fit an SM; narrower rows: two stages, four warps per block.
    constexpr int S = PS >= 128 ? 1 : 2;
    ra.buf = rescore_buf(ra.k);
    ra.warp_bytes = S * RescoreShape<PS>::kStageBytes + PS * 4 + ra.buf * 8;
    const uint32_t warps = S == 1 ? 1u : kRescoreWarps;
    const size_t smem = static_cast<size_t>(warps) * ra.warp_bytes;
    KNN_TRY_CUDA(cudaFuncSetAttribute(tc_rescore_kernel<PS, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
    tc_rescore_kernel<PS, S><<<ceil_div(count, warps), 32 * warps, smem, s>>>(ra);
    KNN_LAUNCHED();
    return KNN_OK;
}

// The exhaustive search's grid, and its partial-list slots per query batch: at most
// max(kExhChunks nq, grid) lists of k keys (exh_chunks).
static uint32_t exh_grid() { return 4u * static_cast<uint32_t>(sm_count()); }
static size_t exh_slots(uint32_t nq) { return std::max<size_t>(static_cast<size_t>(nq) * kExhChunks, exh_grid()); }

uint32_t tc_default_cap(uint32_t k) { return std::min(4096u, std::max(1024u, 16u * k)); }

int bf_tc_query(knn_index* ix, const QueryArgs& a, const QueryPlan& plan, cudaStream_t s) {
    const Range range("tensor-core filter query");
    const uint32_t H = halves(ix->dims);
    if (!tc_supported(ix->dims, a.k)) return fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: dims %u, k %u", ix->dims, a.k);
    QueryPlan plain = plan;
    plain.timing = false;
    plain.bf16 = false;
    // An index the 16-bit formats cannot hold (non-finite norms) answers by its plain search.
    const int prc = tc_prepare(ix, s);
    if (prc == KNN_ERR_UNSUPPORTED) return query_structure(ix, a, plain, s);
    KNN_TRY(prc);
    const auto& T = ix->tc;
    const uint32_t nq = a.count;
    const uint32_t qtiles = ceil_div(nq, kTileM);
    const uint32_t qrows = qtiles * kTileM;
    const uint32_t cap = plan.tc_cap ? plan.tc_cap : tc_default_cap(a.k);
    const size_t qimg_bytes = static_cast<size_t>(qtiles) * a_bytes(H);
    KNN_TRY(ix->tc.ws.reserve(carve_bytes({nq * 4ull, nq * 4ull, nq * 4ull, nq * 4ull, radix_sort_temp_bytes(nq),
                                            qimg_bytes, qrows * 4ull, qtiles * 16ull,
                                            static_cast<size_t>(nq) * cap * 4, static_cast<size_t>(nq) * cap * 4,
                                            nq * 4ull, nq * 4ull, nq * 4ull, nq * 4ull, nq * 4ull,
                                            exh_slots(nq) * a.k * 8, 256})));
    Carver c(ix->tc.ws.ptr);
    uint32_t* k0 = c.take<uint32_t>(nq);
    uint32_t* v0 = c.take<uint32_t>(nq);
    uint32_t* k1 = c.take<uint32_t>(nq);
    uint32_t* v1 = c.take<uint32_t>(nq);
    void* st = c.take<uint8_t>(radix_sort_temp_bytes(nq));
    uint8_t* qimg = c.take<uint8_t>(qimg_bytes);
    float* qnorm = c.take<float>(qrows);
    uint32_t* qhome = c.take<uint32_t>(qtiles * 4ull);
    uint32_t* cand = c.take<uint32_t>(static_cast<size_t>(nq) * cap);
    float* cand_v = c.take<float>(static_cast<size_t>(nq) * cap);
    uint32_t* cnt = c.take<uint32_t>(nq);
    float* final_t = c.take<float>(nq);
    uint32_t* retry = c.take<uint32_t>(nq);
    float* seed = c.take<float>(nq);
    float* retry_r2 = c.take<float>(nq);
    uint64_t* xkeys = c.take<uint64_t>(exh_slots(nq) * a.k);
    uint32_t* small = c.take<uint32_t>(64);  // [0] retry count, [1] error flag, [2] filter tile counter
    KNN_TRY_CUDA(cudaMemsetAsync(small, 0, 64 * sizeof(uint32_t), s));

    // Queries by cell (rows past the live count sort last), with a seed bound from their cell.
    if (T.tree)
        KNN_TRY(launch_descend(ix->dp, a.queries, ix->dims, nq, a.order, a.count_dev, T, a.k, k0, v0, seed, s));
    else {
        // The rows' operand tiles in batch order, then the nearest landmark by the GEMM.
        tc_pack_kernel<<<ceil_div(qrows, 128), 128, 0, s>>>(a.queries, ix->dims, ix->dims, a.order, nq, a.count_dev,
                                                            kTileM, H, T.f16, T.scale, qimg, qnorm, 0.0f, nullptr, 0,
                                                            nullptr, nullptr, qrows, nullptr);
        KNN_LAUNCHED();
        if (H != 1 && H != 2) return fail(KNN_ERR_UNSUPPORTED, "landmark layout at %u dims", ix->dims);
        auto kern = H == 1 ? tc_assign_mma_kernel<1> : tc_assign_mma_kernel<2>;
        const size_t smem = assign_mma_smem(H);
        KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        kern<<<qtiles, 128, smem, s>>>(qimg, T.limg.as<uint8_t>(), T.lnorm.as<float>(), ceil_div(T.cells, kTileN),
                                       T.cells, T.f16 ? idesc_f16(kTileM, kTileN) : idesc_bf16(kTileM, kTileN), nq,
                                       a.order, a.count_dev, a.queries, ix->dims, T.land.as<float>(), T.ps,
                                       T.cell_far.as<float>(), T.cell_start.as<uint32_t>(), a.k, k0, v0, seed,
                                       reinterpret_cast<int*>(small + 1));
        KNN_LAUNCHED();
    }
    bool alt = false;
    KNN_TRY(radix_sort_pairs(k0, v0, k1, v1, nq, static_cast<int>(log2_ceil(T.cells + 1)), st, s, &alt));
    const uint32_t* cell_sorted = alt ? k1 : k0;
    const uint32_t* order = alt ? v1 : v0;
    tc_pack_kernel<<<ceil_div(qrows, 128), 128, 0, s>>>(a.queries, ix->dims, ix->dims, order, nq, a.count_dev, kTileM, H,
                                                        T.f16, T.scale, qimg, qnorm, 0.0f, nullptr, 0, nullptr, nullptr,
                                                        qrows, nullptr);
    KNN_LAUNCHED();
    tc_home_kernel<<<ceil_div(qtiles, 128), 128, 0, s>>>(cell_sorted, a.count_dev, nq, T.cell_start.as<uint32_t>(),
                                                         T.cell_tile.as<uint32_t>(), T.cells,
                                                         std::max(2 * a.k, 512u), qtiles, qhome);
    KNN_LAUNCHED();

    TcParams p{};
    p.qimg = qimg;
    p.pimg = T.img.as<uint8_t>();
    p.cimg = T.cimg.as<uint8_t>();
    p.qnorm = qnorm;
    p.pnorm = T.norm.as<float>();
    p.cdata = T.cdata.as<float>();
    p.pmax = T.pmax.as<float>();
    p.cmax = T.cmax.as<float>();
    p.cell_tile = T.cell_tile.as<uint32_t>();
    p.qhome = qhome;
    p.box = T.tree ? T.box.as<float>() : nullptr;
    p.queries = a.queries;
    p.dims = ix->dims;
    p.scale = T.scale;
    p.cells = T.cells;
    p.ctiles = T.ctiles;
    p.nq = nq;
    p.ksteps = ceil_div(ix->dims, 16);
    p.idesc = T.f16 ? idesc_f16(kTileM, kTileN) : idesc_bf16(kTileM, kTileN);
    p.idesc_half = T.f16 ? idesc_f16(kTileM, kTileN / 2) : idesc_bf16(kTileM, kTileN / 2);
    p.b = make_bounds(ix->dims, T.f16, T.scale);
    p.s2 = T.scale * T.scale;
    p.max_d2 = a.max_d2;
    p.radii = a.radii;
    p.seed = seed;
    p.order = order;
    p.live_count = a.count_dev;
    p.k = a.k;
    p.cap = cap;
    // T' in a heap where two blocks per SM still fit it, unless the plan asks for codes.
    const bool heap = !plan.tc_codes && filter_heap_fits(H, a.k);
    p.codes = filter_codes(H, a.k, heap);
    p.cand = cand;
    p.cand_v = cand_v;
    p.cand_count = cnt;
    p.final_t = final_t;
    p.counters = a.counters;
    p.error = reinterpret_cast<int*>(small + 1);
    p.give_up = plan.test_give_up ? 1u : 0u;
    p.qtiles = qtiles;
    p.tile_counter = small + 2;
    // Rows no block settles (a block that gave up) keep these: the plain search within a huge radius.
    KNN_TRY_CUDA(cudaMemsetAsync(cnt, 0xFF, nq * 4ull, s));
    KNN_TRY_CUDA(cudaMemsetAsync(final_t, 0x7F, nq * 4ull, s));
    const size_t smem = filter_launch_smem(H, a.k, heap);
    const uint32_t acc = accumulators(H, a.k, heap);
    // Persistent blocks (one or two per SM, as TMEM allows) take query tiles in turn, so that
    // tiles of uneven cost balance across the SMs instead of leaving a partial last wave.
    const uint32_t grid = std::min<uint32_t>(qtiles, (acc == 2 ? 1u : 2u) * static_cast<uint32_t>(sm_count()));
    void (*kern)(const TcParams) = nullptr;
    // Up to 32 dims (tree layout, boxes of 16 or 32 dims): 32- or 64-byte rows; beyond, 128-byte.
    if (heap) {  // (one accumulator: the heap mode fits two blocks per SM)
        if (H == 32) kern = tc_filter_kernel<32, 1, 16, true>;
        else if (H == 64) kern = tc_filter_kernel<64, 1, 32, true>;
        else if (H == 1) kern = tc_filter_kernel<1, 1, 0, true>;
        else kern = tc_filter_kernel<2, 1, 0, true>;
    } else if (H == 32) {
        kern = acc == 1 ? tc_filter_kernel<32, 1, 16, false> : tc_filter_kernel<32, 2, 16, false>;
    } else if (H == 64) {
        kern = acc == 1 ? tc_filter_kernel<64, 1, 32, false> : tc_filter_kernel<64, 2, 32, false>;
    } else if (H == 1) {
        kern = acc == 1 ? tc_filter_kernel<1, 1, 0, false> : tc_filter_kernel<1, 2, 0, false>;
    } else {
        kern = acc == 1 ? tc_filter_kernel<2, 1, 0, false> : tc_filter_kernel<2, 2, 0, false>;
    }
    if ((H >= 32) != T.tree || (H == 32 && T.bd != 16) || (H == 64 && T.bd != 32))
        return fail(KNN_ERR_UNSUPPORTED, "tensor-core filter: layout %u for a %s layout", H, T.tree ? "tree" : "landmark");
    KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    if (plan.timing) KNN_TRY(ix->timing.begin(s));
    kern<<<grid, kThreads, smem, s>>>(p);
    KNN_LAUNCHED();
    if (plan.timing) KNN_TRY(ix->timing.end(s));

    RescoreArgs ra{};
    ra.pts = T.pts.as<float>();
    ra.ids = T.ids.as<uint32_t>();
    ra.pnorm = T.norm.as<float>();
    ra.pmax = T.pmax.as<float>();
    ra.queries = a.queries;
    ra.dims = ix->dims;
    ra.nq = nq;
    ra.cap = cap;
    ra.k = a.k;
    ra.max_d2 = a.max_d2;
    ra.radii = a.radii;
    ra.order = order;
    ra.live_count = a.count_dev;
    ra.cand = cand;
    ra.cand_v = cand_v;
    ra.cand_count = cnt;
    ra.qnorm = qnorm;
    ra.final_t = final_t;
    ra.b = p.b;
    ra.out_idx = a.out_idx;
    ra.out_dist = a.out_dist;
    ra.retry = retry;
    ra.retry_count = small;
    ra.retry_r2 = retry_r2;
    ra.inv_s2 = 1.0f / p.s2;
    ra.counters = a.counters;
    switch (T.ps) {
        case 4: KNN_TRY(rescore<4>(ra, nq, s)); break;
        case 8: KNN_TRY(rescore<8>(ra, nq, s)); break;
        case 16: KNN_TRY(rescore<16>(ra, nq, s)); break;
        case 32: KNN_TRY(rescore<32>(ra, nq, s)); break;
        case 64: KNN_TRY(rescore<64>(ra, nq, s)); break;
        default: KNN_TRY(rescore<128>(ra, nq, s)); break;
    }
    // Queries whose candidates overflowed, that the 16-bit format could not hold, or whose filter
    // block gave up: exhaustive search over the layout, one block each, within the radius the
    // filter proved (at least k points lie inside it, so the answer is unchanged).
    const uint32_t eg = exh_grid();
#define KNN_EXH(P_)                                                                                                \
    case P_:                                                                                                       \
        tc_exhaustive_kernel<P_><<<eg, kExhThreads, 0, s>>>(T.pts.as<float>(), T.ids.as<uint32_t>(),              \
                                                             T.norm.as<float>(), T.ptiles * kTileN, a.queries,       \
                                                             ix->dims, a.k, retry, small, retry_r2, xkeys);          \
        break;
    switch (T.ps) {
        KNN_EXH(4) KNN_EXH(8) KNN_EXH(16) KNN_EXH(32) KNN_EXH(64)
        default: KNN_EXH(128)
    }
#undef KNN_EXH
    KNN_LAUNCHED();
    const uint32_t prows = T.ptiles * kTileN;
    uint32_t n2 = 1;  // the merge's keys: as many chunks as exh_chunks can give, k each
    while (n2 < std::max(kExhChunks, std::min(kExhMaxChunks, prows / kExhMinRows)) * a.k) n2 <<= 1;
    KNN_TRY_CUDA(cudaFuncSetAttribute(tc_exhaustive_merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(n2 * 8)));
    tc_exhaustive_merge_kernel<<<eg, kExhThreads, n2 * 8, s>>>(a.k, prows, retry, small, retry_r2, xkeys,
                                                               a.out_idx, a.out_dist);
    KNN_LAUNCHED();
    return KNN_OK;
}

int tc_selftest(uint32_t dims, float* max_rel_err, uint32_t* bad) {
    const uint32_t H = halves(dims);
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
    const size_t ab = a_bytes(H), bb = b_bytes(H);
    KNN_TRY(buf.alloc(carve_bytes({hq.size() * 4, hp.size() * 4, ab, bb, qn * 4ull, pn * 4ull, qn * pn * 4ull, 64})));
    Carver c(buf.ptr);
    float* dq = c.take<float>(hq.size());
    float* dp = c.take<float>(hp.size());
    uint8_t* qimg = c.take<uint8_t>(ab);
    uint8_t* pimg = c.take<uint8_t>(bb);
    float* qnm = c.take<float>(qn);
    float* pnm = c.take<float>(pn);
    float* out = c.take<float>(static_cast<size_t>(qn) * pn);
    int* err = c.take<int>(16);
    KNN_TRY_CUDA(cudaMemcpy(dq, hq.data(), hq.size() * 4, cudaMemcpyHostToDevice));
    KNN_TRY_CUDA(cudaMemcpy(dp, hp.data(), hp.size() * 4, cudaMemcpyHostToDevice));
    double worst = 0;
    uint32_t nbad = 0;
    std::vector<float> ho(static_cast<size_t>(qn) * pn);
    for (int f16 = 0; f16 < 2; ++f16) {
        KNN_TRY_CUDA(cudaMemset(err, 0, 64));
        tc_pack_kernel<<<1, 128>>>(dq, dims, dims, nullptr, qn, nullptr, kTileM, H, f16 != 0, 1.0f, qimg, qnm, 0.0f,
                                   nullptr, 0, nullptr, nullptr, qn, nullptr);
        tc_pack_kernel<<<2, 128>>>(dp, dims, dims, nullptr, pn, nullptr, kTileN, H, f16 != 0, 1.0f, pimg, pnm, 0.0f,
                                   nullptr, 0, nullptr, nullptr, pn, nullptr);
        const size_t smem = 1024 + ab + bb + 64;
        auto kern = H == 32 ? tc_selftest_kernel<32> : H == 64 ? tc_selftest_kernel<64> : H == 1 ? tc_selftest_kernel<1>
                                                                                        : tc_selftest_kernel<2>;
        KNN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        kern<<<1, 128, smem>>>(qimg, pimg, f16 ? idesc_f16(kTileM, kTileN) : idesc_bf16(kTileM, kTileN), out, err);
        KNN_LAUNCHED_N(3);
        KNN_TRY_CUDA(cudaDeviceSynchronize());
        int herr = 0;
        KNN_TRY_CUDA(cudaMemcpy(ho.data(), out, ho.size() * 4, cudaMemcpyDeviceToHost));
        KNN_TRY_CUDA(cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost));
        if (herr) return fail(KNN_ERR_DEVICE_LIMIT, "tensor-core self-test kernel timed out");
        // Inputs are multiples of 1/250 with |x| <= 4; the reference rounds them to the operand
        // format on the host and sums the products in double.
        auto round16 = [&](float x) {
            if (f16) return __half2float(__float2half_rn(x));
            return __bfloat162float(__float2bfloat16_rn(x));
        };
        for (uint32_t i = 0; i < qn; ++i)
            for (uint32_t j = 0; j < pn; ++j) {
                double ref = 0, mag = 0;
                for (uint32_t d = 0; d < dims; ++d) {
                    const double t = static_cast<double>(round16(hq[i * dims + d])) * round16(hp[j * dims + d]);
                    ref += t;
                    mag += std::fabs(t);
                }
                const double e = std::fabs(ho[static_cast<size_t>(i) * pn + j] - ref) / std::max(mag, 1e-30);
                worst = std::max(worst, e);
                if (e > dims * std::ldexp(1.0, -20)) ++nbad;
            }
    }
    *max_rel_err = static_cast<float>(worst);
    *bad = nbad;
    return KNN_OK;
}

}  // namespace knn
