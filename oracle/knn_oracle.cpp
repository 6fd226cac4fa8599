// CPU oracle for the exact-kNN hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the engine (cudaexactknn_gb300/, include/) links or
// calls this file.  It is used by tests/ as the checker, by __graft_entry__.smoke() as the
// checker, and by bench.py as the timed CPU baseline ("port" kind).
//
// It restates, in plain C++, the reference's CPU algorithms for the path:
//   * distance                  src/KnnTrees.cuh:65-77   (sequential sum over d of (a[d]-b[d])^2)
//   * result key / tie rule     src/KnnTrees.cuh:122-134 (key = bits(dist2) << 32 | uint32(index))
//   * sorted-insertion tracker  src/KnnTrees.cuh:136-152
//   * max-heap tracker          src/KnnTrees.cuh:154-189
//   * BruteForce<D>::batchKnn   src/BruteForce.cuh:27-44
//   * KdTree<D> build + query   src/KdTree.cuh:27-71 (build), 79-158 (query)
//   * BallTree<D> build + query src/BallTree.cuh:27-137 (build), 144-237 (query)
//
// Two arithmetic modes for the distance:
//   fma = 1  acc = fmaf(t, t, acc) in dimension order.  This is what nvcc emits for the
//            reference's device code (it contracts `result += d*d`), and what the GB300 engine
//            computes, so it is the bit-exact parity mode.
//   fma = 0  acc = acc + t*t with two roundings, which is what the reference's CPU classes
//            compute when the host compiler does not contract (x86-64 without FMA).
// The file is compiled with -ffp-contract=off so that the two modes stay distinct.
//
// Pruning modes for the trees:
//   strict = 0  prune when bound >= current k-th distance (the reference's rule,
//               src/KdTree.cuh:114,130 and src/BallTree.cuh:177,205,209).  At exact ties on the
//               k-th distance the answer then depends on traversal order.
//   strict = 1  prune only when bound > k-th distance, so every tree returns the same
//               key-ordered top-k as brute force.
//
// Every batch function can spread queries over host threads (threads > 1); each query is
// independent, so results do not depend on the thread count.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

inline uint32_t float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof(u));
    return u;
}

inline float bits_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, sizeof(f));
    return f;
}

// key = (bits(dist2) << 32) | uint32(index); compared as an unsigned 64-bit integer.
// (src/KnnTrees.cuh:122-128)
inline uint64_t make_key(float dist2, int32_t index) {
    return (static_cast<uint64_t>(float_bits(dist2)) << 32) | static_cast<uint32_t>(index);
}

inline float key_dist(uint64_t key) { return bits_float(static_cast<uint32_t>(key >> 32)); }

// Sequential squared distance in dimension order (src/KnnTrees.cuh:65-77).
inline float dist2(const float* a, const float* b, uint32_t dims, bool use_fma) {
    float acc = 0.0f;
    if (use_fma) {
        for (uint32_t d = 0; d < dims; ++d) {
            const float t = a[d] - b[d];
            acc = std::fmaf(t, t, acc);
        }
    } else {
        for (uint32_t d = 0; d < dims; ++d) {
            const float t = a[d] - b[d];
            const float sq = t * t;
            acc = acc + sq;
        }
    }
    return acc;
}

// Top-k tracker over u64 keys.  Sorted mode keeps keys ascending (src/KnnTrees.cuh:136-152);
// heap mode keeps a max-heap rooted at slot 0 (src/KnnTrees.cuh:154-189).  Both return the
// current k-th distance, which is the pruning radius of the tree searches.
struct Tracker {
    std::vector<uint64_t> slot;
    uint32_t k;
    bool heap;

    Tracker(uint32_t k_, bool heap_) : slot(k_), k(k_), heap(heap_) {}

    void reset(float max_dist2) {
        std::fill(slot.begin(), slot.end(), make_key(max_dist2, -1));
    }

    float worst() const { return key_dist(heap ? slot[0] : slot[k - 1]); }

    float offer(int32_t index, float d2) {
        uint64_t x = make_key(d2, index);
        if (!heap) {
            if (x < slot[k - 1]) {
                // Bubble the new key through the sorted array; the largest key falls off.
                for (uint32_t i = 0; i < k; ++i) {
                    const uint64_t cur = slot[i];
                    slot[i] = std::min(cur, x);
                    x = std::max(cur, x);
                }
            }
            return key_dist(slot[k - 1]);
        }
        if (x < slot[0]) {
            // Replace the root and sift the new key down.
            uint32_t pos = 0;
            for (;;) {
                const uint32_t l = 2 * pos + 1;
                if (l >= k) break;
                uint32_t big = l;
                if (l + 1 < k && slot[l + 1] > slot[l]) big = l + 1;
                if (slot[big] <= x) break;
                slot[pos] = slot[big];
                pos = big;
            }
            slot[pos] = x;
        }
        return key_dist(slot[0]);
    }

    void emit(int32_t* idx_row, float* dist_row) const {
        for (uint32_t i = 0; i < k; ++i) {
            idx_row[i] = static_cast<int32_t>(static_cast<uint32_t>(slot[i]));
            dist_row[i] = key_dist(slot[i]);
        }
    }
};

inline uint32_t log2_ceil(uint32_t v) {
    // Smallest r >= 1 with 2^r >= v (src/KnnTrees.cuh:84-93).
    uint32_t r = 1;
    uint64_t c = 2;
    while (c < v) {
        c *= 2;
        r += 1;
    }
    return r;
}

template <class Fn>
void parallel_queries(uint32_t nq, int threads, Fn&& fn) {
    if (threads <= 1 || nq < 2) {
        fn(0u, nq);
        return;
    }
    const uint32_t t = static_cast<uint32_t>(std::min<int64_t>(threads, nq));
    std::vector<std::thread> pool;
    pool.reserve(t);
    for (uint32_t i = 0; i < t; ++i) {
        const uint32_t lo = static_cast<uint32_t>(static_cast<uint64_t>(nq) * i / t);
        const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(nq) * (i + 1) / t);
        pool.emplace_back([&fn, lo, hi] { fn(lo, hi); });
    }
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------------------------
// k-d tree (src/KdTree.cuh).  Balanced: a node of n points gives ceil(n/2) to the left child;
// the split value is the largest left value along dimension depth % dims; internal nodes form
// an implicit heap (children 2i+1, 2i+2); leaves hold 2^skips index slots padded with -1.
// ---------------------------------------------------------------------------------------------
struct KdTree {
    uint32_t dims = 0, skips = 0, node_depth = 0, leaf_slots = 0, node_count = 0, n = 0;
    std::vector<float> split;       // node_count
    std::vector<int32_t> leaf_idx;  // 2^(node_depth) * leaf_slots
    std::vector<float> pts;         // n * dims (copy of the input)

    void build_rec(uint32_t node, int32_t* ids, uint32_t size, uint32_t depth) {
        if (depth < node_depth) {
            const uint32_t right = size / 2;
            const uint32_t left = size - right;
            const uint32_t dim = depth % dims;
            const float* p = pts.data();
            const uint32_t D = dims;
            if (size > 0) {
                std::nth_element(ids, ids + left - 1, ids + size, [p, D, dim](int32_t a, int32_t b) {
                    return p[static_cast<size_t>(a) * D + dim] < p[static_cast<size_t>(b) * D + dim];
                });
                split[node] = p[static_cast<size_t>(ids[left - 1]) * D + dim];
            } else {
                split[node] = 0.0f;
            }
            build_rec(2 * node + 1, ids, left, depth + 1);
            build_rec(2 * node + 2, ids + left, right, depth + 1);
            return;
        }
        const size_t base = static_cast<size_t>(leaf_slots) * (node - node_count);
        for (uint32_t s = 0; s < leaf_slots; ++s) leaf_idx[base + s] = s < size ? ids[s] : -1;
    }

    void build(const float* p, uint32_t n_, uint32_t dims_, uint32_t skips_) {
        n = n_;
        dims = dims_;
        const uint32_t l2 = log2_ceil(n);
        skips = std::min(skips_, l2 - 1);
        node_depth = l2 - skips;
        leaf_slots = 1u << skips;
        node_count = (1u << node_depth) - 1;
        split.assign(node_count, 0.0f);
        leaf_idx.assign(static_cast<size_t>(1u << node_depth) * leaf_slots, -1);
        pts.assign(p, p + static_cast<size_t>(n) * dims);
        std::vector<int32_t> ids(n);
        std::iota(ids.begin(), ids.end(), 0);
        build_rec(0, ids.data(), n, 0);
    }

    // Depth-first search, closest child first; far children are pushed when their splitting
    // plane is within the current radius (src/KdTree.cuh:98-143).
    void query(const float* q, Tracker& tr, float max_dist2, bool use_fma, bool strict) const {
        struct Entry {
            uint32_t node, depth;
            float bound;
        };
        Entry stack[64];
        uint32_t top = 0;
        stack[top++] = {0, 0, 0.0f};
        float radius = max_dist2;
        while (top) {
            const Entry e = stack[--top];
            if (strict ? e.bound > radius : e.bound >= radius) continue;
            uint32_t node = e.node, depth = e.depth;
            while (depth < node_depth) {
                const uint32_t dim = depth % dims;
                const float diff = q[dim] - split[node];
                const uint32_t l = 2 * node + 1;
                const uint32_t close_child = diff < 0.0f ? l : l + 1;
                const uint32_t far_child = diff < 0.0f ? l + 1 : l;
                const float b = diff * diff;
                if (strict ? b <= radius : b < radius) stack[top++] = {far_child, depth + 1, b};
                node = close_child;
                depth += 1;
            }
            const size_t base = static_cast<size_t>(leaf_slots) * (node - node_count);
            for (uint32_t s = 0; s < leaf_slots; ++s) {
                const int32_t id = leaf_idx[base + s];
                if (id == -1) break;
                const float d2 = dist2(q, &pts[static_cast<size_t>(id) * dims], dims, use_fma);
                radius = tr.offer(id, d2);
            }
        }
    }
};

// ---------------------------------------------------------------------------------------------
// Ball tree (src/BallTree.cuh).  At each node: mean and per-dimension variance of its points;
// split on the highest-variance dimension (strict >, first wins) at the left median
// (ceil(n/2) to the left); each node records both children's centroid and radius
// (radius = sqrt of the largest squared distance to the centroid).  skips >= 1.
// ---------------------------------------------------------------------------------------------
struct BallTree {
    uint32_t dims = 0, skips = 0, node_depth = 0, leaf_slots = 0, node_count = 0, n = 0;
    // Per node: [left centroid (dims), left radius, right centroid (dims), right radius].
    std::vector<float> nodes;
    std::vector<int32_t> leaf_idx;
    std::vector<float> leaf_pts;
    std::vector<float> pts;

    size_t node_stride() const { return 2 * (static_cast<size_t>(dims) + 1); }

    float ball_lower_bound(const float* centre, float radius, const float* q) const {
        double s = 0.0;
        for (uint32_t d = 0; d < dims; ++d) {
            const double t = static_cast<double>(q[d]) - static_cast<double>(centre[d]);
            s += t * t;
        }
        const double b = std::max(std::sqrt(s) - static_cast<double>(radius) * (1.0 + 1e-4), 0.0);
        return static_cast<float>(b * b * (1.0 - 1e-4));
    }

    void child_ball(const int32_t* ids, uint32_t cnt, float* centroid, float* radius, bool use_fma) {
        std::vector<float> sum(dims, 0.0f);
        for (uint32_t i = 0; i < cnt; ++i)
            for (uint32_t d = 0; d < dims; ++d) sum[d] += pts[static_cast<size_t>(ids[i]) * dims + d];
        for (uint32_t d = 0; d < dims; ++d) centroid[d] = sum[d] / static_cast<float>(cnt);
        float best = 0.0f;
        for (uint32_t i = 0; i < cnt; ++i) {
            const float d2 = dist2(centroid, &pts[static_cast<size_t>(ids[i]) * dims], dims, use_fma);
            if (d2 > best) best = d2;
        }
        *radius = std::sqrt(best);
    }

    void build_rec(uint32_t node, int32_t* ids, uint32_t size, bool use_fma) {
        if (node < node_count) {
            const uint32_t right = size / 2;
            const uint32_t left = size - right;
            std::vector<float> mean(dims, 0.0f), var(dims, 0.0f);
            for (uint32_t i = 0; i < size; ++i)
                for (uint32_t d = 0; d < dims; ++d) mean[d] += pts[static_cast<size_t>(ids[i]) * dims + d];
            for (uint32_t d = 0; d < dims; ++d) mean[d] = mean[d] / static_cast<float>(size);
            for (uint32_t i = 0; i < size; ++i)
                for (uint32_t d = 0; d < dims; ++d) {
                    const float t = pts[static_cast<size_t>(ids[i]) * dims + d] - mean[d];
                    if (use_fma)
                        var[d] = std::fmaf(t, t, var[d]);
                    else
                        var[d] += t * t;
                }
            for (uint32_t d = 0; d < dims; ++d) var[d] = var[d] / static_cast<float>(size);
            uint32_t dim = 0;
            float best = 0.0f;
            for (uint32_t d = 0; d < dims; ++d)
                if (var[d] > best) {
                    best = var[d];
                    dim = d;
                }
            const float* p = pts.data();
            const uint32_t D = dims;
            if (size > 0)
                std::nth_element(ids, ids + left - 1, ids + size, [p, D, dim](int32_t a, int32_t b) {
                    return p[static_cast<size_t>(a) * D + dim] < p[static_cast<size_t>(b) * D + dim];
                });
            float* rec = &nodes[node * node_stride()];
            child_ball(ids, left, rec, rec + dims, use_fma);
            child_ball(ids + left, right, rec + dims + 1, rec + 2 * dims + 1, use_fma);
            build_rec(2 * node + 1, ids, left, use_fma);
            build_rec(2 * node + 2, ids + left, right, use_fma);
            return;
        }
        const size_t base = static_cast<size_t>(leaf_slots) * (node - node_count);
        for (uint32_t s = 0; s < leaf_slots; ++s) {
            const int32_t id = s < size ? ids[s] : -1;
            leaf_idx[base + s] = id;
            if (id >= 0)
                std::memcpy(&leaf_pts[(base + s) * dims], &pts[static_cast<size_t>(id) * dims],
                            sizeof(float) * dims);
        }
    }

    void build(const float* p, uint32_t n_, uint32_t dims_, uint32_t skips_, bool use_fma) {
        n = n_;
        dims = dims_;
        const uint32_t l2 = log2_ceil(n);
        skips = std::min(std::max(skips_, 1u), l2 - 1);
        node_depth = l2 - skips;
        leaf_slots = 1u << skips;
        node_count = (1u << node_depth) - 1;
        nodes.assign(static_cast<size_t>(node_count) * node_stride(), 0.0f);
        const size_t slots = static_cast<size_t>(1u << node_depth) * leaf_slots;
        leaf_idx.assign(slots, -1);
        leaf_pts.assign(slots * dims, 0.0f);
        pts.assign(p, p + static_cast<size_t>(n) * dims);
        std::vector<int32_t> ids(n);
        std::iota(ids.begin(), ids.end(), 0);
        build_rec(0, ids.data(), n, use_fma);
    }

    // Depth-first search (src/BallTree.cuh:165-222): at each node, the distance from the query
    // to each child ball's border; descend into the closer ball, push the farther one when it
    // is within the radius, stop when even the closer ball is out of range.
    void query(const float* q, Tracker& tr, float max_dist2, bool use_fma, bool strict) const {
        struct Entry {
            uint32_t node;
            float bound;
        };
        Entry stack[64];
        uint32_t top = 0;
        stack[top++] = {0, 0.0f};
        float radius = max_dist2;
        auto out = [strict](float b, float r) { return strict ? b > r : b >= r; };
        while (top) {
            const Entry e = stack[--top];
            if (out(e.bound, radius)) continue;
            uint32_t node = e.node;
            bool pruned = false;
            while (node < node_count) {
                const float* rec = &nodes[node * node_stride()];
                const float dl = std::sqrt(dist2(rec, q, dims, use_fma)) - rec[dims];
                const float dr = std::sqrt(dist2(rec + dims + 1, q, dims, use_fma)) - rec[2 * dims + 1];
                float bl = std::max(dl, 0.0f) * std::max(dl, 0.0f);
                float br = std::max(dr, 0.0f) * std::max(dr, 0.0f);
                if (strict) {
                    // The float bound above can round past a point's own float distance (it
                    // does at exact ties).  Strict mode instead takes the centre distance in
                    // double, widens the radius and shrinks the bound by 1e-4 relative, which
                    // covers the float rounding of the radius and of the point distances for
                    // dims <= 128, so no point with distance <= the k-th is ever pruned.
                    bl = ball_lower_bound(rec, rec[dims], q);
                    br = ball_lower_bound(rec + dims + 1, rec[2 * dims + 1], q);
                }
                const uint32_t l = 2 * node + 1;
                const bool left_close = dl < dr;
                const uint32_t close_child = left_close ? l : l + 1;
                const uint32_t far_child = left_close ? l + 1 : l;
                const float close_b = left_close ? bl : br;
                const float far_b = left_close ? br : bl;
                if (out(close_b, radius)) {
                    pruned = true;
                    break;
                }
                if (!out(far_b, radius)) stack[top++] = {far_child, far_b};
                node = close_child;
            }
            if (pruned) continue;
            const size_t base = static_cast<size_t>(leaf_slots) * (node - node_count);
            for (uint32_t s = 0; s < leaf_slots; ++s) {
                const int32_t id = leaf_idx[base + s];
                if (id == -1) break;
                const float d2 = dist2(q, &leaf_pts[(base + s) * dims], dims, use_fma);
                radius = tr.offer(id, d2);
            }
        }
    }
};

}  // namespace

extern "C" {

// Brute force (src/BruteForce.cuh:27-44): every query against every point in index order.
int oracle_bf_knn(const float* pts, uint32_t n, uint32_t dims, const float* q, uint32_t nq,
                  float max_dist2, uint32_t k, int heap, int use_fma, int32_t* out_idx,
                  float* out_dist, int threads) {
    if (k == 0 || dims == 0) return 1;
    parallel_queries(nq, threads, [&](uint32_t lo, uint32_t hi) {
        Tracker tr(k, heap != 0);
        for (uint32_t i = lo; i < hi; ++i) {
            tr.reset(max_dist2);
            const float* qi = q + static_cast<size_t>(i) * dims;
            for (uint32_t j = 0; j < n; ++j)
                tr.offer(static_cast<int32_t>(j), dist2(qi, pts + static_cast<size_t>(j) * dims, dims, use_fma != 0));
            tr.emit(out_idx + static_cast<size_t>(i) * k, out_dist + static_cast<size_t>(i) * k);
        }
    });
    return 0;
}

void* oracle_kd_build(const float* pts, uint32_t n, uint32_t dims, uint32_t skips) {
    if (n == 0 || dims == 0) return nullptr;
    auto* t = new KdTree();
    t->build(pts, n, dims, skips);
    return t;
}

int oracle_kd_knn(const void* tree, const float* q, uint32_t nq, float max_dist2, uint32_t k,
                  int heap, int use_fma, int strict, int32_t* out_idx, float* out_dist, int threads) {
    const auto* t = static_cast<const KdTree*>(tree);
    if (!t || k == 0) return 1;
    parallel_queries(nq, threads, [&](uint32_t lo, uint32_t hi) {
        Tracker tr(k, heap != 0);
        for (uint32_t i = lo; i < hi; ++i) {
            tr.reset(max_dist2);
            t->query(q + static_cast<size_t>(i) * t->dims, tr, max_dist2, use_fma != 0, strict != 0);
            tr.emit(out_idx + static_cast<size_t>(i) * k, out_dist + static_cast<size_t>(i) * k);
        }
    });
    return 0;
}

void oracle_kd_free(void* tree) { delete static_cast<KdTree*>(tree); }

void* oracle_ball_build(const float* pts, uint32_t n, uint32_t dims, uint32_t skips, int use_fma) {
    if (n == 0 || dims == 0) return nullptr;
    auto* t = new BallTree();
    t->build(pts, n, dims, skips, use_fma != 0);
    return t;
}

int oracle_ball_knn(const void* tree, const float* q, uint32_t nq, float max_dist2, uint32_t k,
                    int heap, int use_fma, int strict, int32_t* out_idx, float* out_dist, int threads) {
    const auto* t = static_cast<const BallTree*>(tree);
    if (!t || k == 0) return 1;
    parallel_queries(nq, threads, [&](uint32_t lo, uint32_t hi) {
        Tracker tr(k, heap != 0);
        for (uint32_t i = lo; i < hi; ++i) {
            tr.reset(max_dist2);
            t->query(q + static_cast<size_t>(i) * t->dims, tr, max_dist2, use_fma != 0, strict != 0);
            tr.emit(out_idx + static_cast<size_t>(i) * k, out_dist + static_cast<size_t>(i) * k);
        }
    });
    return 0;
}

void oracle_ball_free(void* tree) { delete static_cast<BallTree*>(tree); }

// Tree shape figures used by tests: node depth, leaf slots and internal node count.
int oracle_tree_shape(uint32_t n, uint32_t skips, int ball, uint32_t* node_depth, uint32_t* leaf_slots,
                      uint32_t* node_count) {
    const uint32_t l2 = log2_ceil(n);
    uint32_t s = ball ? std::max(skips, 1u) : skips;
    s = std::min(s, l2 - 1);
    *node_depth = l2 - s;
    *leaf_slots = 1u << s;
    *node_count = (1u << (l2 - s)) - 1;
    return 0;
}

// Pairwise squared distance in either arithmetic mode (for the distance-precision tests).
float oracle_dist2(const float* a, const float* b, uint32_t dims, int use_fma) {
    return dist2(a, b, dims, use_fma != 0);
}

}  // extern "C"
