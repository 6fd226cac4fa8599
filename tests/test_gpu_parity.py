"""Parity of the GPU engine with the oracle and with the reference's golden vectors.

Every comparison is exact: rows are compared as sorted u64 keys (bits(dist2) << 32 | index),
so indices, tie order and distance bits must all match.  The engine's distance is the
reference's sequential fused sum, i.e. the oracle's fma mode (tolerance: 0 ulp)."""

import math

import numpy as np
import pytest

import golden_io
import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu

gu = pytest.importorskip("gpu_util")

INF = float("inf")


def _oracle(points, queries, k, r2=INF):
    return oracle.bf_knn(points, queries, k, r2, fma=True, threads=8)


# ---- golden vectors (the reference's own CPU classes) -----------------------------------------

@pytest.mark.parametrize("name", golden_io.names())
def test_goldens(name):
    g = golden_io.load(name)
    pts, qs, k, r2 = g["points"], g["queries"], g["k"], g["max_dist2"]
    want = _oracle(pts, qs, k, r2)
    by_tag = {r["tag"]: r for r in g["runs"]}
    for run in g["runs"]:
        kind, skips = run["kind"], run["skips"]
        ix = gu.make_index(kind, pts, skips)
        got = gu.run(ix, qs, k, r2, heap=bool(run["heap"]))
        gu.assert_sorted_rows(*got)
        # Against brute force's canonical answer: exact.
        gu.assert_rows_equal(*got, *want, what=f"{name} {run['tag']} vs oracle")
        # Against the reference's own output: the contracted build where the compiler fused the
        # distance (it did if that build differs from the plain one), for brute force always,
        # for trees except at exact ties (where the reference's `>=` pruning is order-dependent).
        twin = by_tag[run["tag"][:-1] + "0"]
        fused = not np.array_equal(twin["dist"].view(np.uint32), run["dist"].view(np.uint32))
        if run["fma"] and fused and (kind == "bf" or not name.startswith("ties")):
            gu.assert_rows_equal(*got, run["idx"], run["dist"], what=f"{name} {run['tag']} vs reference")
        if not run["fma"]:
            # Plain-arithmetic reference: same indices where no near-tie, distances within 4 ulp.
            _, gd = oracle.split_keys(oracle.row_keys(*got))
            _, rd = oracle.split_keys(oracle.row_keys(run["idx"], run["dist"]))
            assert oracle.ulp_distance(gd, rd).max() <= 4
        ix.close()


# ---- the reference's correctness test, at its full shape ----------------------------------------

def test_functionality_shape_all_variants():
    """tests/FunctionalityTests.cu: D=4, N=100,000, Q=50,000, K=10, radius 5.9, the ten
    variants it asserts, checked here against brute force exactly (it checks index sets)."""
    w = W.functionality()
    qs = w.queries[:4096]
    want = _oracle(w.points, qs, w.k, w.max_dist2)
    bf = gu.make_index("bf", w.points)
    for heap, sh in ((False, False), (True, False), (False, True)):
        gu.assert_rows_equal(*gu.run(bf, qs, w.k, w.max_dist2, block_size=32, heap=heap, shmem_tracking=sh),
                             *want, what=f"bf heap={heap} sh={sh}")
    kd0 = gu.make_index("kd", w.points, 0)
    gu.assert_rows_equal(*gu.run(kd0, qs, w.k, w.max_dist2, block_size=32, heap=True, shmem_stack=True), *want,
                         what="kd skips0")
    kd3 = gu.make_index("kd", w.points, 3, aux_dims=3)
    gu.assert_rows_equal(*gu.run(kd3, qs, w.k, w.max_dist2, block_size=32, shmem_tracking=True), *want,
                         what="kd<4,3> skips3")
    b0 = gu.make_index("ball", w.points, 0)
    gu.assert_rows_equal(*gu.run(b0, qs, w.k, w.max_dist2, block_size=32, heap=True, shmem_tracking=True,
                                 shmem_stack=True), *want, what="ball skips0")
    b2 = gu.make_index("ball", w.points, 2)
    gu.assert_rows_equal(*gu.run(b2, qs, w.k, w.max_dist2, block_size=32), *want, what="ball skips2")


# ---- every tracker / stack storage variant and block size ----------------------------------------

@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
@pytest.mark.parametrize("heap", [False, True])
@pytest.mark.parametrize("shmem_tracking", [False, True])
@pytest.mark.parametrize("shmem_stack", [False, True])
def test_variants(structure, heap, shmem_tracking, shmem_stack):
    rng = np.random.default_rng(11)
    pts = W.uniform(rng, 20000, 5)
    qs = W.uniform(rng, 5000, 5)
    want = _oracle(pts, qs, 12)
    ix = gu.make_index(structure, pts, 2)
    for traversal in ((0, 1) if structure != "bf" else (0,)):
        for block in (32, 128, 256):
            got = gu.run(ix, qs, 12, block_size=block, heap=heap, shmem_tracking=shmem_tracking,
                         shmem_stack=shmem_stack, traversal=traversal)
            gu.assert_rows_equal(*got, *want, what=f"{structure} block={block} traversal={traversal}")


# ---- dimensions and k across every compiled class --------------------------------------------

@pytest.mark.parametrize("dims", [1, 2, 3, 4, 5, 7, 8, 9, 16, 17, 32, 33, 64, 100, 128])
@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_dims(structure, dims):
    rng = np.random.default_rng(dims)
    n = 3000 if dims <= 32 else 1500
    pts = W.uniform(rng, n, dims)
    qs = W.uniform(rng, 300, dims)
    k = 9
    want = _oracle(pts, qs, k)
    ix = gu.make_index(structure, pts, 1)
    gu.assert_rows_equal(*gu.run(ix, qs, k), *want, what=f"{structure} D={dims}")
    if structure != "bf":
        gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=1), *want, what=f"{structure} D={dims} warp")


@pytest.mark.parametrize("k", [1, 2, 7, 8, 9, 16, 17, 31, 32, 33, 64, 65, 100, 128])
@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_k(structure, k):
    rng = np.random.default_rng(k)
    pts = W.uniform(rng, 4000, 3)
    qs = W.uniform(rng, 500, 3)
    want = _oracle(pts, qs, k)
    ix = gu.make_index(structure, pts, 0)
    for heap in (False, True):
        gu.assert_rows_equal(*gu.run(ix, qs, k, heap=heap), *want, what=f"{structure} k={k} heap={heap}")


# ---- edge cases ------------------------------------------------------------------------------------

@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 8, 9, 31, 33, 1000, 1023, 1025])
def test_small_and_ragged_n(structure, n):
    rng = np.random.default_rng(n)
    pts = W.uniform(rng, n, 3)
    qs = W.uniform(rng, 64, 3)
    k = 8  # more than n for the smallest sets: unfilled slots are (-1, radius)
    for r2 in (INF, 0.05):
        want = _oracle(pts, qs, k, r2)
        for skips in (0, 1, 3, 40):
            ix = gu.make_index(structure, pts, skips)
            for traversal in (0, 1):
                gu.assert_rows_equal(*gu.run(ix, qs, k, r2, traversal=traversal), *want,
                                     what=f"{structure} n={n} skips={skips} r2={r2} traversal={traversal}")
            ix.close()


@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_empty_point_set(structure):
    import torch
    ix = gu.make_index(structure, np.zeros((0, 3), np.float32))
    idx, dist = gu.run(ix, np.random.default_rng(0).random((10, 3), dtype=np.float32), 4, 2.5)
    assert (idx == -1).all() and (dist == np.float32(2.5)).all()
    q = gu.to_dev(np.zeros((0, 3), np.float32))
    ix.knn(q, 4)  # zero queries: no-op
    del torch


@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_duplicates_and_exact_ties(structure):
    rng = np.random.default_rng(3)
    grid = (rng.integers(0, 6, size=(6000, 3)) / 6.0).astype(np.float32)
    qs = (rng.integers(0, 6, size=(700, 3)) / 6.0).astype(np.float32)
    qs[:300] += np.float32(1 / 12)
    for k in (1, 10, 40):
        want = _oracle(grid, qs, k)
        for skips in (0, 2):
            ix = gu.make_index(structure, grid, skips)
            for traversal in (0, 1):
                gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=traversal), *want,
                                     what=f"{structure} ties k={k} skips={skips} traversal={traversal}")


@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_radius_edge(structure):
    rng = np.random.default_rng(5)
    pts = W.uniform(rng, 3000, 4)
    qs = W.uniform(rng, 200, 4)
    ix = gu.make_index(structure, pts, 1)
    for r2 in (0.0, 1e-6, 0.02, 5.9):
        gu.assert_rows_equal(*gu.run(ix, qs, 10, r2), *_oracle(pts, qs, 10, r2), what=f"{structure} r2={r2}")
    # A radius equal to a point's exact distance keeps that point (ties with the slot init key).
    d2 = np.float32(oracle.dist2(qs[0], pts[17], fma=True))
    got = gu.run(ix, qs[:1], 3, float(d2))
    want = _oracle(pts, qs[:1], 3, float(d2))
    gu.assert_rows_equal(*got, *want, what="radius == distance")


@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_per_query_radii(structure):
    import torch
    rng = np.random.default_rng(9)
    pts = W.uniform(rng, 5000, 3)
    qs = W.uniform(rng, 6000, 3)
    radii = rng.uniform(0.0, 0.01, size=6000).astype(np.float32)
    ix = gu.make_index(structure, pts, 1)
    from cudaexactknn_gb300 import knn
    q = knn.Query(gu.to_dev(qs), 6000, 0.0)
    idx, dist = ix.batch_knn_radii(q, torch.from_numpy(radii).cuda(), k=6)
    idx, dist = idx.cpu().numpy(), dist.cpu().numpy()
    for lo in range(0, 6000, 1000):
        for i in range(lo, lo + 5):
            want = _oracle(pts, qs[i:i + 1], 6, float(radii[i]))
            gu.assert_rows_equal(idx[i:i + 1], dist[i:i + 1], *want, what=f"{structure} radii row {i}")


@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_host_buffers(structure):
    rng = np.random.default_rng(12)
    pts = W.uniform(rng, 8000, 3)
    qs = W.uniform(rng, 3000, 3)
    ix = gu.make_index(structure, pts, 0)
    idx, dist = ix.knn_host(qs, 7)
    gu.assert_rows_equal(idx.numpy(), dist.numpy(), *_oracle(pts, qs, 7), what=f"{structure} host")


def test_errors_are_raised_not_swallowed():
    from cudaexactknn_gb300 import KnnError, _lib
    rng = np.random.default_rng(1)
    ix = gu.make_index("kd", W.uniform(rng, 100, 3))
    q = gu.to_dev(W.uniform(rng, 4, 3))
    with pytest.raises(KnnError) as e:
        ix.knn(q, 0)
    assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    with pytest.raises(KnnError) as e:
        ix.knn(q, 129)
    assert e.value.status == _lib.ERR_UNSUPPORTED
    with pytest.raises(KnnError):
        ix.knn(q, 4, -1.0)
    with pytest.raises(KnnError):
        ix.knn(q, 4, math.nan)


def test_build_shape_matches_reference_rules():
    rng = np.random.default_rng(2)
    for n, skips, ball in ((100000, 3, False), (100000, 0, True), (1, 5, False), (4194304 // 64, 0, False)):
        ix = gu.make_index("ball" if ball else "kd", W.uniform(rng, n, 3), skips)
        info = ix.info()
        assert (info.node_depth, info.leaf_slots, info.node_count) == oracle.tree_shape(n, skips, ball)


# ---- autotuned plans -------------------------------------------------------------------------------

@pytest.mark.parametrize("structure,dims,k", [("kd", 3, 16), ("ball", 16, 32), ("bf", 8, 10)])
def test_autotune_is_exact_and_reports_its_plan(structure, dims, k):
    import ctypes
    from cudaexactknn_gb300 import _lib
    rng = np.random.default_rng(dims)
    pts = W.uniform(rng, 40000, dims)
    qs = W.uniform(rng, 9000, dims)
    ix = gu.make_index(structure, pts, 0 if structure == "kd" else 1)
    want = _oracle(pts, qs, k)
    gu.assert_rows_equal(*gu.run(ix, qs, k, flags=_lib.QF_AUTOTUNE), *want, what=f"{structure} autotune")
    o = _lib.QueryOpts()
    ms = ctypes.c_float()
    _lib.check(_lib.load().knn_tuned_plan(ix.handle, k, 0, ctypes.byref(o), ctypes.byref(ms)))
    assert o.block_size in (32, 64, 128, 256) and ms.value > 0
    assert o.reserved >= (3 if structure == "bf" else 10)
    # The tuned plan is reused on later calls and still exact.
    gu.assert_rows_equal(*gu.run(ix, qs, k, flags=_lib.QF_AUTOTUNE), *want, what=f"{structure} autotune again")


@pytest.mark.parametrize("leaf_scan", [2, 8, 32, 100000])
@pytest.mark.parametrize("structure", ["kd", "ball"])
def test_leaf_bucket_scan(structure, leaf_scan):
    rng = np.random.default_rng(leaf_scan)
    pts = W.uniform(rng, 5001, 4)
    qs = W.uniform(rng, 700, 4)
    want = _oracle(pts, qs, 9)
    ix = gu.make_index(structure, pts, 1)
    for traversal in (0, 1):
        gu.assert_rows_equal(*gu.run(ix, qs, 9, leaf_scan=leaf_scan, traversal=traversal), *want,
                             what=f"{structure} leaf_scan={leaf_scan} traversal={traversal}")


# ---- the reference's range-limited speed test shape (tests/DimXSpeedTests.cu:10-58) -------------

@pytest.mark.parametrize("dims", [6, 11, 17])
@pytest.mark.parametrize("structure", ["bf", "kd", "ball"])
def test_range_limited(structure, dims):
    """Uniform points, K=5, maxDistance2 = 0.01 D (many rows unfilled), kd depthSkips 3, ball 1;
    the plain form with the reference benchmark's template choices and the autotuned form."""
    from cudaexactknn_gb300 import _lib
    w = W.range_limited(0.04, dims, structure)
    want = _oracle(w.points, w.queries, w.k, w.max_dist2)
    ix = gu.make_index(structure, w.points, w.depth_skips)
    plain = {"kd": dict(block_size=32, shmem_stack=True),
             "ball": dict(block_size=16, heap=True, shmem_tracking=True, shmem_stack=True),
             "bf": dict(block_size=32)}[structure]
    for kw in (plain, dict(flags=_lib.QF_AUTOTUNE)):
        got = gu.run(ix, w.queries, w.k, w.max_dist2, **kw)
        gu.assert_rows_equal(*got, *want, what=f"range {structure}{dims} {kw}")
    ix.close()
