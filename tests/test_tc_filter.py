"""Queries through the 16-bit tensor-core filter (tcgen05: FP16 with power-of-two scaling, or
BF16 for wide data), cell-ordered tiles with ball-bound tile skipping, and exact FP32 rescoring.

The filter is only a filter: every returned row must equal the plain brute force's exactly
(same keys: indices, tie order and distance bits), whatever the index, data, k or radius."""

import ctypes

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")


def _flags():
    from cudaexactknn_gb300 import _lib
    return _lib.QF_BF16_FILTER


def _codes():
    """The running k-th bound as buffered codes also where the heap fits."""
    from cudaexactknn_gb300 import _lib
    return _lib.QF_FILTER_CODES


@pytest.mark.parametrize("dims", [3, 9, 16, 17, 24, 32, 40, 64, 100, 128])
def test_tensor_core_selftest(dims):
    """tcgen05.mma over one 128x256 tile matches exact products of the FP16 and BF16 inputs, in
    each operand layout: 32-byte rows (dims <= 16), 64-byte rows (<= 32), 128-byte rows (one or
    two blocks of 64)."""
    from cudaexactknn_gb300 import _lib
    err = ctypes.c_float()
    bad = ctypes.c_uint32()
    _lib.check(_lib.load().knn_tc_selftest(dims, ctypes.byref(err), ctypes.byref(bad)))
    assert bad.value == 0, (bad.value, err.value)
    assert err.value <= dims * 2.0 ** -20


@pytest.mark.parametrize("dims", [16, 17, 32, 64, 100, 128])
@pytest.mark.parametrize("k", [1, 10, 100, 128])
def test_filter_exact(dims, k):
    """Both forms of the running k-th bound: buffered codes, and the heap where it fits."""
    rng = np.random.default_rng(dims * 1000 + k)
    pts, centres = W.gauss_mix(rng, 6000, dims, 24, 0.3)
    qs, _ = W.gauss_mix(rng, 300, dims, 24, 0.3, centres)
    ix = gu.make_index("bf", pts)
    want = oracle.bf_knn(pts, qs, k, fma=True, threads=8)
    for codes in (0, _codes()):
        gu.assert_rows_equal(*gu.run(ix, qs, k, flags=_flags() | codes), *want,
                             what=f"bf16 filter D={dims} k={k} codes={codes}")


@pytest.mark.parametrize("n,nq", [(1, 5), (255, 129), (257, 127), (1025, 1), (3000, 1000)])
def test_filter_ragged_sizes(n, nq):
    rng = np.random.default_rng(n)
    pts = W.uniform(rng, n, 24)
    qs = W.uniform(rng, nq, 24)
    ix = gu.make_index("bf", pts)
    for r2 in (float("inf"), 2.0):
        want = oracle.bf_knn(pts, qs, 16, r2, fma=True, threads=8)
        gu.assert_rows_equal(*gu.run(ix, qs, 16, r2, flags=_flags()), *want, what=f"n={n} nq={nq} r2={r2}")


def test_filter_ties_and_duplicates():
    rng = np.random.default_rng(3)
    grid = (rng.integers(0, 3, size=(4000, 16)) / 2.0).astype(np.float32)
    qs = np.concatenate([grid[:100], (rng.integers(0, 3, size=(100, 16)) / 2.0).astype(np.float32)])
    ix = gu.make_index("bf", grid)
    for k in (1, 32, 128):
        want = oracle.bf_knn(grid, qs, k, fma=True, threads=8)
        for codes in (0, _codes()):
            gu.assert_rows_equal(*gu.run(ix, qs, k, flags=_flags() | codes), *want, what=f"grid ties k={k} codes={codes}")


def test_bound_buffer_flushes_on_wide_data():
    """128 dims, k = 128: the filter (not the plain search) answers, and the buffered k-th bounds
    are flushed many times per query tile (dense home tiles, then sparse kept cells), with every
    row exact."""
    from cudaexactknn_gb300 import knn
    rng = np.random.default_rng(21)
    pts, centres = W.gauss_mix(rng, 20000, 128, 32, 0.2)
    qs, _ = W.gauss_mix(rng, 640, 128, 32, 0.2, centres)
    ix = gu.make_index("bf", pts)
    for k in (100, 128):
        want = oracle.bf_knn(pts, qs, k, fma=True, threads=8)
        gu.assert_rows_equal(*gu.run(ix, qs, k, flags=_flags()), *want, what=f"D=128 k={k}")
        c = ix.stats(knn.Query(gu.to_dev(qs), len(qs), float("inf")), k, flags=_flags())
        assert c.leaves_visited > 0 and c.fallback_queries <= len(qs) // 100, (k, c.leaves_visited, c.fallback_queries)


@pytest.mark.parametrize("n", [300, 256 * 8 + 44])
def test_infinite_seed_bounds(n):
    """A query whose cell holds fewer than k points starts with an infinite bound: every column
    is a candidate and its first flush takes the largest buffered value (tree layout, 24 dims: the
    cells are 256-point tiles and the last one is partial; the queries are the points themselves,
    so some descend to that cell)."""
    rng = np.random.default_rng(n)
    pts = W.uniform(rng, n, 24)
    ix = gu.make_index("bf", pts)
    for k in (100, 128):
        want = oracle.bf_knn(pts, pts, k, fma=True, threads=8)
        for codes in (0, _codes()):
            gu.assert_rows_equal(*gu.run(ix, pts, k, flags=_flags() | codes), *want, what=f"n={n} k={k} codes={codes}")


def test_candidate_overflow_falls_back_exactly():
    rng = np.random.default_rng(4)
    pts = W.uniform(rng, 5000, 32)
    qs = W.uniform(rng, 700, 32)
    ix = gu.make_index("bf", pts)
    want = oracle.bf_knn(pts, qs, 20, fma=True, threads=8)
    # A candidate capacity below k forces every query through the plain path.
    gu.assert_rows_equal(*gu.run(ix, qs, 20, flags=_flags(), tc_cap=8), *want, what="cap 8")
    gu.assert_rows_equal(*gu.run(ix, qs, 20, flags=_flags(), tc_cap=64), *want, what="cap 64")


def test_filter_with_learned_radius():
    from cudaexactknn_gb300 import _lib
    rng = np.random.default_rng(6)
    pts, centres = W.gauss_mix(rng, 20000, 64, 32, 0.3)
    qs, _ = W.gauss_mix(rng, 1500, 64, 32, 0.3, centres)
    train, _ = W.gauss_mix(rng, 4096, 64, 32, 0.3, centres)
    ix = gu.make_index("bf", pts)
    ix.train_radius_model(gu.to_dev(train), 50, steps=300)
    want = oracle.bf_knn(pts, qs, 50, fma=True, threads=8)
    got = gu.run(ix, qs, 50, flags=_flags() | _lib.QF_LEARNED_RADIUS)
    gu.assert_rows_equal(*got, *want, what="bf16 filter + learned radius")


@pytest.mark.parametrize("structure,dims,k", [("kd", 16, 8), ("kd", 20, 32), ("ball", 16, 32), ("ball", 32, 10),
                                              ("ball", 100, 64)])
def test_filter_on_trees(structure, dims, k):
    """Trees answer through the same filter (their leaf slots are the point set)."""
    rng = np.random.default_rng(dims * 7 + k)
    pts, basis = W.subspace(rng, 30000, dims, 4, 0.05)
    qs, _ = W.subspace(rng, 2000, dims, 4, 0.05, basis)
    ix = gu.make_index(structure, pts)
    for r2 in (float("inf"), 0.5):
        want = oracle.bf_knn(pts, qs, k, r2, fma=True, threads=8)
        for codes in (0, _codes()):
            gu.assert_rows_equal(*gu.run(ix, qs, k, r2, flags=_flags() | codes), *want,
                                 what=f"{structure} D={dims} k={k} r2={r2} codes={codes}")


def test_clustered_data_skips_tiles():
    """Well separated clusters: most point tiles are skipped, answers stay exact."""
    from cudaexactknn_gb300 import knn
    rng = np.random.default_rng(11)
    pts, centres = W.gauss_mix(rng, 60000, 64, 64, 0.1)
    qs, _ = W.gauss_mix(rng, 2048, 64, 64, 0.1, centres)
    ix = gu.make_index("bf", pts)
    want = oracle.bf_knn(pts, qs, 20, fma=True, threads=8)
    gu.assert_rows_equal(*gu.run(ix, qs, 20, flags=_flags()), *want, what="clustered")
    c = ix.stats(knn.Query(gu.to_dev(qs), len(qs), float("inf")), 20, flags=_flags())
    full_scan = (len(qs) // 128) * (60000 // 256)  # point tiles a brute-force pass would scan
    assert 0 < c.leaves_visited < full_scan // 4, (c.leaves_visited, full_scan)
    assert c.fallback_queries == 0
    assert c.nodes_visited >= len(qs) * 20  # candidates rescored


@pytest.mark.parametrize("scale", [1e-20, 1e-3, 1e5, 1e30])
def test_filter_magnitudes(scale):
    """Tiny data (large FP16 scale), huge data (BF16 format): exact either way."""
    rng = np.random.default_rng(12)
    pts, centres = W.gauss_mix(rng, 5000, 24, 16, 0.3)
    qs, _ = W.gauss_mix(rng, 400, 24, 16, 0.3, centres)
    pts = (pts * np.float32(scale)).astype(np.float32)
    qs = (qs * np.float32(scale)).astype(np.float32)
    ix = gu.make_index("bf", pts)
    want = oracle.bf_knn(pts, qs, 12, fma=True, threads=8)
    gu.assert_rows_equal(*gu.run(ix, qs, 12, flags=_flags()), *want, what=f"scale {scale}")


def test_queries_outside_the_format_fall_back():
    """Queries whose scaled coordinates overflow FP16 take the plain search, exactly."""
    from cudaexactknn_gb300 import knn
    rng = np.random.default_rng(13)
    pts = W.uniform(rng, 4000, 32)
    qs = W.uniform(rng, 300, 32)
    qs[::7] *= np.float32(1e6)
    ix = gu.make_index("bf", pts)
    want = oracle.bf_knn(pts, qs, 10, fma=True, threads=8)
    gu.assert_rows_equal(*gu.run(ix, qs, 10, flags=_flags()), *want, what="fp16 overflow queries")
    c = ix.stats(knn.Query(gu.to_dev(qs), len(qs), float("inf")), 10, flags=_flags())
    assert c.fallback_queries == len(range(0, 300, 7))


@pytest.mark.parametrize("structure,dims,k,nq", [("bf", 128, 100, 24000), ("ball", 16, 32, 48000), ("bf", 64, 10, 48000)])
def test_persistent_blocks_take_several_query_tiles(structure, dims, k, nq):
    """More 128-query tiles than resident filter blocks (one per SM with two accumulators, two with
    one), so blocks take further tiles from the counter; a sample of rows against the oracle."""
    rng = np.random.default_rng(dims + k)
    if structure == "ball":
        pts, basis = W.subspace(rng, 20000, dims, 4, 0.05)
        qs, _ = W.subspace(rng, nq, dims, 4, 0.05, basis)
    else:
        pts, centres = W.gauss_mix(rng, 20000, dims, 32, 0.3)
        qs, _ = W.gauss_mix(rng, nq, dims, 32, 0.3, centres)
    ix = gu.make_index(structure, pts, 1 if structure == "ball" else None)
    rows = np.random.default_rng(1).choice(nq, size=1500, replace=False)
    want = oracle.bf_knn(pts, qs[rows], k, fma=True, threads=8)
    for codes in (0, _codes()):
        idx, dist = gu.run(ix, qs, k, flags=_flags() | codes)
        gu.assert_rows_equal(idx[rows], dist[rows], *want, what=f"{structure} D={dims} k={k} nq={nq} codes={codes}")
    ix.close()


@pytest.mark.parametrize("structure,dims,k,nq", [("bf", 32, 10, 700), ("bf", 128, 100, 40000), ("ball", 16, 32, 3000)])
def test_filter_blocks_that_give_up_leave_exact_answers(structure, dims, k, nq):
    """Every filter block gives up right after its first point-tile copy, as when one of its
    bounded waits runs out (test flag): it drains the copies and MMAs it issued, frees its tensor
    memory and flags the error, and the call still returns.  The give-ups are counted, every query
    goes to the exhaustive search, and every row equals the oracle's."""
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(dims * 7 + k)
    if structure == "ball":
        pts, basis = W.subspace(rng, 20000, dims, 4, 0.05)
        qs, _ = W.subspace(rng, nq, dims, 4, 0.05, basis)
    else:
        pts, centres = W.gauss_mix(rng, 20000, dims, 32, 0.3)
        qs, _ = W.gauss_mix(rng, nq, dims, 32, 0.3, centres)
    ix = gu.make_index(structure, pts, 1 if structure == "ball" else None)
    flags = _flags() | _lib.QF_TEST_FILTER_GIVE_UP
    q = knn.Query(gu.to_dev(qs), len(qs), float("inf"))
    c = ix.stats(q, k, flags=flags)
    assert c.filter_give_ups >= 1
    assert c.fallback_queries == nq, (c.fallback_queries, nq)
    idx, dist = q.r_indexes.cpu().numpy(), q.r_distances.cpu().numpy()
    rows = np.arange(nq) if nq <= 3000 else np.random.default_rng(2).choice(nq, size=1000, replace=False)
    want = oracle.bf_knn(pts, qs[rows], k, fma=True, threads=8)
    gu.assert_rows_equal(idx[rows], dist[rows], *want, what=f"give-up {structure} D={dims} k={k}")
    # The same index answers normally afterwards (nothing left behind by the blocks that gave up).
    c2 = ix.stats(q, k, flags=_flags())
    assert c2.filter_give_ups == 0
    gu.assert_rows_equal(q.r_indexes.cpu().numpy()[rows], q.r_distances.cpu().numpy()[rows], *want,
                         what=f"after give-up {structure} D={dims} k={k}")
    ix.close()
