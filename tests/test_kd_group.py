"""The k-d tree's warp-group search (traversal 2): a warp's 32 queries walk the tree once against
tight node boxes from per-query radii and share out their bucket scans; and the per-thread search
over the same boxes (traversal 3).  Every row must equal the
oracle's brute force exactly (sorted u64 keys), whether the radii come from each query's own
subtree or from the radius model, with a caller's radius, per-query radii, ties, duplicates that
overflow a query's candidate list, and point sets smaller than k."""

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")

INF = float("inf")


def _want(pts, qs, k, r2=INF):
    return oracle.bf_knn(pts, qs, k, r2, fma=True, threads=8)


@pytest.mark.parametrize("dims", [1, 2, 3, 4, 5, 8, 12, 16])
@pytest.mark.parametrize("skips", [0, 1, 3])
def test_group_self_seeded_dims(dims, skips):
    rng = np.random.default_rng(100 + dims * 7 + skips)
    pts = W.uniform(rng, 30000, dims)
    qs = W.uniform(rng, 5000, dims)
    ix = gu.make_index("kd", pts, skips)
    for k in (1, 8, 16, 32):
        want = _want(pts, qs, k)
        for leaf in (0, 4, 8, 32):
            got = gu.run(ix, qs, k, traversal=2, leaf_scan=leaf)
            gu.assert_sorted_rows(*got)
            gu.assert_rows_equal(*got, *want, what=f"D={dims} skips={skips} k={k} leaf={leaf}")
            gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=3, leaf_scan=leaf), *want,
                                 what=f"box D={dims} skips={skips} k={k} leaf={leaf}")
    for k in (33, 64, 128):  # the box search takes every k
        gu.assert_rows_equal(*gu.run(ix, qs[:500], k, traversal=3), *_want(pts, qs[:500], k), what=f"box D={dims} k={k}")
    ix.close()


@pytest.mark.parametrize("k", [1, 3, 9, 16, 17, 31, 32])
def test_group_mixture_and_radius(k):
    rng = np.random.default_rng(k)
    pts, centres = W.mixture(rng, 200000, 3, 64, 0.01)
    qs, _ = W.mixture(rng, 20000, 3, 64, 0.01, centres)
    ix = gu.make_index("kd", pts, 0)
    gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=2), *_want(pts, qs, k), what=f"mixture k={k}")
    r2 = 2e-5
    gu.assert_rows_equal(*gu.run(ix, qs, k, r2, traversal=2), *_want(pts, qs, k, r2), what=f"radius k={k}")
    gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=3), *_want(pts, qs, k), what=f"box k={k}")
    ix.close()


def test_group_per_query_radii_and_learned_seeds():
    import torch
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(3)
    pts, centres = W.mixture(rng, 300000, 3, 64, 0.01)
    qs, _ = W.mixture(rng, 30000, 3, 64, 0.01, centres)
    train, _ = W.mixture(rng, 16384, 3, 64, 0.01, centres)
    k = 16
    ix = gu.make_index("kd", pts, 0)
    ix.train_radius_model(gu.to_dev(train), k, steps=800)
    # Learned seeds, unbounded caller's radius.
    got = gu.run(ix, qs, k, traversal=2, flags=_lib.QF_LEARNED_RADIUS)
    gu.assert_rows_equal(*got, *_want(pts, qs, k), what="learned seeds")
    # Per-query caller's radii: some below the k-th distance (unfilled slots), some above.
    radii = rng.uniform(0.0, 3e-5, size=len(qs)).astype(np.float32)
    q = knn.Query(gu.to_dev(qs), len(qs), INF)
    for flags in (0, _lib.QF_LEARNED_RADIUS):
        idx, dist = ix.batch_knn_radii(q, torch.from_numpy(radii).cuda(), k, traversal=2, flags=flags)
        want_rows = [_want(pts, qs[i:i + 1], k, float(radii[i])) for i in range(0, len(qs), 97)]
        got_i, got_d = idx.cpu().numpy(), dist.cpu().numpy()
        for j, i in enumerate(range(0, len(qs), 97)):
            gu.assert_rows_equal(got_i[i:i + 1], got_d[i:i + 1], *want_rows[j], what=f"radii flags={flags} row {i}")
    ix.close()


def test_group_ties_and_overflowing_duplicates():
    """Grid points (many equal distances) and 300 copies of a few points: a query at a copy has
    more than a candidate list of points at distance 0, so it goes to the per-thread fallback."""
    from cudaexactknn_gb300 import _lib, knn
    g = np.stack(np.meshgrid(*[np.arange(24, dtype=np.float32)] * 3, indexing="ij"), -1).reshape(-1, 3) / 24
    dup = np.repeat(g[[5, 777, 4000]], 300, axis=0)
    pts = np.concatenate([g, dup]).astype(np.float32)
    rng = np.random.default_rng(1)
    qs = np.concatenate([g[rng.choice(len(g), 2000)], dup[::50], (g[:500] + 0.5 / 24)]).astype(np.float32)
    ix = gu.make_index("kd", pts, 0)
    for k in (1, 6, 16, 32):
        want = _want(pts, qs, k)
        gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=2), *want, what=f"ties k={k}")
        gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=3), *want, what=f"box ties k={k}")
    st = ix.stats(knn.Query(gu.to_dev(qs), len(qs), INF), 16, traversal=2)
    assert st.fallback_queries >= len(dup[::50]), st.fallback_queries
    ix.close()


@pytest.mark.parametrize("n", [1, 2, 5, 16, 31, 40, 200])
def test_group_small_sets(n):
    rng = np.random.default_rng(n)
    pts = W.uniform(rng, n, 3)
    qs = W.uniform(rng, 300, 3)
    ix = gu.make_index("kd", pts, 0)
    for k in (1, 16, 32):
        gu.assert_rows_equal(*gu.run(ix, qs, k, traversal=2), *_want(pts, qs, k), what=f"n={n} k={k}")
        gu.assert_rows_equal(*gu.run(ix, qs, k, 0.01, traversal=2), *_want(pts, qs, k, 0.01),
                             what=f"n={n} k={k} r2=0.01")
        gu.assert_rows_equal(*gu.run(ix, qs, k, 0.01, traversal=3), *_want(pts, qs, k, 0.01),
                             what=f"box n={n} k={k} r2=0.01")
    ix.close()


def test_group_autotuned_learned_pass_is_exact_and_reports_its_plan():
    import ctypes
    from cudaexactknn_gb300 import _lib
    rng = np.random.default_rng(12)
    pts, centres = W.mixture(rng, 500000, 3, 64, 0.01)
    qs, _ = W.mixture(rng, 100000, 3, 64, 0.01, centres)
    train, _ = W.mixture(rng, 16384, 3, 64, 0.01, centres)
    ix = gu.make_index("kd", pts, 0)
    ix.train_radius_model(gu.to_dev(train), 16, steps=800)
    got = gu.run(ix, qs, 16, flags=_lib.QF_AUTOTUNE | _lib.QF_LEARNED_RADIUS)
    plain = gu.run(ix, qs, 16)
    np.testing.assert_array_equal(got[0], plain[0])
    np.testing.assert_array_equal(got[1].view(np.uint32), plain[1].view(np.uint32))
    rows = np.arange(0, len(qs), 211)
    gu.assert_rows_equal(got[0][rows], got[1][rows], *_want(pts, qs[rows], 16), what="autotuned sample")
    o = _lib.QueryOpts()
    ms = ctypes.c_float()
    _lib.check(_lib.load().knn_tuned_plan(ix.handle, 16, 1, ctypes.byref(o), ctypes.byref(ms)))
    assert o.traversal in (0, 1, 2)
    ix.close()
