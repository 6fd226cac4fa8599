"""The seeded synthetic workloads have the shapes, sizes and value distributions of the benchmark
configurations they stand in for, and the same seed gives the same arrays (no GPU needed)."""

import math

import numpy as np
import pytest

from cudaexactknn_gb300 import workloads as W


def test_c1_uniform_brute_force():
    w = W.c1()
    assert (w.structure, w.k, w.heap, w.dims) == ("bf", 8, True, 3)
    assert w.points.shape == (65536, 3) and w.queries.shape == (4096, 3)
    assert w.points.dtype == np.float32 and w.queries.dtype == np.float32
    assert math.isinf(w.max_dist2)
    for a in (w.points, w.queries):
        assert a.min() >= 0.0 and a.max() < 1.0
        assert abs(float(a.mean()) - 0.5) < 0.01


def test_c2_mixture_kd_tree():
    w = W.c2()
    assert (w.structure, w.k, w.depth_skips) == ("kd", 16, 0)
    assert w.points.shape == (4194304, 3) and w.queries.shape == (1048576, 3)
    assert w.extra["train"].shape == (65536, 3)
    # 64 components, sigma 0.01: every point lies within a few sigma of one of 64 centres.  The
    # centres are recovered from the generator (same seed, same first draw).
    centres = np.random.Generator(np.random.PCG64(1002)).random((64, 3))
    assert centres.min() >= 0.0 and centres.max() < 1.0
    sample = w.points[:20000].astype(np.float64)
    d2 = ((sample[:, None, :] - centres[None, :, :]) ** 2).sum(-1).min(1)
    # Squared distance to the own centre / sigma^2 is chi-square with 3 degrees of freedom.
    assert np.sqrt(d2.max()) < 0.01 * 7
    assert abs(d2.mean() / 0.01 ** 2 - 3.0) < 0.15


def test_c3_subspace_ball_tree():
    w = W.c3()
    assert (w.structure, w.k, w.depth_skips, w.dims) == ("ball", 32, 1, 16)
    assert w.points.shape == (1048576, 16) and w.queries.shape == (262144, 16)
    rng = np.random.Generator(np.random.PCG64(1003))
    basis = W.orthonormal_basis(rng, 16, 4)
    assert np.allclose(basis.T @ basis, np.eye(4), atol=1e-12)
    x = w.points[:50000].astype(np.float64)
    resid = x - (x @ basis) @ basis.T
    # The noise outside the subspace is N(0, 0.05^2) in 12 directions; inside, latent N(0, 1).
    assert abs(np.sqrt((resid ** 2).sum(1).mean() / 12) - 0.05) < 0.001
    assert abs((x @ basis).std() - math.sqrt(1 + 0.05 ** 2)) < 0.02


def test_c4_gaussian_mixture_shapes_at_reduced_scale():
    w = W.c4(scale=1 / 64)
    assert (w.structure, w.k, w.dims) == ("bf", 100, 128)
    assert w.points.shape == (16384, 128) and w.queries.shape == (1024, 128)
    # Centres N(0, I) in 128 dims, sigma 0.3: per-coordinate spread sqrt(1 + 0.09).
    assert abs(float(w.points.std()) - math.sqrt(1.09)) < 0.05


def test_c5_uneven_sets():
    sets = W.c5_sets(scale=1 / 64)
    assert len(sets) == 64
    full = W.c5_sets.__defaults__  # (scale, count)
    assert full == (1.0, 64)
    for s in sets:
        assert s.dims in (3, 8, 32) and s.k in (1, 10, 64)
        assert s.structure == ("kd" if s.dims <= 8 else "ball")
        assert s.depth_skips == (0 if s.structure == "kd" else 1)
        n = s.points.shape[0]
        assert 16 <= n <= 1048576 // 64
        assert s.queries.shape[0] == max(n // 8, 1)
        assert s.points.min() >= 0.0 and s.points.max() < 1.0
    assert {s.dims for s in sets} == {3, 8, 32} and {s.k for s in sets} == {1, 10, 64}


@pytest.mark.parametrize("dims,structure,skips", [(6, "kd", 3), (16, "ball", 1), (17, "bf", 0)])
def test_range_limited_workload(dims, structure, skips):
    w = W.range_limited(scale=0.01, dims=dims, structure=structure)
    assert w.points.shape == (5000, dims) and w.queries.shape == (100, dims)
    assert w.k == 5 and w.depth_skips == skips
    assert w.max_dist2 == pytest.approx(0.01 * dims)
    with pytest.raises(ValueError):
        W.range_limited(dims=5)


def test_same_seed_same_arrays():
    a, b = W.c3(scale=1 / 256), W.c3(scale=1 / 256)
    assert np.array_equal(a.points, b.points) and np.array_equal(a.queries, b.queries)
    assert np.array_equal(a.extra["train"], b.extra["train"])
    assert not np.array_equal(a.queries[: len(a.extra["train"])], a.extra["train"][: len(a.queries)])
