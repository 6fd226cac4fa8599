"""Learned search radius: gradients of the GPU kernels against a float64 NumPy oracle, and exact
answers (with fallbacks) when the model seeds the search."""

import numpy as np
import pytest

import oracle
import radius_model_ref as ref
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")


def _random_params(d, rng):
    e = d + 64
    n = 64 * e + 64 + 64 * 64 + 64 + 64 + 1
    p = np.zeros(n + 32 * d + 2 * d + 1, np.float32)
    p[:n] = rng.standard_normal(n).astype(np.float32) * 0.2
    p[n:n + 32 * d] = rng.standard_normal(32 * d) * 4.0            # projection B
    p[n + 32 * d:n + 33 * d] = -1.0 + 0.1 * rng.standard_normal(d)  # lo
    p[n + 33 * d:n + 34 * d] = 0.3 + 0.1 * rng.random(d)            # inv_range
    return p


@pytest.mark.parametrize("d", [3, 16, 32])
def test_gradients_match_float64_oracle(d):
    from cudaexactknn_gb300 import knn
    rng = np.random.default_rng(d)
    p = _random_params(d, rng)
    x = rng.standard_normal((257, d)).astype(np.float32)
    t = rng.standard_normal(257).astype(np.float32)
    loss, grad = knn.radius_model_gradients(p, d, x, t)
    want_loss, want_grad = ref.loss_and_grad(p, d, x, t)
    assert abs(loss - want_loss) <= 1e-4 * max(1.0, abs(want_loss))
    scale = np.abs(want_grad).max()
    np.testing.assert_allclose(grad, want_grad, rtol=2e-3, atol=1e-4 * scale)


def test_gradients_match_finite_differences():
    from cudaexactknn_gb300 import knn
    rng = np.random.default_rng(5)
    d = 3
    p = _random_params(d, rng).astype(np.float64)
    x = rng.standard_normal((64, d))
    t = rng.standard_normal(64)
    _, g = knn.radius_model_gradients(p, d, x, t)
    # Central differences of the float64 loss agree with the GPU gradient; the reference's own
    # analytic gradient agrees with both.
    _, g64 = ref.loss_and_grad(p, d, x, t)
    for i in rng.choice(len(g), size=25, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-4
        num = (ref.loss_and_grad(p + e, d, x, t)[0] - ref.loss_and_grad(p - e, d, x, t)[0]) / 2e-4
        assert abs(g64[i] - num) <= 1e-5 * max(1.0, abs(num)), i
        assert abs(g[i] - num) <= 2e-3 * max(1.0, abs(num)) + 1e-4 * np.abs(g64).max(), i


@pytest.mark.parametrize("structure,skips,d,k", [("kd", 0, 3, 16), ("ball", 1, 16, 32), ("bf", 0, 8, 10)])
def test_learned_radius_is_exact_and_falls_back(structure, skips, d, k):
    import torch
    from cudaexactknn_gb300 import _lib
    rng = np.random.default_rng(100 + d)
    if d == 16:
        pts, basis = W.subspace(rng, 60000, 16, 4, 0.05)
        qs, _ = W.subspace(rng, 8000, 16, 4, 0.05, basis)
        train, _ = W.subspace(rng, 8192, 16, 4, 0.05, basis)
    else:
        pts, centres = W.mixture(rng, 60000, d, 16, 0.02)
        qs, _ = W.mixture(rng, 8000, d, 16, 0.02, centres)
        train, _ = W.mixture(rng, 8192, d, 16, 0.02, centres)
    ix = gu.make_index(structure, pts, skips)
    rep = ix.train_radius_model(gu.to_dev(train), k, steps=400)
    assert rep.samples == 8192 and 0.9 <= rep.coverage <= 1.0
    # Predictions match the float64 model on the exported parameters.
    params = ix.export_radius_model()
    pred = ix.predict_log_kth(gu.to_dev(qs[:500])).cpu().numpy()
    np.testing.assert_allclose(pred, ref.predict(params, d, qs[:500]), rtol=1e-4, atol=1e-3)
    want = oracle.bf_knn(pts, qs, k, fma=True, threads=8)
    got = gu.run(ix, qs, k, flags=_lib.QF_LEARNED_RADIUS)
    gu.assert_rows_equal(*got, *want, what=f"{structure} learned radius")
    # Range-limited queries stay exact too (the seed never exceeds the caller's radius).
    r2 = float(np.quantile(want[1][:, -1], 0.5))
    got = gu.run(ix, qs, k, r2, flags=_lib.QF_LEARNED_RADIUS)
    gu.assert_rows_equal(*got, *oracle.bf_knn(pts, qs, k, r2, fma=True, threads=8), what="learned + radius")
    # A model with its margin forced very negative makes every query fall back: still exact.
    bad = params.copy()
    bad[-1] = -20.0
    ix.import_radius_model(bad, k)
    from cudaexactknn_gb300 import knn
    q = knn.Query(gu.to_dev(qs), len(qs), float("inf"))
    c = ix.stats(q, k, flags=_lib.QF_LEARNED_RADIUS)
    assert c.fallback_queries == len(qs)
    gu.assert_rows_equal(q.r_indexes.cpu().numpy(), q.r_distances.cpu().numpy(), *want, what="all fall back")


def test_untrained_index_refuses_learned_radius():
    from cudaexactknn_gb300 import KnnError, _lib
    rng = np.random.default_rng(0)
    ix = gu.make_index("kd", W.uniform(rng, 1000, 3))
    with pytest.raises(KnnError) as e:
        gu.run(ix, W.uniform(rng, 10, 3), 4, flags=_lib.QF_LEARNED_RADIUS)
    assert e.value.status == _lib.ERR_NOT_TRAINED


@pytest.mark.parametrize("structure,d,k", [("kd", 3, 16), ("ball", 16, 32)])
def test_learned_radius_gains_over_the_unseeded_search(structure, d, k):
    """What the trained network buys: the seeded search visits fewer tree nodes and points than
    the same search without a seed, and answers the same rows."""
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(7 + d)
    if d == 16:
        pts, basis = W.subspace(rng, 200000, 16, 4, 0.05)
        qs, _ = W.subspace(rng, 20000, 16, 4, 0.05, basis)
        train, _ = W.subspace(rng, 16384, 16, 4, 0.05, basis)
    else:
        pts, centres = W.mixture(rng, 400000, d, 64, 0.01)
        qs, _ = W.mixture(rng, 20000, d, 64, 0.01, centres)
        train, _ = W.mixture(rng, 16384, d, 64, 0.01, centres)
    ix = gu.make_index(structure, pts)
    ix.train_radius_model(gu.to_dev(train), k, steps=1500)
    q_plain = knn.Query(gu.to_dev(qs), len(qs), float("inf"))
    q_seed = knn.Query(gu.to_dev(qs), len(qs), float("inf"))
    plain = ix.stats(q_plain, k)
    seeded = ix.stats(q_seed, k, flags=_lib.QF_LEARNED_RADIUS)
    np.testing.assert_array_equal(q_plain.r_indexes.cpu().numpy(), q_seed.r_indexes.cpu().numpy())
    np.testing.assert_array_equal(q_plain.r_distances.cpu().numpy(), q_seed.r_distances.cpu().numpy())
    assert seeded.fallback_queries < len(qs) // 10
    print(f"{structure}: nodes {seeded.nodes_visited / plain.nodes_visited:.3f}, "
          f"points {seeded.points_scanned / plain.points_scanned:.3f} of the unseeded search, "
          f"fallback {seeded.fallback_queries} of {len(qs)}")
    assert seeded.nodes_visited < plain.nodes_visited, (seeded.nodes_visited, plain.nodes_visited)
    assert seeded.points_scanned < plain.points_scanned, (seeded.points_scanned, plain.points_scanned)
