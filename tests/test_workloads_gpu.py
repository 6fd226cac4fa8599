"""The benchmark workloads at their full sizes, checked through properties that hold at any size.

The oracle cannot answer a million queries against four million points in test time, so at full
size each workload is checked by:
  * the chosen form (autotuned plan, learned radius where the workload has a training sample)
    equals the plain form bit for bit on every row, two searches that share no pruning scheme;
  * every row is in ascending (distance, index) order, every slot filled (k <= n, unbounded
    radius) with an index in [0, n);
  * a second chosen pass returns the same rows (nothing carries over between passes);
  * a seeded sample of rows equals the oracle's brute force exactly."""

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")

SAMPLE_ROWS = 256


def _sorted_and_filled(idx, dist, n):
    import torch
    d0, d1 = dist[:, :-1], dist[:, 1:]
    i0, i1 = idx[:, :-1], idx[:, 1:]
    ascending = (d1 > d0) | ((d1 == d0) & (i1 > i0))
    assert bool(ascending.all()), "rows must be in ascending key order"
    assert bool(((idx >= 0) & (idx < n)).all()), "every slot must hold a point index"
    assert bool(torch.isfinite(dist).all())


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "c4"])
def test_full_size_workload(name):
    import torch
    from cudaexactknn_gb300 import _lib
    w = W.CONFIGS[name]()
    n, k = w.points.shape[0], w.k
    ix = gu.make_index(w.structure, w.points, w.depth_skips)
    qs = gu.to_dev(w.queries)
    flags = _lib.QF_AUTOTUNE
    if "train" in w.extra:
        rep = ix.train_radius_model(gu.to_dev(w.extra["train"]), k, steps=1000)
        assert 0.9 <= rep.coverage <= 1.0
        flags |= _lib.QF_LEARNED_RADIUS
    plain_i, plain_d = ix.knn(qs, k, heap=w.heap)
    chosen_i, chosen_d = ix.knn(qs, k, flags=flags)
    torch.cuda.synchronize()
    _sorted_and_filled(plain_i, plain_d, n)
    assert torch.equal(chosen_i, plain_i), f"{name}: chosen and plain indices differ"
    assert torch.equal(chosen_d.view(torch.int32), plain_d.view(torch.int32)), f"{name}: distances differ"
    again_i, again_d = ix.knn(qs, k, flags=flags)
    assert torch.equal(again_i, chosen_i) and torch.equal(again_d.view(torch.int32), chosen_d.view(torch.int32))
    rows = np.sort(np.random.default_rng(5).choice(len(w.queries), size=SAMPLE_ROWS, replace=False))
    want = oracle.bf_knn(w.points, w.queries[rows], k, w.max_dist2, fma=True, threads=16)
    sel = torch.from_numpy(rows).to(chosen_i.device)
    gu.assert_rows_equal(chosen_i[sel].cpu().numpy(), chosen_d[sel].cpu().numpy(), *want, what=f"{name} sample")
    ix.close()


def _same_rows(a_i, a_d, b_i, b_d, what):
    import torch
    assert torch.equal(a_i, b_i), f"{what}: indices differ"
    assert torch.equal(a_d.view(torch.int32), b_d.view(torch.int32)), f"{what}: distances differ"


def test_c5_uneven_batch_full_size():
    """The 64 uneven sets of the batch workload at full size, in one autotuned graph launch: every
    row of every set equals one plain knn call on that set, a second run repeats the first, and a
    seeded sample of each set's rows equals the oracle's brute force."""
    import torch
    from cudaexactknn_gb300 import knn
    sets = W.c5_sets()
    built = [(gu.make_index(w.structure, w.points, w.depth_skips), w) for w in sets]
    batch = knn.Batch([(ix, gu.to_dev(w.queries), w.k, w.max_dist2) for ix, w in built], autotune=True)
    res = [(i.clone(), d.clone()) for i, d in batch.run()]
    again = batch.run()
    rng = np.random.default_rng(55)
    for j, ((ix, w), (oi, od)) in enumerate(zip(built, res)):
        _same_rows(oi, od, *again[j], f"set {j} second run")
        pi, pd = ix.knn(gu.to_dev(w.queries), w.k, w.max_dist2)
        torch.cuda.synchronize()
        _same_rows(oi, od, pi, pd, f"set {j} ({w.name}) batch vs plain")
        rows = np.sort(rng.choice(len(w.queries), size=min(16, len(w.queries)), replace=False))
        want = oracle.bf_knn(w.points, w.queries[rows], w.k, w.max_dist2, fma=True, threads=16)
        sel = torch.from_numpy(rows).to(oi.device)
        gu.assert_rows_equal(oi[sel].cpu().numpy(), od[sel].cpu().numpy(), *want, what=f"set {j} oracle sample")
    batch.close()
    for ix, _ in built:
        ix.close()


@pytest.mark.parametrize("structure", ["kd", "ball", "bf"])
def test_range_limited_full_size(structure):
    """The reference's range-limited workload (tests/DimXSpeedTests.cu) at full size, D = 16:
    N = 500,000, Q = 10,000, K = 5, maxDistance2 = 0.16.  The autotuned form equals the plain form
    (the reference benchmarks' template choices) on every row; most rows are partly unfilled, and
    unfilled slots hold (-1, maxDistance2); a sample equals the oracle."""
    import torch
    from cudaexactknn_gb300 import _lib
    w = W.range_limited(1.0, 16, structure)
    ix = gu.make_index(structure, w.points, w.depth_skips)
    qs = gu.to_dev(w.queries)
    plain_kw = {"kd": dict(block_size=32, shmem_stack=True),
                "ball": dict(block_size=16, heap=True, shmem_tracking=True, shmem_stack=True),
                "bf": dict(block_size=32)}[structure]
    pi, pd = ix.knn(qs, w.k, w.max_dist2, **plain_kw)
    ci, cd = ix.knn(qs, w.k, w.max_dist2, flags=_lib.QF_AUTOTUNE)
    torch.cuda.synchronize()
    _same_rows(ci, cd, pi, pd, f"range {structure}")
    unfilled = ci < 0
    assert bool(unfilled.any()), "the range-limited workload leaves slots unfilled"
    assert bool((cd[unfilled] == float(np.float32(w.max_dist2))).all())
    rows = np.sort(np.random.default_rng(6).choice(len(w.queries), size=SAMPLE_ROWS, replace=False))
    want = oracle.bf_knn(w.points, w.queries[rows], w.k, w.max_dist2, fma=True, threads=16)
    sel = torch.from_numpy(rows).to(ci.device)
    gu.assert_rows_equal(ci[sel].cpu().numpy(), cd[sel].cpu().numpy(), *want, what=f"range {structure} sample")
    ix.close()
