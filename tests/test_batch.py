"""Batches of independent sets (uneven n, dims, k) in one graph launch: every item's rows must
equal its own brute force, with and without autotuning and the locality sort, run after run."""

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")

# (n, dims, k, structure, max_distance2)
SPECS = [(1024, 3, 1, "kd", np.inf), (5000, 3, 10, "kd", np.inf), (70000, 3, 64, "kd", np.inf),
         (3000, 8, 10, "kd", 0.05), (20000, 8, 1, "kd", np.inf), (2048, 32, 64, "ball", np.inf),
         (9000, 32, 10, "ball", np.inf), (40000, 32, 1, "ball", np.inf), (1500, 3, 10, "kd", np.inf),
         (777, 5, 13, "ball", 0.3)]


def _sets(seed, specs):
    rng = np.random.default_rng(seed)
    out = []
    for n, d, k, structure, r2 in specs:
        pts = W.uniform(rng, n, d)
        qs = W.uniform(rng, max(1, n // 8 + 37), d)
        out.append((gu.make_index(structure, pts), pts, qs, k, float(r2)))
    return out


@pytest.mark.parametrize("mode", ["plain", "autotune", "keep_order"])
def test_batch_exact(mode):
    from cudaexactknn_gb300 import knn
    sets = _sets(5, SPECS)
    b = knn.Batch([(ix, gu.to_dev(qs), k, r2) for ix, _, qs, k, r2 in sets],
                  autotune=mode == "autotune", keep_order=mode == "keep_order")
    classes, kernels = b.info()
    # k classes: (kd,3,<=8) (kd,3,<=16: two sets) (kd,3,<=64) (kd,8,<=16) (kd,8,<=8) (ball,5,<=16) (ball,32) x 3
    assert classes == 9
    assert kernels >= classes if mode == "keep_order" else kernels >= 3 * classes
    for run in range(2):
        for _, _, oi, od in b.items:
            oi.fill_(7)
            od.fill_(-1.0)
        res = b.run()
        for (ix, pts, qs, k, r2), (oi, od) in zip(sets, res):
            want = oracle.bf_knn(pts, qs, k, r2, fma=True)
            gu.assert_rows_equal(oi.cpu().numpy(), od.cpu().numpy(), *want,
                                 what=f"{mode} run {run} n={len(pts)} d={pts.shape[1]} k={k}")
    b.close()


def test_batch_matches_single_queries():
    """The batch answers exactly what a knn call per set answers."""
    from cudaexactknn_gb300 import knn
    sets = _sets(9, [(30000, 3, 16, "kd", np.inf), (100, 3, 16, "kd", np.inf), (5000, 16, 8, "ball", np.inf)])
    res = knn.Batch([(ix, gu.to_dev(qs), k, r2) for ix, _, qs, k, r2 in sets]).run()
    for (ix, pts, qs, k, r2), (oi, od) in zip(sets, res):
        gi, gd = gu.run(ix, qs, k, r2)
        np.testing.assert_array_equal(oi.cpu().numpy(), gi)
        np.testing.assert_array_equal(od.cpu().numpy(), gd)


def test_batch_errors_and_empty():
    import torch
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(1)
    kd = gu.make_index("kd", W.uniform(rng, 1000, 3))
    bf = gu.make_index("bf", W.uniform(rng, 100, 3))
    q = gu.to_dev(W.uniform(rng, 50, 3))
    with pytest.raises(_lib.KnnError) as e:
        knn.Batch([(kd, q, 0, np.inf)])
    assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    with pytest.raises(_lib.KnnError) as e:
        knn.Batch([(bf, q, 4, np.inf)])
    assert e.value.status == _lib.ERR_UNSUPPORTED
    with pytest.raises(_lib.KnnError) as e:
        knn.Batch([(kd, q, 4, -1.0)])
    assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    # zero-query items and an empty batch run as no-ops
    b = knn.Batch([(kd, torch.empty((0, 3), device="cuda"), 4, np.inf)])
    assert b.info() == (0, 0)
    b.run()
    assert knn.Batch([]).info() == (0, 0)
