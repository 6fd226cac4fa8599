"""Streams and host buffers: different indexes on different non-default streams run at the same
time, queries on one index from two streams are ordered on the device (they share its scratch),
and knn_query_host (result rows copied out in pieces on several streams) returns what the
device-buffer call returns."""

import numpy as np
import pytest

import oracle
from cudaexactknn_gb300 import workloads as W

pytestmark = pytest.mark.gpu
gu = pytest.importorskip("gpu_util")

INF = float("inf")


def test_two_indexes_on_two_streams_at_once():
    import torch
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(21)
    p1, c1 = W.mixture(rng, 200000, 3, 64, 0.01)
    q1, _ = W.mixture(rng, 50000, 3, 64, 0.01, c1)
    p2, b2 = W.subspace(rng, 60000, 16, 4, 0.05)
    q2, _ = W.subspace(rng, 8000, 16, 4, 0.05, b2)
    kd = gu.make_index("kd", p1, 0)
    ball = gu.make_index("ball", p2, 1)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    a = knn.Query(gu.to_dev(q1), len(q1), INF)
    b = knn.Query(gu.to_dev(q2), len(q2), INF)
    torch.cuda.synchronize()
    for _ in range(3):
        for t in (a.r_indexes, b.r_indexes):
            if t is not None:
                t.fill_(7)
        kd.batch_knn(a, 16, traversal=2, sync=False, stream=s1)
        ball.batch_knn(b, 32, flags=_lib.QF_BF16_FILTER, sync=False, stream=s2)
        torch.cuda.synchronize()
        rows1 = np.arange(0, len(q1), 37)
        gu.assert_rows_equal(a.r_indexes.cpu().numpy()[rows1], a.r_distances.cpu().numpy()[rows1],
                             *oracle.bf_knn(p1, q1[rows1], 16, fma=True, threads=8), what="kd on stream 1")
        rows2 = np.arange(0, len(q2), 7)
        gu.assert_rows_equal(b.r_indexes.cpu().numpy()[rows2], b.r_distances.cpu().numpy()[rows2],
                             *oracle.bf_knn(p2, q2[rows2], 32, fma=True, threads=8), what="ball on stream 2")
    kd.close()
    ball.close()


@pytest.mark.parametrize("structure", ["kd", "ball", "bf"])
def test_one_index_from_two_streams(structure):
    """Two batches on one index, issued back to back on two streams without a host wait: the
    second waits on the device for the first (shared workspace), and both are exact."""
    import torch
    from cudaexactknn_gb300 import _lib, knn
    rng = np.random.default_rng(5)
    pts = W.uniform(rng, 100000, 8)
    qa = W.uniform(rng, 30000, 8)
    qb = W.uniform(rng, 20000, 8)
    ix = gu.make_index(structure, pts)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    a = knn.Query(gu.to_dev(qa), len(qa), INF)
    b = knn.Query(gu.to_dev(qb), len(qb), INF)
    torch.cuda.synchronize()
    for rep in range(3):
        ix.batch_knn(a, 10, flags=_lib.QF_AUTOTUNE, sync=False, stream=s1)
        ix.batch_knn(b, 10, flags=_lib.QF_AUTOTUNE, sync=False, stream=s2)
        ix.batch_knn(a, 10, sync=False, stream=s2)
        torch.cuda.synchronize()
        for q, qs in ((a, qa), (b, qb)):
            rows = np.arange(0, len(qs), 29)
            gu.assert_rows_equal(q.r_indexes.cpu().numpy()[rows], q.r_distances.cpu().numpy()[rows],
                                 *oracle.bf_knn(pts, qs[rows], 10, fma=True, threads=8),
                                 what=f"{structure} rep {rep} n={len(qs)}")
    ix.close()


@pytest.mark.parametrize("learned", [False, True])
def test_host_pipeline_matches_device_call(learned):
    """600,000 queries through knn_query_host: rows equal knn_query on device buffers, bit for
    bit, call after call, and a sample equals the oracle."""
    import torch
    from cudaexactknn_gb300 import _lib
    rng = np.random.default_rng(8)
    pts, centres = W.mixture(rng, 400000, 3, 64, 0.01)
    qs, _ = W.mixture(rng, 600000, 3, 64, 0.01, centres)
    ix = gu.make_index("kd", pts, 0)
    flags = _lib.QF_AUTOTUNE
    if learned:
        train, _ = W.mixture(rng, 16384, 3, 64, 0.01, centres)
        ix.train_radius_model(gu.to_dev(train), 16, steps=600)
        flags |= _lib.QF_LEARNED_RADIUS
    dev_i, dev_d = gu.run(ix, qs, 16, flags=flags)
    h_q = torch.from_numpy(qs).pin_memory()
    h_i = torch.full((len(qs), 16), 7, dtype=torch.int32).pin_memory()
    h_d = torch.full((len(qs), 16), 7.0).pin_memory()
    for _ in range(2):
        ix.knn_host(h_q, 16, INF, h_i, h_d, flags=flags)
        np.testing.assert_array_equal(h_i.numpy(), dev_i)
        np.testing.assert_array_equal(h_d.numpy().view(np.uint32), dev_d.view(np.uint32))
    rows = np.arange(0, len(qs), 1999)
    gu.assert_rows_equal(h_i.numpy()[rows], h_d.numpy()[rows], *oracle.bf_knn(pts, qs[rows], 16, fma=True, threads=8),
                         what="host pipeline sample")
    # Pageable host memory takes the same path.
    q_np = np.ascontiguousarray(qs[:300000])
    i_np, d_np = ix.knn_host(q_np, 16, INF, flags=flags)
    np.testing.assert_array_equal(i_np.numpy(), dev_i[:300000])
    ix.close()
