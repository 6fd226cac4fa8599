"""Helpers of the GPU parity tests: run the engine through the C ABI (via the Python mirror)
on numpy inputs and compare rows with the oracle under the reference's tie rule."""

import numpy as np
import torch

import oracle
from cudaexactknn_gb300 import knn

DEV = torch.device("cuda:0")


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(DEV)


def make_index(structure, points, depth_skips=None, aux_dims=None):
    p = to_dev(points)
    if structure == "bf":
        return knn.BruteForceGpu(p)
    if structure == "kd":
        return knn.KdTreeGpu(p, depth_skips=0 if depth_skips is None else depth_skips, aux_dims=aux_dims)
    return knn.BallTreeGpu(p, depth_skips=1 if depth_skips is None else depth_skips)


def run(ix, queries, k, max_distance2=float("inf"), **kw):
    idx, dist = ix.knn(to_dev(queries), k, max_distance2, **kw)
    return idx.cpu().numpy(), dist.cpu().numpy()


def assert_rows_equal(got_idx, got_dist, want_idx, want_dist, what=""):
    g = oracle.row_keys(got_idx, got_dist)
    w = oracle.row_keys(want_idx, want_dist)
    bad = np.where((g != w).any(axis=1))[0]
    if len(bad):
        i = bad[0]
        gi, gd = oracle.split_keys(g[i:i + 1])
        wi, wd = oracle.split_keys(w[i:i + 1])
        raise AssertionError(f"{what}: {len(bad)} rows differ; first row {i}:\n got  {gi}\n      {gd}\n want {wi}\n      {wd}")


def assert_sorted_rows(idx, dist):
    keys = (dist.view(np.uint32).astype(np.uint64) << np.uint64(32)) | idx.view(np.uint32).astype(np.uint64)
    assert (keys[:, 1:] >= keys[:, :-1]).all(), "rows must come back in ascending key order"
