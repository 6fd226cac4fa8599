"""The allocation-free brute-force entry point (knn_bf_query_noalloc).

It exists for callers that cannot allocate device memory at query time (inside a CUDA graph
capture, under an allocator that forbids side allocations): they pass their own points, queries
and result buffers, and the query's scratch comes from a fixed array inside the library.  Its
rows must equal those of the regular entry point (knn_query on a brute-force index of the same
points), bit for bit, on consecutive calls that reuse that array.  This file is collected last,
so a run that stops at the first failure has run every other test first; it also passes on its
own in a fresh process."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, pts, qs, k, r2, idx, dist):
    return lib.knn_bf_query_noalloc(pts.data_ptr(), pts.shape[0], pts.shape[1], qs.data_ptr(), qs.shape[0],
                                    float(r2), k, idx.data_ptr(), dist.data_ptr(), None)


@pytest.mark.parametrize("dims,n,nq,k,r2", [(3, 70000, 3000, 8, float("inf")),
                                            (16, 20000, 900, 32, float("inf")),
                                            (5, 9001, 4096, 10, 0.05)])
def test_noalloc_matches_regular_entry_point_twice(dims, n, nq, k, r2):
    import torch
    from cudaexactknn_gb300 import _lib, knn
    lib = _lib.load()
    rng = np.random.default_rng(dims + n)
    pts = torch.from_numpy(rng.random((n, dims), dtype=np.float32)).cuda()
    index = knn.BruteForceGpu(pts)
    for call in range(2):
        qs = torch.from_numpy(rng.random((nq, dims), dtype=np.float32)).cuda()
        want_i, want_d = index.knn(qs, k, r2)
        got_i = torch.full((nq, k), 7, dtype=torch.int32, device="cuda")
        got_d = torch.full((nq, k), 7.0, dtype=torch.float32, device="cuda")
        _lib.check(_noalloc(lib, pts, qs, k, r2, got_i, got_d))
        torch.cuda.synchronize()
        assert torch.equal(got_i, want_i), f"call {call}: indices differ"
        assert torch.equal(got_d.view(torch.int32), want_d.view(torch.int32)), f"call {call}: distances differ"
    index.close()


def test_noalloc_rejects_batches_beyond_its_scratch():
    import torch
    from cudaexactknn_gb300 import _lib
    lib = _lib.load()
    pts = torch.rand(1000, 3, device="cuda")
    qs = torch.rand(8193, 3, device="cuda")
    idx = torch.empty((8193, 128), dtype=torch.int32, device="cuda")
    dist = torch.empty((8193, 128), dtype=torch.float32, device="cuda")
    st = _noalloc(lib, pts, qs, 128, float("inf"), idx, dist)  # 8193 * 128 > 1,048,576
    assert st == _lib.ERR_UNSUPPORTED
    assert b"16 MiB" in lib.knn_last_error()


def test_noalloc_leaves_free_device_memory_unchanged():
    """After a first call (which may let the runtime size its per-thread stack pool for the
    kernel), a further call changes the device's free memory by nothing: the entry point itself
    allocates nothing."""
    import torch
    from cudaexactknn_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(17)
    pts = torch.from_numpy(rng.random((50000, 8), dtype=np.float32)).cuda()
    qs = torch.from_numpy(rng.random((2000, 8), dtype=np.float32)).cuda()
    idx = torch.empty((2000, 64), dtype=torch.int32, device="cuda")
    dist = torch.empty((2000, 64), dtype=torch.float32, device="cuda")
    _lib.check(_noalloc(lib, pts, qs, 64, float("inf"), idx, dist))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _lib.check(_noalloc(lib, pts, qs, 64, float("inf"), idx, dist))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
