"""The Python mirror's argument checks, which need no GPU.

The C ABI trusts the sizes it is given (as the reference's classes trust their raw pointers), so
the mirror holds every size it passes to the tensors behind the pointers: a wrong shape, dtype,
layout or device must raise here, before any call into the library."""

import numpy as np
import pytest
import torch

from cudaexactknn_gb300 import knn


def test_size_never_exceeds_the_rows():
    p = torch.zeros(10, 3)
    assert knn._check_size(p, None) == 10
    assert knn._check_size(p, 4) == 4
    assert knn._check_size(p, 0) == 0
    with pytest.raises(ValueError):
        knn._check_size(p, 11)
    with pytest.raises(ValueError):
        knn._check_size(p, -1)


def test_dims_must_match_the_index():
    knn._check_dims(torch.zeros(5, 3), 3, "q")
    for bad in (torch.zeros(5, 2), torch.zeros(5, 4), torch.zeros(15)):
        with pytest.raises(ValueError):
            knn._check_dims(bad, 3, "q")


@pytest.mark.parametrize("case", ["ok", "dtype", "k", "rows", "strided", "device", "1d", "not a tensor"])
def test_result_buffers(case):
    cpu, count, k = torch.device("cpu"), 6, 4
    idx = torch.zeros(count, k, dtype=torch.int32)
    dist = torch.zeros(count, k, dtype=torch.float32)
    if case == "dtype":
        idx = idx.long()
    elif case == "k":
        dist = torch.zeros(count, k + 1)
    elif case == "rows":
        idx = torch.zeros(count - 1, k, dtype=torch.int32)
    elif case == "strided":
        dist = torch.zeros(k, count).t()
    elif case == "device":
        dist = torch.zeros(count, k, device="meta")
    elif case == "1d":
        idx = torch.zeros(count * k, dtype=torch.int32)
    elif case == "not a tensor":
        dist = np.zeros((count, k), np.float32)
    if case == "ok":
        knn._check_results(idx, dist, count, k, cpu)
        knn._check_results(torch.zeros(count + 3, k, dtype=torch.int32), dist, count, k, cpu)  # spare rows
    else:
        with pytest.raises(TypeError):
            knn._check_results(idx, dist, count, k, cpu)


def _unbuilt_index(dims):
    """An index object without a handle: any call that reached the library would fail there."""
    ix = knn.KdTreeGpu.__new__(knn.KdTreeGpu)
    knn._Index.__init__(ix)
    ix.dims = dims
    return ix


def test_host_query_checks_shapes_before_the_library():
    ix = _unbuilt_index(3)
    qs = np.zeros((5, 3), np.float32)
    with pytest.raises(ValueError):
        ix.knn_host(np.zeros((5, 4), np.float32), 2)
    with pytest.raises(TypeError):
        ix.knn_host(qs, 2, out_idx=torch.zeros(5, 3, dtype=torch.int32))
    with pytest.raises(TypeError):
        ix.knn_host(qs, 2, out_dist=torch.zeros(4, 2))
    with pytest.raises(TypeError):
        ix.knn_host(qs.astype(np.float64), 2)


def test_device_entry_points_refuse_host_tensors():
    ix = _unbuilt_index(3)
    with pytest.raises(TypeError):
        knn.BruteForceGpu(torch.zeros(10, 3))
    with pytest.raises(TypeError):
        ix.knn(torch.zeros(4, 3), 2)
    with pytest.raises(TypeError):
        ix.train_radius_model(torch.zeros(100, 3), 4)
