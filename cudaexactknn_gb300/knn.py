"""Python mirror of the reference's GPU API (namespace KnnTrees of rezvoj/CudaExactKnn).

Same names, argument meanings and error behaviour, with torch CUDA tensors standing in for the
reference's raw device pointers:

    reference (src/KnnTrees.cuh, src/*Gpu.cuh)            here
    ------------------------------------------------------------------------------------------
    Query<Dims,K>{points, count, maxDistance2,            Query(points, count, max_distance2,
                  rIndexes, rDistances}                         r_indexes, r_distances)
    BruteForceGpu<Dims>(devicePoints, size)               BruteForceGpu(points, size)
    KdTreeGpu<Dims,AuxDims,CBlockSize>(p, size, skips)    KdTreeGpu(points, size, depth_skips,
                                                                    aux_dims, c_block_size)
    BallTreeGpu<Dims,CBlockSize>(p, size, skips)          BallTreeGpu(points, size, depth_skips,
                                                                      c_block_size)
    bf.batchKnn<K,BLOCK,HEAP,SH_NN>(query)                bf.batch_knn(query, block_size, heap,
                                                                       shmem_tracking)
    tree.batchKnn<K,BLOCK,HEAP,SH_NN,SH_STACK>(query)     tree.batch_knn(query, block_size, heap,
                                                                         shmem_tracking, shmem_stack)
    KnnTrees::CudaException                               CudaException (a KnnError)

K is the second dimension of r_indexes / r_distances ([count, K] int32 / float32 tensors).
Like the reference, batch_knn waits for the work to finish (``sync=False`` leaves it enqueued on
the current torch stream).  Results are the reference's answers with every row in ascending
(distance, index) order.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import torch

from . import _lib
from ._lib import KnnError

CudaException = KnnError


def _stream_handle(stream: torch.cuda.Stream | None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _check_points(points: torch.Tensor, name: str = "points") -> torch.Tensor:
    if not isinstance(points, torch.Tensor) or not points.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if points.dtype != torch.float32 or points.dim() != 2:
        raise TypeError(f"{name} must be float32 [n, dims]")
    return points.contiguous()


# The C ABI takes raw pointers and trusts the sizes it is given, as the reference's classes do.
# The checks below hold every size the mirror passes to the sizes of the tensors behind the
# pointers, so that a wrong shape is an exception here instead of an out-of-bounds access.

def _check_size(points: torch.Tensor, size: int | None) -> int:
    """Points the index takes: `size` (the reference's size argument) or every row, never more."""
    rows = int(points.shape[0])
    n = rows if size is None else int(size)
    if n < 0 or n > rows:
        raise ValueError(f"size {n}: points has {rows} rows")
    return n


def _check_dims(t: torch.Tensor, dims: int, name: str) -> None:
    if t.dim() != 2 or int(t.shape[1]) != dims:
        raise ValueError(f"{name} must be [count, {dims}] for this index, got {list(t.shape)}")


def _check_results(indexes, distances, count: int, k: int, device: torch.device) -> None:
    """Result buffers the engine writes: contiguous [>= count, k] int32 / float32 on `device`."""
    for t, dt in ((indexes, torch.int32), (distances, torch.float32)):
        if (not isinstance(t, torch.Tensor) or t.dtype != dt or t.dim() != 2 or t.shape[0] < count
                or t.shape[1] != k or not t.is_contiguous() or t.device != device):
            raise TypeError(f"result buffers must be contiguous [count, k] int32 / float32 tensors on {device}")


@dataclass
class Query:
    """Query<Dims,K> (src/KnnTrees.cuh:224-231): device points and result buffers."""

    points: torch.Tensor
    count: int
    max_distance2: float
    r_indexes: torch.Tensor | None = None
    r_distances: torch.Tensor | None = None

    def ensure_outputs(self, k: int) -> None:
        dev = self.points.device
        if self.r_indexes is None:
            self.r_indexes = torch.empty((self.count, k), dtype=torch.int32, device=dev)
        if self.r_distances is None:
            self.r_distances = torch.empty((self.count, k), dtype=torch.float32, device=dev)


class _Index:
    structure = -1

    def __init__(self):
        self._h = ctypes.c_void_p()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def info(self) -> _lib.IndexInfo:
        out = _lib.IndexInfo()
        _lib.check(_lib.load().knn_index_get_info(self._h, ctypes.byref(out)))
        return out

    def close(self) -> None:
        if self._h:
            _lib.load().knn_destroy(self._h)
            self._h = ctypes.c_void_p()

    def serialize(self, stream=None) -> bytes:
        """The index (device arrays and any radius model) as bytes (knn_index_serialize)."""
        lib = _lib.load()
        size = ctypes.c_size_t()
        _lib.check(lib.knn_index_serialize(self._h, None, 0, ctypes.byref(size), _stream_handle(stream)))
        buf = ctypes.create_string_buffer(size.value)
        _lib.check(lib.knn_index_serialize(self._h, buf, size.value, ctypes.byref(size), _stream_handle(stream)))
        return buf.raw

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _query(self, query: Query, k: int | None, o: _lib.QueryOpts, sync: bool, stream, radii=None):
        q = _check_points(query.points, "query.points")
        _check_dims(q, self.dims, "query.points")
        if k is None:
            if query.r_indexes is None:
                raise ValueError("k is needed when the query has no result buffers")
            k = int(query.r_indexes.shape[1])
        query.ensure_outputs(k)
        _check_results(query.r_indexes, query.r_distances, query.count, k, q.device)
        if q.shape[0] < query.count:
            raise ValueError("query.points has fewer rows than query.count")
        lib = _lib.load()
        if radii is None:
            st = lib.knn_query(self._h, q.data_ptr(), query.count, float(query.max_distance2), k,
                               query.r_indexes.data_ptr(), query.r_distances.data_ptr(),
                               ctypes.byref(o), _stream_handle(stream))
        else:
            st = lib.knn_query_radii(self._h, q.data_ptr(), query.count, radii.data_ptr(), k,
                                     query.r_indexes.data_ptr(), query.r_distances.data_ptr(),
                                     ctypes.byref(o), _stream_handle(stream))
        _lib.check(st)
        if sync:
            torch.cuda.synchronize(q.device)
        return query.r_indexes, query.r_distances

    def batch_knn(self, query: Query, k: int | None = None, block_size: int = 0, heap: bool = False,
                  shmem_tracking: bool = False, shmem_stack: bool = False, flags: int = 0,
                  leaf_scan: int = 0, traversal: int = 0, tc_cap: int = 0, sync: bool = True, stream=None):
        """batchKnn<K,BLOCK_SIZE,USE_HEAP_TRACKING,USE_TRACKING_SHMEM,USE_STACK_SHMEM>(query)."""
        o = _lib.opts(block_size, heap, shmem_tracking, shmem_stack, flags, leaf_scan, traversal, tc_cap)
        return self._query(query, k, o, sync, stream)

    def batch_knn_radii(self, query: Query, radii: torch.Tensor, k: int | None = None, sync: bool = True,
                        stream=None, **kw):
        """batch_knn with one max_distance2 per query (float32 CUDA tensor [count])."""
        if (radii.dtype != torch.float32 or not radii.is_cuda or radii.numel() < query.count
                or radii.device != query.points.device):
            raise TypeError("radii must be a float32 CUDA tensor with one entry per query, on the queries' device")
        o = _lib.opts(**{key: kw[key] for key in kw})
        return self._query(query, k, o, sync, stream, radii=radii.contiguous())

    def knn(self, queries: torch.Tensor, k: int, max_distance2: float = math.inf, **kw):
        """Convenience: new result tensors for `queries` ([count, dims] CUDA float32)."""
        q = Query(queries, int(queries.shape[0]), max_distance2)
        return self.batch_knn(q, k, **kw)

    def knn_host(self, queries, k: int, max_distance2: float = math.inf, out_idx=None, out_dist=None,
                 block_size=0, heap=False, shmem_tracking=False, shmem_stack=False, flags=0, leaf_scan=0,
                 traversal=0, stream=None):
        """End-to-end query on host buffers (numpy or CPU tensors; pinned memory is fastest)."""
        qt = torch.as_tensor(queries)
        if qt.dtype != torch.float32 or not qt.is_contiguous() or qt.is_cuda:
            raise TypeError("host queries must be a contiguous float32 CPU array")
        _check_dims(qt, self.dims, "queries")
        count = int(qt.shape[0])
        if out_idx is None:
            out_idx = torch.empty((count, k), dtype=torch.int32, pin_memory=qt.is_pinned())
        if out_dist is None:
            out_dist = torch.empty((count, k), dtype=torch.float32, pin_memory=qt.is_pinned())
        _check_results(out_idx, out_dist, count, k, torch.device("cpu"))
        o = _lib.opts(block_size, heap, shmem_tracking, shmem_stack, flags, leaf_scan, traversal)
        st = _lib.load().knn_query_host(self._h, qt.data_ptr(), count, float(max_distance2), k,
                                        out_idx.data_ptr(), out_dist.data_ptr(), ctypes.byref(o),
                                        _stream_handle(stream))
        _lib.check(st)
        return out_idx, out_dist

    # ---- learned radius ---------------------------------------------------------------------
    def train_radius_model(self, samples: torch.Tensor, k: int, steps: int = 0, batch: int = 0, lr: float = 0.0,
                           coverage: float = 0.0, seed: int = 0, stream=None) -> _lib.TrainReport:
        """Trains the index's radius model on sample queries (CUDA float32 [count, dims])."""
        s = _check_points(samples, "samples")
        _check_dims(s, self.dims, "samples")
        o = _lib.TrainOpts()
        o.steps, o.batch, o.lr, o.coverage, o.seed = steps, batch, lr, coverage, seed
        rep = _lib.TrainReport()
        _lib.check(_lib.load().knn_radius_model_train(self._h, s.data_ptr(), int(s.shape[0]), k, ctypes.byref(o),
                                                      _stream_handle(stream), ctypes.byref(rep)))
        return rep

    def predict_log_kth(self, queries: torch.Tensor) -> torch.Tensor:
        q = _check_points(queries, "queries")
        _check_dims(q, self.dims, "queries")
        out = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
        _lib.check(_lib.load().knn_radius_model_predict(self._h, q.data_ptr(), int(q.shape[0]), out.data_ptr(),
                                                        _stream_handle(None)))
        return out

    def export_radius_model(self):
        import numpy as np
        lib = _lib.load()
        n = lib.knn_radius_model_size(self.dims)
        out = np.empty(n, dtype=np.float32)
        _lib.check(lib.knn_radius_model_export(self._h, out.ctypes.data, n))
        return out

    def import_radius_model(self, params, k: int) -> None:
        import numpy as np
        p = np.ascontiguousarray(params, dtype=np.float32)
        _lib.check(_lib.load().knn_radius_model_import(self._h, p.ctypes.data, p.size, k))

    def stats(self, query: Query, k: int, **kw) -> _lib.QueryCounters:
        """Runs the query with device counters (nodes visited, leaves, points scanned)."""
        q = _check_points(query.points, "query.points")
        _check_dims(q, self.dims, "query.points")
        if q.shape[0] < query.count:
            raise ValueError("query.points has fewer rows than query.count")
        query.ensure_outputs(k)
        _check_results(query.r_indexes, query.r_distances, query.count, k, q.device)
        o = _lib.opts(**kw)
        out = _lib.QueryCounters()
        st = _lib.load().knn_query_stats(self._h, q.data_ptr(), query.count, float(query.max_distance2), k,
                                         query.r_indexes.data_ptr(), query.r_distances.data_ptr(),
                                         ctypes.byref(o), _stream_handle(None), ctypes.byref(out))
        _lib.check(st)
        return out


class BruteForceGpu(_Index):
    """BruteForceGpu<Dims> (src/BruteForceGpu.cuh:54-85)."""

    structure = _lib.BRUTE_FORCE

    def __init__(self, points: torch.Tensor, size: int | None = None, stream=None):
        super().__init__()
        p = _check_points(points)
        n = _check_size(p, size)
        self.dims = int(p.shape[1])
        _lib.check(_lib.load().knn_bf_create(p.data_ptr(), n, self.dims, _stream_handle(stream),
                                             ctypes.byref(self._h)))


class KdTreeGpu(_Index):
    """KdTreeGpu<Dims,AuxDims,CBlockSize> (src/KdTreeGpu.cuh:282-412: constructor 375-385, batchKnn 393-410)."""

    structure = _lib.KD_TREE

    def __init__(self, points: torch.Tensor, size: int | None = None, depth_skips: int = 0,
                 aux_dims: int | None = None, c_block_size: int = 256, stream=None):
        super().__init__()
        p = _check_points(points)
        n = _check_size(p, size)
        self.dims = int(p.shape[1])
        aux = self.dims if aux_dims is None else int(aux_dims)
        _lib.check(_lib.load().knn_kd_create(p.data_ptr(), n, self.dims, aux, depth_skips, c_block_size,
                                             _stream_handle(stream), ctypes.byref(self._h)))


class BallTreeGpu(_Index):
    """BallTreeGpu<Dims,CBlockSize> (src/BallTreeGpu.cuh:463-650)."""

    structure = _lib.BALL_TREE

    def __init__(self, points: torch.Tensor, size: int | None = None, depth_skips: int = 1,
                 c_block_size: int = 256, stream=None):
        super().__init__()
        p = _check_points(points)
        n = _check_size(p, size)
        self.dims = int(p.shape[1])
        _lib.check(_lib.load().knn_ball_create(p.data_ptr(), n, self.dims, depth_skips, c_block_size,
                                               _stream_handle(stream), ctypes.byref(self._h)))


def load_index(blob: bytes, stream=None) -> _Index:
    """An index rebuilt from `_Index.serialize()` bytes on the current device (knn_index_deserialize)."""
    h = ctypes.c_void_p()
    buf = ctypes.create_string_buffer(bytes(blob), len(blob))
    _lib.check(_lib.load().knn_index_deserialize(buf, len(blob), _stream_handle(stream), ctypes.byref(h)))
    info = _lib.IndexInfo()
    _lib.check(_lib.load().knn_index_get_info(h, ctypes.byref(info)))
    cls = {_lib.BRUTE_FORCE: BruteForceGpu, _lib.KD_TREE: KdTreeGpu, _lib.BALL_TREE: BallTreeGpu}[info.structure]
    ix = cls.__new__(cls)
    _Index.__init__(ix)
    ix._h = h
    ix.dims = int(info.dims)
    return ix


class Batch:
    """Many (tree, query batch) pairs answered by one CUDA-graph launch (knn_batch_create/run).

    ``items`` is a list of ``(index, queries, k, max_distance2)``; the result tensors are made
    here and reused by every ``run``.  Refill the query tensors in place between runs: their
    addresses are part of the captured graph.  The reference answers each pair with its own
    batchKnn call (src/KdTreeGpu.cuh:392-410, src/BallTreeGpu.cuh:630-648)."""

    def __init__(self, items, autotune: bool = False, keep_order: bool = False, stream=None):
        self._h = ctypes.c_void_p()
        self.items = []
        arr = (_lib.BatchItem * max(1, len(items)))()
        for j, (ix, queries, k, r2) in enumerate(items):
            q = _check_points(queries, "queries")
            if q.shape[1] != ix.dims:
                raise ValueError(f"item {j}: queries have {q.shape[1]} dims, the index {ix.dims}")
            oi = torch.empty((q.shape[0], k), dtype=torch.int32, device=q.device)
            od = torch.empty((q.shape[0], k), dtype=torch.float32, device=q.device)
            self.items.append((ix, q, oi, od))
            arr[j] = _lib.BatchItem(ix.handle.value, q.data_ptr(), q.shape[0], r2, k, oi.data_ptr(), od.data_ptr())
        flags = (_lib.QF_AUTOTUNE if autotune else 0) | (_lib.QF_KEEP_ORDER if keep_order else 0)
        _lib.check(_lib.load().knn_batch_create(arr, len(items), flags, _stream_handle(stream), ctypes.byref(self._h)))

    def run(self, sync: bool = True, stream=None):
        """Answers every item; returns [(indexes, distances)] in item order."""
        _lib.check(_lib.load().knn_batch_run(self._h, _stream_handle(stream)))
        if sync:
            (stream or torch.cuda.current_stream()).synchronize()
        return [(oi, od) for _, _, oi, od in self.items]

    def info(self) -> tuple[int, int]:
        """(classes, kernel launches per run)."""
        c, k = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(_lib.load().knn_batch_info(self._h, ctypes.byref(c), ctypes.byref(k)))
        return c.value, k.value

    def close(self) -> None:
        if self._h:
            _lib.load().knn_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_index(structure: str, points: torch.Tensor, depth_skips: int | None = None, **kw) -> _Index:
    if structure == "bf":
        return BruteForceGpu(points, **kw)
    if structure == "kd":
        return KdTreeGpu(points, depth_skips=0 if depth_skips is None else depth_skips, **kw)
    if structure == "ball":
        return BallTreeGpu(points, depth_skips=1 if depth_skips is None else depth_skips, **kw)
    raise ValueError(structure)


def radius_model_gradients(params, dims: int, x, targets):
    """Forward + backward of the radius model on the GPU for a host batch: (loss, gradients)."""
    import numpy as np
    lib = _lib.load()
    p = np.ascontiguousarray(params, np.float32)
    xb = np.ascontiguousarray(x, np.float32)
    tb = np.ascontiguousarray(targets, np.float32)
    n = lib.knn_radius_model_size(dims)
    trainable = n - dims * 32 - 2 * dims - 1
    grad = np.empty(trainable, np.float32)
    loss = ctypes.c_float()
    _lib.check(lib.knn_radius_model_gradients(p.ctypes.data, dims, xb.ctypes.data, tb.ctypes.data, len(tb),
                                              grad.ctypes.data, ctypes.byref(loss)))
    return loss.value, grad
