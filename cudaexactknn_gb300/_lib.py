"""ctypes binding of the engine's C ABI (include/cudaexactknn.h).

The shared library is built in-tree by ``cudaexactknn_gb300.build`` (or ``__graft_entry__.build``).
There is no fallback: if the library is missing, ``load()`` raises.
"""

from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libcudaexactknn.so")
HEADER = os.path.join(ROOT, "include", "cudaexactknn.h")

# Status codes (enum knn_status).
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_OUT_OF_MEMORY = 4
ERR_DEVICE_LIMIT = 5
ERR_NOT_TRAINED = 6

BRUTE_FORCE, KD_TREE, BALL_TREE = 0, 1, 2

QF_SYNC = 1
QF_AUTOTUNE = 2
QF_LEARNED_RADIUS = 4
QF_BF16_FILTER = 8
QF_KEEP_ORDER = 16
QF_TIMING = 32
QF_FILTER_CODES = 64
QF_TEST_FILTER_GIVE_UP = 0x40000000


class QueryOpts(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_uint32), ("heap_tracking", ctypes.c_uint32),
                ("shmem_tracking", ctypes.c_uint32), ("shmem_stack", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("leaf_scan", ctypes.c_uint32),
                ("traversal", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class QueryCounters(ctypes.Structure):
    _fields_ = [("nodes_visited", ctypes.c_uint64), ("leaves_visited", ctypes.c_uint64),
                ("points_scanned", ctypes.c_uint64), ("fallback_queries", ctypes.c_uint64),
                ("filter_give_ups", ctypes.c_uint64), ("reserved", ctypes.c_uint64 * 3)]


class IndexInfo(ctypes.Structure):
    _fields_ = [("structure", ctypes.c_uint32), ("n", ctypes.c_uint32), ("dims", ctypes.c_uint32),
                ("aux_dims", ctypes.c_uint32), ("depth_skips", ctypes.c_uint32),
                ("node_depth", ctypes.c_uint32), ("leaf_slots", ctypes.c_uint32),
                ("node_count", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64),
                ("build_ms", ctypes.c_float), ("radius_model", ctypes.c_uint32)]


class TrainOpts(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint32), ("batch", ctypes.c_uint32), ("lr", ctypes.c_float),
                ("coverage", ctypes.c_float), ("seed", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 3)]


class TrainReport(ctypes.Structure):
    _fields_ = [("train_ms", ctypes.c_float), ("final_batch_loss", ctypes.c_float), ("rmse", ctypes.c_float),
                ("margin", ctypes.c_float), ("coverage", ctypes.c_float), ("samples", ctypes.c_uint32),
                ("steps", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class BatchItem(ctypes.Structure):
    _fields_ = [("index", ctypes.c_void_p), ("d_queries", ctypes.c_void_p), ("count", ctypes.c_uint32),
                ("max_distance2", ctypes.c_float), ("k", ctypes.c_uint32), ("d_indexes", ctypes.c_void_p),
                ("d_distances", ctypes.c_void_p)]


class KnnError(RuntimeError):
    """A non-zero knn_status; ``.status`` holds the code (the reference throws CudaException)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} [status {status}]")
        self.status = status


_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_f = ctypes.c_float
_pp = ctypes.POINTER(ctypes.c_void_p)

_SIGNATURES = {
    "knn_bf_create": [_vp, _u32, _u32, _vp, _pp],
    "knn_kd_create": [_vp, _u32, _u32, _u32, _u32, _u32, _vp, _pp],
    "knn_ball_create": [_vp, _u32, _u32, _u32, _u32, _vp, _pp],
    "knn_destroy": [_vp],
    "knn_index_get_info": [_vp, ctypes.POINTER(IndexInfo)],
    "knn_index_serialize": [_vp, _vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), _vp],
    "knn_index_deserialize": [_vp, ctypes.c_size_t, _vp, _pp],
    "knn_query": [_vp, _vp, _u32, _f, _u32, _vp, _vp, ctypes.POINTER(QueryOpts), _vp],
    "knn_query_radii": [_vp, _vp, _u32, _vp, _u32, _vp, _vp, ctypes.POINTER(QueryOpts), _vp],
    "knn_query_host": [_vp, _vp, _u32, _f, _u32, _vp, _vp, ctypes.POINTER(QueryOpts), _vp],
    "knn_query_stats": [_vp, _vp, _u32, _f, _u32, _vp, _vp, ctypes.POINTER(QueryOpts), _vp,
                        ctypes.POINTER(QueryCounters)],
    "knn_radius_model_train": [_vp, _vp, _u32, _u32, ctypes.POINTER(TrainOpts), _vp, ctypes.POINTER(TrainReport)],
    "knn_radius_model_predict": [_vp, _vp, _u32, _vp, _vp],
    "knn_radius_model_size": [_u32],
    "knn_radius_model_export": [_vp, _vp, _u32],
    "knn_radius_model_import": [_vp, _vp, _u32, _u32],
    "knn_radius_model_gradients": [_vp, _u32, _vp, _vp, _u32, _vp, _vp],
    "knn_last_query_timing": [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
    "knn_launch_count": [],
    "knn_batch_create": [ctypes.POINTER(BatchItem), _u32, _u32, _vp, _pp],
    "knn_batch_run": [_vp, _vp],
    "knn_batch_info": [_vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)],
    "knn_batch_destroy": [_vp],
    "knn_bf_query_noalloc": [_vp, _u32, _u32, _vp, _u32, _f, _u32, _vp, _vp, _vp],
    "knn_tc_selftest": [_u32, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32)],
    "knn_tuned_plan": [_vp, _u32, _u32, ctypes.POINTER(QueryOpts), ctypes.POINTER(ctypes.c_float)],
    "knn_status_string": [ctypes.c_int],
    "knn_last_error": [],
    "knn_version": [],
}

_lib = None


def header_symbols() -> list[str]:
    """Names of the functions include/cudaexactknn.h declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"KNN_API\s+(?:const\s+char\s*\*|int|uint64_t|uint32_t)\s+(knn_\w+)\s*\(", text)))


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        if name in ("knn_status_string", "knn_last_error"):
            fn.restype = ctypes.c_char_p
        elif name == "knn_launch_count":
            fn.restype = ctypes.c_uint64
        elif name == "knn_radius_model_size":
            fn.restype = ctypes.c_uint32
        else:
            fn.restype = ctypes.c_int
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        lib = load()
        raise KnnError(status, lib.knn_last_error().decode(errors="replace") or
                       lib.knn_status_string(status).decode())


def opts(block_size=0, heap=False, shmem_tracking=False, shmem_stack=False, flags=0, leaf_scan=0,
         traversal=0, tc_cap=0) -> QueryOpts:
    o = QueryOpts()
    o.traversal = traversal
    o.reserved = tc_cap
    o.block_size = block_size
    o.heap_tracking = int(bool(heap))
    o.shmem_tracking = int(bool(shmem_tracking))
    o.shmem_stack = int(bool(shmem_stack))
    o.flags = flags
    o.leaf_scan = leaf_scan
    return o
