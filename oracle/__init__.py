"""CPU oracle for the exact-kNN path (ctypes wrapper over oracle/libknn_oracle.so).

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module, as the checker or as the timed CPU baseline.  The engine
(``cudaexactknn_gb300``) never imports it.

``knn_oracle.cpp`` restates the reference's CPU algorithms (src/BruteForce.cuh, src/KdTree.cuh,
src/BallTree.cuh, src/KnnTrees.cuh); ``ref_bridge.cu`` compiles the reference's own classes into
``oracle/_ref`` when the reference sources are present, and ``ref_knn`` below calls them.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(HERE, "libknn_oracle.so")
_REF_SO = os.path.join(HERE, "_ref", "libknn_ref.so")
_REF_FMA_SO = os.path.join(HERE, "_ref", "libknn_ref_fma.so")

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32 = ctypes.c_uint32

_lib = None
_ref = {}


def build(with_reference: bool = True) -> None:
    """Compile the oracle (and, when the reference sources exist, oracle/_ref)."""
    target = [] if with_reference else ["oracle"]
    subprocess.run(["make", "-s", "-C", HERE] + target, check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_ORACLE_SO):
            build(with_reference=False)
        lib = ctypes.CDLL(_ORACLE_SO)
        lib.oracle_bf_knn.argtypes = [_f32p, _u32, _u32, _f32p, _u32, ctypes.c_float, _u32,
                                      ctypes.c_int, ctypes.c_int, _i32p, _f32p, ctypes.c_int]
        lib.oracle_bf_knn.restype = ctypes.c_int
        lib.oracle_kd_build.argtypes = [_f32p, _u32, _u32, _u32]
        lib.oracle_kd_build.restype = ctypes.c_void_p
        lib.oracle_kd_knn.argtypes = [ctypes.c_void_p, _f32p, _u32, ctypes.c_float, _u32,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _f32p,
                                      ctypes.c_int]
        lib.oracle_kd_knn.restype = ctypes.c_int
        lib.oracle_kd_free.argtypes = [ctypes.c_void_p]
        lib.oracle_ball_build.argtypes = [_f32p, _u32, _u32, _u32, ctypes.c_int]
        lib.oracle_ball_build.restype = ctypes.c_void_p
        lib.oracle_ball_knn.argtypes = lib.oracle_kd_knn.argtypes
        lib.oracle_ball_knn.restype = ctypes.c_int
        lib.oracle_ball_free.argtypes = [ctypes.c_void_p]
        lib.oracle_tree_shape.argtypes = [_u32, _u32, ctypes.c_int, ctypes.POINTER(_u32),
                                          ctypes.POINTER(_u32), ctypes.POINTER(_u32)]
        lib.oracle_dist2.argtypes = [_f32p, _f32p, _u32, ctypes.c_int]
        lib.oracle_dist2.restype = ctypes.c_float
        _lib = lib
    return _lib


def _c(a: np.ndarray, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f32p)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_i32p)


def _out(nq: int, k: int):
    return np.empty((nq, k), np.int32), np.empty((nq, k), np.float32)


def bf_knn(points, queries, k, max_dist2=float("inf"), heap=False, fma=True, threads=1):
    """Brute force, every query against every point (src/BruteForce.cuh:27-44)."""
    lib = _load()
    p, q = _c(points, np.float32), _c(queries, np.float32)
    n, d = p.shape
    idx, dist = _out(q.shape[0], k)
    rc = lib.oracle_bf_knn(_fp(p), n, d, _fp(q), q.shape[0], max_dist2, k, int(heap), int(fma),
                           _ip(idx), _fp(dist), threads)
    if rc:
        raise ValueError("oracle_bf_knn rejected its arguments")
    return idx, dist


class _Tree:
    def __init__(self, kind, points, skips, fma=True):
        self._lib = _load()
        self.kind = kind
        self.points = _c(points, np.float32)
        n, d = self.points.shape
        self.dims = d
        if kind == "kd":
            self._h = self._lib.oracle_kd_build(_fp(self.points), n, d, skips)
        else:
            self._h = self._lib.oracle_ball_build(_fp(self.points), n, d, skips, int(fma))
        if not self._h:
            raise ValueError("empty point set")

    def knn(self, queries, k, max_dist2=float("inf"), heap=False, fma=True, strict=True, threads=1):
        q = _c(queries, np.float32)
        idx, dist = _out(q.shape[0], k)
        fn = self._lib.oracle_kd_knn if self.kind == "kd" else self._lib.oracle_ball_knn
        rc = fn(self._h, _fp(q), q.shape[0], max_dist2, k, int(heap), int(fma), int(strict),
                _ip(idx), _fp(dist), threads)
        if rc:
            raise ValueError("oracle tree query rejected its arguments")
        return idx, dist

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            (self._lib.oracle_kd_free if self.kind == "kd" else self._lib.oracle_ball_free)(h)
            self._h = None


def kd_tree(points, skips=0):
    """k-d tree of src/KdTree.cuh:27-71 (split dim = depth % dims)."""
    return _Tree("kd", points, skips)


def ball_tree(points, skips=1, fma=True):
    """Ball tree of src/BallTree.cuh:27-137."""
    return _Tree("ball", points, skips, fma)


def tree_shape(n, skips, ball=False):
    """(node_depth, leaf_slots, node_count) the reference derives from n and depthSkips."""
    lib = _load()
    a, b, c = _u32(), _u32(), _u32()
    lib.oracle_tree_shape(n, skips, int(ball), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def dist2(a, b, fma=True) -> float:
    lib = _load()
    a, b = _c(a, np.float32), _c(b, np.float32)
    return float(lib.oracle_dist2(_fp(a), _fp(b), a.shape[0], int(fma)))


# ----------------------------------------------------------------------------------------------
# The reference's own CPU classes (oracle/_ref), available where the reference sources were
# present at build time and the build machine matches this one.
# ----------------------------------------------------------------------------------------------

def ref_available(fma: bool = False) -> bool:
    try:
        _ref_lib(fma)
        return True
    except OSError:
        return False


def _ref_lib(fma: bool):
    key = bool(fma)
    if key not in _ref:
        lib = ctypes.CDLL(_REF_FMA_SO if fma else _REF_SO)
        lib.ref_knn.argtypes = [ctypes.c_int, _f32p, _u32, _u32, _f32p, _u32, ctypes.c_float, _u32,
                                _u32, ctypes.c_int, _i32p, _f32p, ctypes.c_int]
        lib.ref_knn.restype = ctypes.c_int
        lib.ref_has_pair.argtypes = [_u32, _u32]
        lib.ref_has_pair.restype = ctypes.c_int
        _ref[key] = lib
    return _ref[key]


def ref_has_pair(dims: int, k: int) -> bool:
    return bool(_ref_lib(False).ref_has_pair(dims, k))


def ref_knn(kind, points, queries, k, max_dist2=float("inf"), skips=0, heap=False, fma=False,
            threads=1):
    """Run the reference's BruteForce/KdTree/BallTree (kind 'bf'/'kd'/'ball') on the CPU."""
    lib = _ref_lib(fma)
    p, q = _c(points, np.float32), _c(queries, np.float32)
    idx, dist = _out(q.shape[0], k)
    code = {"bf": 0, "kd": 1, "ball": 2}[kind]
    rc = lib.ref_knn(code, _fp(p), p.shape[0], p.shape[1], _fp(q), q.shape[0], max_dist2, k, skips,
                     int(heap), _ip(idx), _fp(dist), threads)
    if rc:
        raise ValueError(f"reference bridge has no instantiation for dims={p.shape[1]} k={k}")
    return idx, dist


# ----------------------------------------------------------------------------------------------
# Row comparison under the reference's tie rule.
# ----------------------------------------------------------------------------------------------

def row_keys(idx: np.ndarray, dist: np.ndarray) -> np.ndarray:
    """u64 keys (bits(dist) << 32 | uint32(idx)), each row sorted ascending.

    Heap tracking returns rows in heap order (src/KnnTrees.cuh:154-189); sorting by key gives
    the canonical order every tracking mode agrees on.
    """
    hi = np.ascontiguousarray(dist, np.float32).view(np.uint32).astype(np.uint64) << np.uint64(32)
    lo = np.ascontiguousarray(idx, np.int32).view(np.uint32).astype(np.uint64)
    return np.sort(hi | lo, axis=1)


def split_keys(keys: np.ndarray):
    idx = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.int32)
    dist = (keys >> np.uint64(32)).astype(np.uint32).view(np.float32)
    return idx, dist


def ulp_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """|a - b| in units in the last place, for non-negative float32 values."""
    ai = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ai - bi)
