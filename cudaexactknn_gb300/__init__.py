"""GB300 (sm_103a) exact k-nearest-neighbour engine: brute force, k-d tree and ball tree behind
the reference's KnnTrees API, with hand-written CUDA kernels behind a C ABI
(include/cudaexactknn.h, built into libcudaexactknn.so)."""

from . import _lib  # noqa: F401
from ._lib import KnnError  # noqa: F401


def __getattr__(name):
    # The torch-facing API is imported lazily so that the C-ABI binding works without torch.
    if name in ("BruteForceGpu", "KdTreeGpu", "BallTreeGpu", "Query", "CudaException", "build_index"):
        from . import knn
        return getattr(knn, name)
    raise AttributeError(name)
