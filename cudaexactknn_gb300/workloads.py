"""Seeded synthetic workloads for the exact-kNN path.

No public dataset is involved: every workload is generated here from a fixed seed
(numpy PCG64), with the shapes and value distributions of the reference's benchmark
configurations:

* ``uniform``      points i.i.d. uniform in [0, 1)^D (tests/Tests.cuh:85-98 uses this with an
                   unseeded generator; here the seed is fixed).
* ``mixture``      isotropic Gaussian mixture: centres uniform in [0,1)^D, equal weights.
* ``subspace``     a 4-dimensional linear subspace of R^D (random orthonormal basis by
                   Gram-Schmidt in float64), latent N(0, I), plus isotropic N(0, noise^2).
* ``gauss_mix``    Gaussian mixture with centres N(0, I) and per-component sigma.

Named configurations (seed = 1000 + configuration number):

* ``c1``  BruteForce<3>:  N=65,536 uniform, Q=4,096, K=8, max radius +inf, heap tracking.
* ``c2``  KdTreeGpu<3>, depthSkips 0: N=4,194,304 from a 64-component mixture (sigma 0.01),
          Q=1,048,576 from the same mixture, K=16.
* ``c3``  BallTreeGpu<16>, depthSkips 1: N=1,048,576 subspace points (noise 0.05),
          Q=262,144, K=32.
* ``c4``  BruteForceGpu<128>: N=1,048,576 from a 256-component mixture (centres N(0,1),
          sigma 0.3), Q=65,536, K=100.
* ``c5``  64 independent sets: N log-uniform in [1,024, 1,048,576], D from {3, 8, 32},
          K from {1, 10, 64}, uniform points, Q = N/8; k-d tree for D <= 8, ball tree for D = 32.
* ``range``  the reference's range-limited speed test (tests/DimXSpeedTests.cu:10-58): N=500,000
          uniform points in [0,1)^D, Q=10,000 uniform queries, K=5, maxDistance2 = 0.01 D, for D
          in 6..17; k-d tree (depthSkips 3), ball tree (depthSkips 1) or brute force.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

INF = float("inf")


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def uniform(rng: np.random.Generator, n: int, d: int) -> np.ndarray:
    return rng.random((n, d), dtype=np.float32)


def mixture(rng: np.random.Generator, n: int, d: int, components: int, sigma: float,
            centres: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    if centres is None:
        centres = rng.random((components, d)).astype(np.float64)
    comp = rng.integers(0, components, size=n)
    x = centres[comp] + sigma * rng.standard_normal((n, d))
    return x.astype(np.float32), centres


def gauss_mix(rng: np.random.Generator, n: int, d: int, components: int, sigma: float,
              centres: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    if centres is None:
        centres = rng.standard_normal((components, d))
    comp = rng.integers(0, components, size=n)
    x = centres[comp] + sigma * rng.standard_normal((n, d))
    return x.astype(np.float32), centres


def orthonormal_basis(rng: np.random.Generator, d: int, r: int) -> np.ndarray:
    """d x r orthonormal basis by classical Gram-Schmidt on a Gaussian matrix (float64)."""
    g = rng.standard_normal((d, r))
    basis = np.zeros((d, r))
    for j in range(r):
        v = g[:, j].copy()
        for i in range(j):
            v -= np.dot(basis[:, i], g[:, j]) * basis[:, i]
        basis[:, j] = v / np.linalg.norm(v)
    return basis


def subspace(rng: np.random.Generator, n: int, d: int, r: int, noise: float,
             basis: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    if basis is None:
        basis = orthonormal_basis(rng, d, r)
    z = rng.standard_normal((n, r))
    x = z @ basis.T + noise * rng.standard_normal((n, d))
    return x.astype(np.float32), basis


@dataclass
class Workload:
    name: str
    structure: str          # "bf", "kd" or "ball"
    points: np.ndarray
    queries: np.ndarray
    k: int
    max_dist2: float = INF
    depth_skips: int = 0
    heap: bool = False
    extra: dict = field(default_factory=dict)

    @property
    def dims(self) -> int:
        return int(self.points.shape[1])


def c1(scale: float = 1.0) -> Workload:
    rng = _rng(1001)
    n, q = int(65536 * scale), int(4096 * scale)
    return Workload("c1_bf3_n65536_q4096_k8", "bf", uniform(rng, n, 3), uniform(rng, q, 3), 8,
                    INF, 0, heap=True)


def c2(scale: float = 1.0) -> Workload:
    # extra["train"]: sample queries for the learned radius, 65,536 further draws of the same
    # mixture (seeded apart from the benchmark queries); likewise for c3 and c4.
    rng = _rng(1002)
    n, q = int(4194304 * scale), int(1048576 * scale)
    pts, centres = mixture(rng, n, 3, 64, 0.01)
    qs, _ = mixture(rng, q, 3, 64, 0.01, centres)
    train, _ = mixture(_rng(2002), 65536, 3, 64, 0.01, centres)
    return Workload("c2_kd3_n4194304_q1048576_k16", "kd", pts, qs, 16, INF, 0, extra={"train": train})


def c3(scale: float = 1.0) -> Workload:
    rng = _rng(1003)
    n, q = int(1048576 * scale), int(262144 * scale)
    pts, basis = subspace(rng, n, 16, 4, 0.05)
    qs, _ = subspace(rng, q, 16, 4, 0.05, basis)
    train, _ = subspace(_rng(2003), 65536, 16, 4, 0.05, basis)
    return Workload("c3_ball16_n1048576_q262144_k32", "ball", pts, qs, 32, INF, 1, extra={"train": train})


def c4(scale: float = 1.0) -> Workload:
    rng = _rng(1004)
    n, q = int(1048576 * scale), int(65536 * scale)
    pts, centres = gauss_mix(rng, n, 128, 256, 0.3)
    qs, _ = gauss_mix(rng, q, 128, 256, 0.3, centres)
    train, _ = gauss_mix(_rng(2004), 16384, 128, 256, 0.3, centres)
    return Workload("c4_bf128_n1048576_q65536_k100", "bf", pts, qs, 100, INF, 0, extra={"train": train})


def c5_sets(scale: float = 1.0, count: int = 64) -> list[Workload]:
    rng = _rng(1005)
    out = []
    lo, hi = np.log(1024.0), np.log(1048576.0)
    for i in range(count):
        n = int(np.exp(rng.uniform(lo, hi)) * scale)
        n = max(n, 16)
        d = int(rng.choice([3, 8, 32]))
        k = int(rng.choice([1, 10, 64]))
        q = max(n // 8, 1)
        pts = uniform(rng, n, d)
        qs = uniform(rng, q, d)
        structure = "kd" if d <= 8 else "ball"
        skips = 0 if structure == "kd" else 1
        out.append(Workload(f"c5_set{i}_{structure}{d}_n{n}_k{k}", structure, pts, qs, k, INF,
                            skips))
    return out


def range_limited(scale: float = 1.0, dims: int = 16, structure: str = "kd") -> Workload:
    if not 6 <= dims <= 17:
        raise ValueError("the range-limited test sweeps D = 6..17")
    rng = _rng(1100 + dims)
    n, q = int(500000 * scale), int(10000 * scale)
    skips = {"kd": 3, "ball": 1, "bf": 0}[structure]
    return Workload(f"range_{structure}{dims}_n{n}_q{q}_k5", structure, uniform(rng, n, dims), uniform(rng, q, dims),
                    5, 0.01 * dims, skips)


def functionality(scale: float = 1.0) -> Workload:
    """Shape of the reference's correctness test: D=4, N=100,000, Q=50,000, K=10, radius 5.9."""
    rng = _rng(1000)
    n, q = int(100000 * scale), int(50000 * scale)
    return Workload("functionality_d4", "bf", uniform(rng, n, 4), uniform(rng, q, 4), 10, 5.9, 0)


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4}
