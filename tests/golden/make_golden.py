"""Generate the golden fixtures in this directory from the reference's own CPU classes.

The reference ships no golden vectors or known-answer tests (its only correctness test,
tests/FunctionalityTests.cu, draws unseeded random points and cross-checks implementations).
These fixtures are therefore produced by running the reference's BruteForce / KdTree /
BallTree (src/BruteForce.cuh, src/KdTree.cuh, src/BallTree.cuh), compiled from the reference
sources by oracle/Makefile into oracle/_ref, on small seeded inputs.

Two builds are recorded per case:
  ``fma0``  the reference's CPU code as the x86-64 host compiler builds it (no contraction);
  ``fma1``  the same code with `result += d*d` contracted to a fused multiply-add, which is
            the arithmetic nvcc gives the reference's device code.

Run from the repository root (needs the reference sources, so only where they are mounted):
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cudaexactknn_gb300 import workloads as W  # noqa: E402

INF = float("inf")


def cases():
    rng = np.random.Generator(np.random.PCG64(20240))
    out = []

    # Brute force at the C1 shape, scaled down (D=3, K=8, radius +inf, heap tracking).
    out.append(dict(name="bf_d3_k8", points=W.uniform(rng, 2048, 3), queries=W.uniform(rng, 128, 3),
                    k=8, max_dist2=INF,
                    runs=[("bf", 0, 1), ("bf", 0, 0)]))

    # The reference correctness test's variants (tests/FunctionalityTests.cu:40-107), scaled down.
    out.append(dict(name="func_d4_k10", points=W.uniform(rng, 4000, 4), queries=W.uniform(rng, 256, 4),
                    k=10, max_dist2=5.9,
                    runs=[("bf", 0, 0), ("bf", 0, 1), ("kd", 3, 0), ("kd", 0, 1), ("ball", 3, 0),
                          ("ball", 0, 1)]))

    # k-d tree at the C2 shape (Gaussian mixture, D=3, K=16, depthSkips 0).
    pts, centres = W.mixture(rng, 8192, 3, 64, 0.01)
    qs, _ = W.mixture(rng, 256, 3, 64, 0.01, centres)
    out.append(dict(name="kd_d3_k16_mix", points=pts, queries=qs, k=16, max_dist2=INF,
                    runs=[("kd", 0, 1), ("kd", 0, 0), ("bf", 0, 0)]))

    # Ball tree at the C3 shape (4-dim subspace of R^16 plus noise, K=32, depthSkips 1).
    pts, basis = W.subspace(rng, 4096, 16, 4, 0.05)
    qs, _ = W.subspace(rng, 128, 16, 4, 0.05, basis)
    out.append(dict(name="ball_d16_k32_sub", points=pts, queries=qs, k=32, max_dist2=INF,
                    runs=[("ball", 1, 1), ("ball", 1, 0), ("bf", 0, 0)]))

    # Exact ties and duplicate points: coordinates on an 8-level grid.
    grid = (rng.integers(0, 8, size=(1500, 3)) / 8.0).astype(np.float32)
    qgrid = (rng.integers(0, 8, size=(100, 3)) / 8.0 + 1.0 / 16).astype(np.float32)
    qgrid[:20] = grid[:20]  # some queries sit exactly on points
    out.append(dict(name="ties_d3_k16", points=grid, queries=qgrid, k=16, max_dist2=INF,
                    runs=[("bf", 0, 0), ("bf", 0, 1), ("kd", 0, 0), ("kd", 2, 1), ("ball", 1, 0)]))

    # Range-limited queries (tests/DimXSpeedTests.cu:16-67 uses radius 0.01 * D): some rows
    # keep unfilled slots (index -1, distance = the radius).
    out.append(dict(name="range_d8_k5", points=W.uniform(rng, 3000, 8), queries=W.uniform(rng, 200, 8),
                    k=5, max_dist2=0.08,
                    runs=[("bf", 0, 0), ("kd", 3, 0), ("ball", 1, 1)]))

    # Fewer points than K.
    out.append(dict(name="small_n_d2_k5", points=W.uniform(rng, 3, 2), queries=W.uniform(rng, 10, 2),
                    k=5, max_dist2=INF,
                    runs=[("bf", 0, 0), ("bf", 0, 1), ("kd", 0, 0), ("ball", 1, 1)]))

    # One dimension.
    out.append(dict(name="d1_k4", points=W.uniform(rng, 100, 1), queries=W.uniform(rng, 20, 1),
                    k=4, max_dist2=INF, runs=[("bf", 0, 0), ("kd", 0, 0), ("ball", 1, 0)]))

    # The speed-up benchmark's dimension (tests/SpeedupSpeedTests.cu, D=5, K=10).
    out.append(dict(name="d5_k10", points=W.uniform(rng, 3000, 5), queries=W.uniform(rng, 100, 5),
                    k=10, max_dist2=5.9, runs=[("bf", 0, 0), ("kd", 3, 0), ("ball", 1, 1)]))

    # Ball tree in 32 dimensions with K=64 (the C5 ball-tree sets' shape).
    out.append(dict(name="ball_d32_k64", points=W.uniform(rng, 2000, 32), queries=W.uniform(rng, 48, 32),
                    k=64, max_dist2=INF, runs=[("ball", 1, 0), ("bf", 0, 0)]))

    # K = 1.
    out.append(dict(name="kd_d3_k1", points=W.uniform(rng, 1000, 3), queries=W.uniform(rng, 100, 3),
                    k=1, max_dist2=INF, runs=[("kd", 0, 0), ("bf", 0, 1)]))

    # Brute force at the C4 shape, scaled down (D=128 Gaussian mixture, K=100).
    pts, centres = W.gauss_mix(rng, 512, 128, 16, 0.3)
    qs, _ = W.gauss_mix(rng, 12, 128, 16, 0.3, centres)
    out.append(dict(name="bf_d128_k100", points=pts, queries=qs, k=100, max_dist2=INF,
                    runs=[("bf", 0, 0), ("bf", 0, 1)]))
    return out


def main():
    if not oracle.ref_available(False) or not oracle.ref_available(True):
        raise SystemExit("oracle/_ref is not built; run `make -C oracle` where the reference is mounted")
    for case in cases():
        arrays = {"points": case["points"], "queries": case["queries"]}
        meta = {k: case[k] for k in ("name", "k", "max_dist2")}
        meta["runs"] = []
        for kind, skips, heap in case["runs"]:
            for fma in (0, 1):
                idx, dist = oracle.ref_knn(kind, case["points"], case["queries"], case["k"],
                                           case["max_dist2"], skips, bool(heap), bool(fma))
                tag = f"{kind}_s{skips}_h{heap}_fma{fma}"
                arrays[tag + "_idx"] = idx
                arrays[tag + "_dist"] = dist
                meta["runs"].append(dict(kind=kind, skips=skips, heap=heap, fma=fma, tag=tag))
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        path = os.path.join(HERE, case["name"] + ".npz")
        np.savez_compressed(path, **arrays)
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
