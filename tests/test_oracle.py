"""The CPU oracle against the golden vectors produced by the reference's own CPU classes."""

import numpy as np
import pytest

import oracle
import golden_io

CASES = golden_io.names()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_goldens(name):
    g = golden_io.load(name)
    pts, qs, k, r2 = g["points"], g["queries"], g["k"], g["max_dist2"]
    trees = {}
    by_tag = {r["tag"]: r for r in g["runs"]}
    for run in g["runs"]:
        kind, skips, heap, fma = run["kind"], run["skips"], bool(run["heap"]), bool(run["fma"])
        if fma:
            # The contracted build of the reference fuses `acc += d*d` only where the host
            # compiler chose to (it does at D <= 16; at D = 32 and 128 it vectorises the product
            # instead).  Where that build came out identical to the plain one, it is plain
            # arithmetic and is compared with the oracle's plain mode.
            twin = by_tag[run["tag"][:-1] + "0"]
            if np.array_equal(twin["dist"].view(np.uint32), run["dist"].view(np.uint32)) and \
                    np.array_equal(twin["idx"], run["idx"]):
                fma = False
        if kind == "bf":
            idx, dist = oracle.bf_knn(pts, qs, k, r2, heap=heap, fma=fma)
            # Brute force inserts in index order, so even heap order is reproduced exactly.
            assert np.array_equal(idx, run["idx"]), (name, run["tag"])
            assert np.array_equal(dist.view(np.uint32), run["dist"].view(np.uint32)), (name, run["tag"])
            continue
        if run["fma"] and not np.array_equal(by_tag[run["tag"][:-1] + "0"]["idx"], run["idx"]) \
                and name.startswith("ties"):
            # Exact ties plus `>=` pruning make the returned tie members depend on the tree
            # shape, and in the contracted build the shape depends on where the compiler fused
            # the variance sums.  Check what ties cannot change: each row's sorted distances.
            _, want = oracle.split_keys(oracle.row_keys(*oracle.bf_knn(pts, qs, k, r2, fma=True)))
            _, got = oracle.split_keys(oracle.row_keys(run["idx"], run["dist"]))
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (name, run["tag"])
            continue
        key = (kind, skips, fma)
        if key not in trees:
            trees[key] = (oracle.kd_tree(pts, skips) if kind == "kd"
                          else oracle.ball_tree(pts, skips, fma=fma))
        # strict=False restates the reference's `>=` pruning, so ties resolve the same way.
        idx, dist = trees[key].knn(qs, k, r2, heap=heap, fma=fma, strict=False)
        assert np.array_equal(oracle.row_keys(idx, dist), oracle.row_keys(run["idx"], run["dist"])), \
            (name, run["tag"])


@pytest.mark.parametrize("name", CASES)
def test_strict_trees_equal_brute_force(name):
    """With pruning on `bound > k-th` the trees return brute force's key-ordered top-k."""
    g = golden_io.load(name)
    pts, qs, k, r2 = g["points"], g["queries"], g["k"], g["max_dist2"]
    want = oracle.row_keys(*oracle.bf_knn(pts, qs, k, r2))
    for kind in ("kd", "ball"):
        for skips in (0, 1, 3):
            t = oracle.kd_tree(pts, skips) if kind == "kd" else oracle.ball_tree(pts, skips)
            got = oracle.row_keys(*t.knn(qs, k, r2, strict=True))
            assert np.array_equal(got, want), (name, kind, skips)


def test_fma_and_plain_modes_differ_by_few_ulp():
    g = golden_io.load("ball_d16_k32_sub")
    a = g["runs"][-2]  # bf fma0
    b = g["runs"][-1]  # bf fma1
    assert a["tag"].endswith("fma0") and b["tag"].endswith("fma1")
    _, da = oracle.split_keys(oracle.row_keys(a["idx"], a["dist"]))
    _, db = oracle.split_keys(oracle.row_keys(b["idx"], b["dist"]))
    assert oracle.ulp_distance(da, db).max() <= 4


def test_tree_shape_matches_reference_rules():
    # levels = log2Ceil(n) - skips, leaves of 2^skips slots (src/KnnTrees.cuh:84-93,
    # src/KdTree.cuh:56-61); the ball tree forces skips >= 1 (src/BallTree.cuh:124).
    assert oracle.tree_shape(4194304, 0) == (22, 1, (1 << 22) - 1)
    assert oracle.tree_shape(1048576, 1, ball=True) == (19, 2, (1 << 19) - 1)
    assert oracle.tree_shape(1048576, 0, ball=True) == (19, 2, (1 << 19) - 1)
    assert oracle.tree_shape(100000, 3) == (14, 8, (1 << 14) - 1)
    assert oracle.tree_shape(1, 5) == (1, 1, 1)
    assert oracle.tree_shape(3, 4) == (1, 2, 1)


def _round_f32(x):
    """Round an exact rational to the nearest float32 (ties to even)."""
    from fractions import Fraction
    f = np.float32(float(x))  # within one float32 ulp of x
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        err = abs(Fraction(float(c)) - x)
        even = (int(np.array(c, np.float32).view(np.uint32)) & 1) == 0
        if best is None or err < best[0] or (err == best[0] and even):
            best = (err, c)
    return np.float32(best[1])


def _fma_dist2_exact(a, b):
    """acc = fma(t, t, acc) in dimension order, each step rounded once from the exact value."""
    from fractions import Fraction
    acc = np.float32(0.0)
    for x, y in zip(a, b):
        t = np.float32(x) - np.float32(y)  # float32 subtraction, one rounding
        acc = _round_f32(Fraction(float(t)) * Fraction(float(t)) + Fraction(float(acc)))
    return acc


@pytest.mark.parametrize("dims", [1, 3, 16, 32, 128])
def test_oracle_fma_mode_is_a_single_rounding_per_step(dims):
    rng = np.random.default_rng(dims)
    for _ in range(40):
        a = rng.standard_normal(dims).astype(np.float32)
        b = rng.standard_normal(dims).astype(np.float32)
        want = _fma_dist2_exact(a, b)
        got = np.float32(oracle.dist2(a, b, fma=True))
        assert got.view(np.uint32) == want.view(np.uint32)


def test_radius_model_reference_gradient_is_consistent():
    """The float64 model restatement (the checker of the GPU kernels) against central differences."""
    import radius_model_ref as ref
    rng = np.random.default_rng(0)
    d = 3
    e = d + 64
    n = 64 * e + 64 + 64 * 64 + 64 + 64 + 1
    p = np.zeros(n + 32 * d + 2 * d + 1)
    p[:n] = rng.standard_normal(n) * 0.2
    p[n:n + 32 * d] = rng.standard_normal(32 * d) * 4
    p[n + 33 * d:n + 34 * d] = 0.5
    x = rng.standard_normal((50, d))
    t = rng.standard_normal(50)
    _, g = ref.loss_and_grad(p, d, x, t)
    for i in rng.choice(len(g), size=30, replace=False):
        h = np.zeros_like(p)
        h[i] = 1e-5
        num = (ref.loss_and_grad(p + h, d, x, t)[0] - ref.loss_and_grad(p - h, d, x, t)[0]) / 2e-5
        assert abs(g[i] - num) <= 1e-6 * max(1.0, abs(num))


REF_PAIRS = [(1, 4), (2, 5), (3, 1), (3, 8), (3, 16), (4, 10), (5, 10), (8, 5), (8, 10), (16, 32), (32, 64)]


@pytest.mark.parametrize("dims,k", REF_PAIRS)
@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_matches_the_reference_build_on_fresh_seeds(dims, k, seed):
    """Beyond the committed vectors: the reference's own CPU classes (oracle/_ref, built from its
    sources where they are mounted) and the restatement agree on fresh seeded data, every
    structure, several depthSkips, both tracking modes, with and without a radius.  Skipped where
    oracle/_ref is absent (it is built for this machine only)."""
    if not (oracle.ref_available(False) and oracle.ref_available(True)):
        pytest.skip("oracle/_ref not built on this machine")
    rng = np.random.default_rng(seed * 1000 + dims * 10 + k)
    n = int(rng.integers(k, 3000))
    if seed % 2:
        pts = rng.random((n, dims), dtype=np.float32)
        qs = rng.random((200, dims), dtype=np.float32)
    else:
        centres = rng.random((8, dims))
        pts = (centres[rng.integers(0, 8, n)] + 0.02 * rng.standard_normal((n, dims))).astype(np.float32)
        qs = (centres[rng.integers(0, 8, 200)] + 0.02 * rng.standard_normal((200, dims))).astype(np.float32)
    r2_small = float(np.float32(0.05 * dims * (0.02 if seed % 2 == 0 else 0.2)))
    for r2 in (float("inf"), r2_small):
        for kind, skips_list in (("bf", (0,)), ("kd", (0, 2)), ("ball", (1, 3))):
            for skips in skips_list:
                for heap in (False, True):
                    plain = oracle.ref_knn(kind, pts, qs, k, r2, skips, heap, fma=False)
                    fused = oracle.ref_knn(kind, pts, qs, k, r2, skips, heap, fma=True)
                    for ref_fma, (ri, rd) in ((False, plain), (True, fused)):
                        # Where the contracted build came out identical to the plain one, the
                        # host compiler did not fuse it: compare with the plain arithmetic.
                        fma = ref_fma and not (np.array_equal(ri, plain[0]) and
                                               np.array_equal(rd.view(np.uint32), plain[1].view(np.uint32)))
                        if kind == "bf":
                            oi, od = oracle.bf_knn(pts, qs, k, r2, heap=heap, fma=fma)
                            assert np.array_equal(oi, ri), (kind, r2, heap, ref_fma)
                            assert np.array_equal(od.view(np.uint32), rd.view(np.uint32)), (kind, r2, heap, ref_fma)
                            continue
                        t = oracle.kd_tree(pts, skips) if kind == "kd" else oracle.ball_tree(pts, skips, fma=fma)
                        got = t.knn(qs, k, r2, heap=heap, fma=fma, strict=False)
                        assert np.array_equal(oracle.row_keys(*got), oracle.row_keys(ri, rd)), \
                            (kind, skips, r2, heap, ref_fma)
