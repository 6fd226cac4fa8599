"""The ball tree's pruning bound, restated with exact directed rounding and checked on the CPU.

The ball search skips a ball when its lower bound exceeds the current k-th distance, so the bound
must never exceed the float distance (the reference's sequential fused sum) from the query to
any point of the ball.  The device functions (cudaexactknn_gb300/csrc/knn_common.cuh):
  radius  r = sqrt_ru(m *ru (1 + margin))          m = largest float dist2(centre, point)
  bound     s_lo = s *rd (1 - margin), dq = sqrt_rd(s_lo), gap = dq -rd r,
            b = gap *rd gap, bound = b *rd (1 - margin)   (0 when gap <= 0)
with s the float dist2(query, centre) and margin = (D + 4) 2^-23.  Here every directed-rounding
step is computed exactly (Python fractions) and rounded to float32 in the stated direction; the
float distances come from the oracle's fused mode, the engine's own arithmetic."""

from fractions import Fraction

import numpy as np
import pytest

import oracle


def _f32_down(x: Fraction) -> np.float32:
    f = np.float32(float(x))
    while Fraction(float(f)) > x:
        f = np.nextafter(f, np.float32(-np.inf))
    while Fraction(float(np.nextafter(f, np.float32(np.inf)))) <= x:
        f = np.nextafter(f, np.float32(np.inf))
    return f


def _f32_up(x: Fraction) -> np.float32:
    f = np.float32(float(x))
    while Fraction(float(f)) < x:
        f = np.nextafter(f, np.float32(np.inf))
    while Fraction(float(np.nextafter(f, np.float32(-np.inf)))) >= x:
        f = np.nextafter(f, np.float32(-np.inf))
    return f


def _sqrt_down(x: np.float32) -> np.float32:
    f = np.float32(np.sqrt(np.float64(x)))
    fx = Fraction(float(x))
    while Fraction(float(f)) ** 2 > fx:
        f = np.nextafter(f, np.float32(-np.inf))
    while Fraction(float(np.nextafter(f, np.float32(np.inf)))) ** 2 <= fx:
        f = np.nextafter(f, np.float32(np.inf))
    return f


def _sqrt_up(x: np.float32) -> np.float32:
    f = np.float32(np.sqrt(np.float64(x)))
    fx = Fraction(float(x))
    while Fraction(float(f)) ** 2 < fx:
        f = np.nextafter(f, np.float32(np.inf))
    while Fraction(float(np.nextafter(f, np.float32(-np.inf)))) ** 2 >= fx:
        f = np.nextafter(f, np.float32(-np.inf))
    return f


def margin(dims):
    return np.float32(np.float32(dims + 4) * np.float32(1.1920928955078125e-07))


def ball_radius(m, marg):
    prod = _f32_up(Fraction(float(m)) * Fraction(float(np.float32(1.0) + marg)))
    return _sqrt_up(prod)


def ball_bound(s, r, marg):
    one_m = Fraction(float(np.float32(1.0) - marg))
    s_lo = _f32_down(Fraction(float(s)) * one_m)
    dq = _sqrt_down(s_lo)
    gap = _f32_down(Fraction(float(dq)) - Fraction(float(r)))
    if not gap > 0:
        return np.float32(0.0)
    b = _f32_down(Fraction(float(gap)) ** 2)
    return _f32_down(Fraction(float(b)) * one_m)


def _check_ball(points, centre, queries):
    dims = points.shape[1]
    marg = margin(dims)
    m = max(np.float32(oracle.dist2(centre, p, fma=True)) for p in points)
    r = ball_radius(m, marg)
    worst = 0.0
    for q in queries:
        bound = ball_bound(np.float32(oracle.dist2(q, centre, fma=True)), r, marg)
        nearest = min(np.float32(oracle.dist2(q, p, fma=True)) for p in points)
        assert bound <= nearest, (bound, nearest)
        if nearest > 0:
            worst = max(worst, float(bound) / float(nearest))
    return worst


@pytest.mark.parametrize("dims", [1, 3, 16, 32, 128])
@pytest.mark.parametrize("scale", [1e-15, 1.0, 1e12])
def test_ball_bound_never_exceeds_a_member_distance(dims, scale):
    rng = np.random.default_rng(dims)
    for _ in range(4):
        pts = (rng.standard_normal((24, dims)) * scale).astype(np.float32)
        centre = pts.mean(axis=0, dtype=np.float64).astype(np.float32)
        # Queries just outside the ball: its farthest point pushed outward by a hair, and random
        # directions at 1.001 to 3 radii from the centre.
        far = pts[np.argmax(((pts - centre) ** 2).sum(1))]
        out = centre + (far - centre) * np.float32(1.0 + 1e-6)
        dirs = rng.standard_normal((12, dims))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        rad = np.sqrt(((pts.astype(np.float64) - centre) ** 2).sum(1).max())
        shells = centre + dirs * rad * rng.uniform(1.001, 3.0, (12, 1))
        queries = np.vstack([out[None, :], shells]).astype(np.float32)
        _check_ball(pts, centre, queries)


def test_ball_bound_is_close_to_the_nearest_member_on_the_far_side():
    """A query on the line through the centre and a member on the ball's surface: the bound
    nearly reaches that member's distance (the margins cost a few ulps, not a loose factor)."""
    dims = 16
    rng = np.random.default_rng(3)
    d = rng.standard_normal(dims)
    d /= np.linalg.norm(d)
    centre = np.zeros(dims, np.float32)
    surface = (d * 1.0).astype(np.float32)
    inner = (rng.standard_normal((10, dims)) * 0.1).astype(np.float32)
    pts = np.vstack([surface[None, :], -surface[None, :], inner])
    q = (d * 3.0).astype(np.float32)[None, :]
    worst = _check_ball(pts, centre, q)
    assert worst > 0.999
