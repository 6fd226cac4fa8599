"""The tensor-core filter's GEMM error bound, checked on the CPU against emulated 16-bit GEMMs.

The filter keeps a point only if its tensor-core dot product G could put it among a query's k
nearest, with |G - q'.p'| <= E = c1 |q'||p'| + c3 (|q'| + |p'|) + c4 (the derivation in the
header comment of cudaexactknn_gb300/csrc/bf_tc.cu; constants as make_bounds there builds them):
  c1 = (2u + u^2 + D 2^-20 (1+u)^2)(1 + 2^-10),  c3 = 1.01 delta (1+u) sqrt(D),  c4 = 1.01 D delta^2,
u the format's unit roundoff, delta its largest absolute rounding error in the subnormal range.
If E were too small, the filter could drop a true neighbour; the GPU tests catch that only when
it happens on their data.  Here the bound is checked directly: the operands are scaled and rounded
as the engine does (largest |coordinate| scaled into [2^13, 2^14), FP16 with subnormals; BF16
unscaled for data beyond FP16's range), every
product is exact, and the FP32 accumulation runs in several orders, including truncating every
addition, which is more error than the hardware's accumulator makes.  The exact dot product of
the scaled FP32 vectors is math.fsum of exact float64 products."""

import math

import numpy as np
import pytest

U16 = 2.0 ** -11
DELTA16 = 2.0 ** -14
UBF16 = 2.0 ** -8
DELTABF16 = 2.0 ** -100


def constants(dims, u=U16, delta=DELTA16):
    c1 = (2 * u + u * u + dims * 2.0 ** -20 * (1 + u) ** 2) * (1 + 2.0 ** -10)
    c3 = 1.01 * delta * (1 + u) * math.sqrt(dims)
    c4 = 1.01 * dims * delta * delta
    return np.float32(c1), np.float32(c3), np.float32(c4)


def scale_exponent(x):
    """e >= 0 with the largest |coordinate| * 2^e in [2^13, 2^14) (e = 0 if already above)."""
    m = float(np.abs(x).max())
    if m == 0.0:
        return 0
    e = 13 - math.floor(math.log2(m))
    return max(e, 0)


def to_f32_trunc(x):
    """float64 -> float32 rounded toward zero."""
    f = np.float32(x)
    if abs(float(f)) > abs(x):
        f = np.nextafter(f, np.float32(0.0))
    return f


def accumulate(products, order):
    """FP32 sum of exact float64 products in a given order and rounding."""
    p = list(products)
    if order == "reverse":
        p = p[::-1]
    if order in ("sequential", "reverse"):
        acc = np.float32(0.0)
        for v in p:
            acc = np.float32(float(acc) + v)  # float64 sum of two exact values, one rounding
        return float(acc)
    if order == "truncate":
        acc = np.float32(0.0)
        for v in p:
            acc = to_f32_trunc(float(acc) + v)
        return float(acc)
    if order == "pairwise":
        vals = [np.float32(v) for v in p]
        while len(vals) > 1:
            vals = [np.float32(float(vals[i]) + float(vals[i + 1])) if i + 1 < len(vals) else vals[i]
                    for i in range(0, len(vals), 2)]
        return float(vals[0])
    if order == "k16_truncate":
        # Each K step of 16 products summed exactly, then added into the accumulator truncating.
        acc = np.float32(0.0)
        for i in range(0, len(p), 16):
            acc = to_f32_trunc(float(acc) + math.fsum(p[i:i + 16]))
        return float(acc)
    raise ValueError(order)


ORDERS = ["sequential", "reverse", "truncate", "pairwise", "k16_truncate"]


def to_bf16(x):
    """float32 -> bfloat16 (round to nearest even), returned as float64."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def check_pair(q, p, dims, data_max=0.0):
    """Largest |G - q'.p'| / E over the accumulation orders, for one scaled pair (the scale set
    by the largest |coordinate| of the pair and of the rest of the data, `data_max`).  Data whose
    largest |coordinate| exceeds 2^14 goes to BF16 unscaled, as in the engine."""
    e = scale_exponent(np.concatenate([q, p, [data_max]]))
    qs = (q.astype(np.float32) * np.float32(2.0 ** e)).astype(np.float32)
    ps = (p.astype(np.float32) * np.float32(2.0 ** e)).astype(np.float32)
    bf16 = max(np.abs(qs).max(), np.abs(ps).max(), data_max) >= 2 ** 14
    if bf16:
        assert e == 0
        qh, ph = to_bf16(qs), to_bf16(ps)
        c1, c3, c4 = (float(c) for c in constants(dims, UBF16, DELTABF16))
    else:
        qh = qs.astype(np.float16).astype(np.float64)
        ph = ps.astype(np.float16).astype(np.float64)
        c1, c3, c4 = (float(c) for c in constants(dims))
    prods = qh * ph  # exact: 11-bit (or 8-bit) significands
    exact = math.fsum(qs.astype(np.float64) * ps.astype(np.float64))
    nq = math.sqrt(math.fsum(qs.astype(np.float64) ** 2))
    npn = math.sqrt(math.fsum(ps.astype(np.float64) ** 2))
    bound = c1 * nq * npn + c3 * (nq + npn) + c4
    worst = 0.0
    for order in ORDERS:
        g = accumulate(prods, order)
        worst = max(worst, abs(g - exact) / bound)
    return worst


def _cases(rng, dims):
    yield "gaussian", rng.standard_normal(dims), rng.standard_normal(dims), 0.0
    q = rng.standard_normal(dims)
    yield "near neighbour", q, q + 1e-3 * rng.standard_normal(dims), 0.0
    # Cancellation: a large dot product of alternating signs that sums to almost nothing.
    a = rng.uniform(0.5, 1.0, dims)
    b = a * np.where(np.arange(dims) % 2 == 0, 1.0, -1.0)
    yield "cancellation", a, b, 0.0
    # One large coordinate sets the scale (2^13); the rest fall into FP16's subnormal range
    # (below 2^-14 once scaled).
    q = rng.standard_normal(dims) * 1e-9
    q[0] = 1.0
    p = rng.standard_normal(dims) * 1e-9
    p[-1] = -1.0
    yield "subnormal tail", q, p, 0.0
    # Both vectors tiny beside the data's largest coordinate (1.0): every element subnormal.
    yield "subnormal vectors", rng.standard_normal(dims) * 2e-9, rng.standard_normal(dims) * 2e-9, 1.0
    # Coordinates at FP16 rounding midpoints after scaling (worst rounding of every element).
    k = rng.integers(2 ** 10, 2 ** 11, dims)
    q = (k + 0.5) * 2.0 ** 3
    q[0] = 2.0 ** 13 + 2.0 ** 2
    p = (rng.integers(2 ** 10, 2 ** 11, dims) + 0.5) * 2.0 ** 3
    yield "midpoints", q / 2 ** 14, p / 2 ** 14, 0.0
    # Beyond FP16's range: BF16 without scaling.
    yield "bf16 wide", rng.standard_normal(dims) * 1e6, rng.standard_normal(dims) * 1e6, 0.0
    q = rng.standard_normal(dims) * 1e6
    yield "bf16 near neighbour", q, q + 10.0 * rng.standard_normal(dims), 0.0


@pytest.mark.parametrize("dims", [3, 16, 17, 32, 64, 100, 128])
def test_gemm_error_bound_holds(dims):
    rng = np.random.default_rng(dims)
    worst = {}
    for _ in range(12):
        for name, q, p, data_max in _cases(rng, dims):
            worst[name] = max(worst.get(name, 0.0),
                              check_pair(q.astype(np.float32), p.astype(np.float32), dims, data_max))
    assert max(worst.values()) <= 1.0, worst


def test_bound_is_not_loose_by_orders_of_magnitude():
    """The bound keeps few extra candidates only if it is near the real error: on midpoint data
    (every product rounded the most) at 128 dims, the real error reaches a fair share of it."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(40):
        for name, q, p, _ in _cases(rng, 128):
            if name == "midpoints":
                worst = max(worst, check_pair(q.astype(np.float32), p.astype(np.float32), 128))
    assert 0.01 < worst <= 1.0
