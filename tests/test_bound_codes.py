"""The tensor-core filter's running k-th bound in its buffered-codes form (csrc/bf_tc.cu:
bound_code, put_code and the flush in tc_filter_kernel), restated on the CPU for one query row.

The filter may only drop a point whose lower bound exceeds the bound T, so T must never undercut
the k-th smallest upper bound recorded so far (or the query's seed, which bounds it by
assumption); to keep few candidates it should also stay close to it.  For every order of the
recorded values, ties, saturating codes, rows whose buffer is full, and an infinite starting bound:
after each flush, at least k recorded values lie at or below T (validity), and with nothing
dropped and a finite start T lies within one code unit (2^13 float bits, at most 2^-10 relative)
above the k-th smallest value recorded (tightness)."""

import numpy as np
import pytest

SHIFT = 13  # the code unit in float bits (kCodeShift)


def bits(x) -> int:
    return int(np.float32(x).view(np.uint32))


def flt(b: int) -> np.float32:
    return np.uint32(b).view(np.float32)


class Row:
    """One query row: its bound T, its buffered codes, and (while T is infinite) the largest
    buffered value."""

    def __init__(self, k: int, capacity: int, seed: float):
        self.k, self.cap, self.T = k, capacity, np.float32(seed)
        self.codes: list[int] = []
        self.umax = 0

    def record(self, u: np.float32) -> None:
        if not u < self.T:
            return  # not a candidate for the k nearest: the filter records no code
        if len(self.codes) >= self.cap:
            return  # a full buffer drops the value (T stays valid, only less tight)
        if not np.isfinite(self.T):
            self.umax = max(self.umax, bits(u))
        self.codes.append(min((bits(self.T) - bits(u)) >> SHIFT, 0xFFFF))

    def flush(self) -> None:
        if len(self.codes) < self.k:
            self.codes = [c for c in self.codes if c >= 1]  # (codes 0 make room)
            return
        if not np.isfinite(self.T):
            self.T, self.codes = flt(self.umax), []
            return
        top, cstar = max(self.codes), 0
        for bit in range(top.bit_length() - 1, -1, -1):
            cand = cstar | (1 << bit)
            if sum(c >= cand for c in self.codes) >= self.k:
                cstar = cand
        keep = max(cstar, 1)
        self.codes = [c - cstar for c in self.codes if c >= keep]
        if cstar:
            self.T = flt(bits(self.T) - (cstar << SHIFT))


def run(values, k, capacity, seed, step):
    """Records the values in order, flushing once k codes are buffered and then every `step`
    codes; checks validity (and returns the rows' history for tightness checks)."""
    row = Row(k, capacity, seed)
    seen: list[float] = []
    due = k
    out = []
    for v in values:
        v = np.float32(v)
        seen.append(float(v))
        row.record(v)
        if len(row.codes) >= due:
            row.flush()
            due = max(k, len(row.codes) + step)
            s = np.sort(np.asarray(seen, dtype=np.float32))
            if np.isfinite(row.T) and row.T != np.float32(seed):
                assert np.count_nonzero(s <= row.T) >= k, "T undercuts the k-th smallest value seen"
            out.append((row.T, s[k - 1] if len(s) >= k else None))
    return out


@pytest.mark.parametrize("k", [1, 10, 100, 128])
@pytest.mark.parametrize("dist", ["lognormal", "uniform", "clustered"])
def test_flushed_bound_is_valid_and_tight(k, dist):
    rng = np.random.default_rng(k * 7 + len(dist))
    n = 4000
    if dist == "lognormal":
        vals = rng.lognormal(0.0, 1.0, n)
    elif dist == "uniform":
        vals = rng.uniform(1.0, 2.0, n)
    else:
        vals = np.concatenate([rng.normal(5.0, 0.01, n // 2), rng.normal(1.0, 0.001, n // 2)])
        rng.shuffle(vals)
    vals = np.abs(vals).astype(np.float32)
    seed = float(vals.max()) * 4.0
    for t, kth in run(vals, k, capacity=10 * n, seed=seed, step=max(16, k // 4)):
        assert t >= kth
        # one code unit at most above the k-th smallest value (the first flushes may saturate:
        # a seed far above the data puts them more than 2^16 units below it)
        if bits(seed) - bits(kth) < (0xFFFF << SHIFT):
            assert bits(t) - bits(kth) < (1 << SHIFT), (t, kth)


def test_ties_and_full_buffers_stay_valid():
    rng = np.random.default_rng(3)
    vals = rng.integers(1, 4, size=3000).astype(np.float32)  # many exact ties
    for k in (1, 32, 128):
        for t, kth in run(vals, k, capacity=k + 48, seed=10.0, step=16):
            assert t >= kth


def test_infinite_seed_takes_the_largest_buffered_value():
    """Codes relative to an infinite bound all saturate: the first flush takes the largest value
    buffered (at least k lie at or below it) and starts the buffer again, so later flushes tighten
    T from the values recorded after it (valid throughout, tight only as those accumulate)."""
    rng = np.random.default_rng(4)
    vals = rng.lognormal(0.0, 2.0, 2000).astype(np.float32)
    k = 50
    hist = run(vals, k, capacity=4000, seed=np.inf, step=16)
    assert hist and all(np.isfinite(t) for t, _ in hist)
    assert hist[0][0] == np.float32(vals[:k].max())  # the first flush, at exactly k values
    for t, kth in hist:
        assert t >= kth
    assert hist[-1][0] < hist[0][0] / 4
