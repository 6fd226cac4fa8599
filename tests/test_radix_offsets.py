"""The radix sort's scatter offsets (csrc/primitives.cu: radix_sort_pairs, radix_scatter_kernel),
restated on the CPU: per-digit exclusive scans over the blocks' digit counts (one row per digit),
plus, in each block, the keys of all smaller digits from the rows' totals, equal the exclusive
scan of the digit-major count matrix that one serial scan used to give, and every block's
destinations for every digit stay within [0, n)."""

import numpy as np
import pytest

TILE = 4096  # keys per sort block (kSortTile)


@pytest.mark.parametrize("n", [1, 5, 4095, 4096, 4097, 100_000, 1 << 20])
@pytest.mark.parametrize("shift", [0, 8, 24])
def test_per_digit_scans_give_the_serial_offsets(n, shift):
    rng = np.random.default_rng(n + shift)
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    nb = (n + TILE - 1) // TILE
    digit = (keys >> np.uint32(shift)) & np.uint32(255)
    counts = np.zeros((256, nb), dtype=np.int64)  # counts[digit * nblocks + block]
    for b in range(nb):
        counts[:, b] = np.bincount(digit[b * TILE:(b + 1) * TILE], minlength=256)
    flat = counts.reshape(-1)
    serial = (np.cumsum(flat) - flat).reshape(256, nb)
    rows = np.cumsum(counts, axis=1) - counts            # one exclusive scan per digit row
    totals = rows[:, nb - 1] + counts[:, nb - 1]          # a digit's keys in the whole pass
    smaller = np.cumsum(totals) - totals                  # each block's 256-value scan
    assert np.array_equal(smaller[:, None] + rows, serial)
    assert ((serial + counts) <= n).all() and (serial >= 0).all()
