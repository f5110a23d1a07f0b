"""The probe's table slots for rows without a carried hash come from a multiplicative mix of
the key (`table_slot` in csrc/vj_join_kernels.cuh): x = key words as a 64-bit word,
x ^= x >> 32, slot = top 14 bits of x * 0x9e3779b97f4a7c15, masked to the table size. This
restates that rule in numpy and checks that key sets whose differences sit in few bits
still spread over a table's slots (a 2048-row item at 8 slots a row), so the probe's
linear-probing walks stay short. Correctness does not depend on it (the GPU tests compare
every join with the oracle); the probe's speed does."""
from __future__ import annotations

import numpy as np
import pytest

C = np.uint64(0x9E3779B97F4A7C15)


def slots(keys: np.ndarray, cap: int) -> np.ndarray:
    x = keys.astype(np.uint64)
    x = x ^ (x >> np.uint64(32))
    with np.errstate(over="ignore"):
        m = x * C
    return ((m >> np.uint64(50)) & np.uint64(cap - 1)).astype(np.int64)


def longest_run(occupied: np.ndarray) -> int:
    # longest stretch of consecutive occupied slots, wrapping around
    occ = np.concatenate([occupied, occupied])
    best = cur = 0
    for v in occ:
        cur = cur + 1 if v else 0
        best = max(best, cur)
    return min(best, occupied.size)


PATTERNS = {
    "sequential": lambda i: i,
    "high_word": lambda i: i << np.uint64(32),
    "equal_halves": lambda i: (i << np.uint64(32)) | i,
    "top_bits": lambda i: i << np.uint64(50),
    "stride_2p20": lambda i: i << np.uint64(20),
    "random": lambda i: np.random.default_rng(1).integers(0, 2**63, size=i.size, dtype=np.int64).astype(np.uint64),
}


@pytest.mark.parametrize("name", sorted(PATTERNS))
def test_patterned_keys_spread_over_a_table(name):
    n, cap = 2048, 2048 * 8
    keys = PATTERNS[name](np.arange(1, n + 1, dtype=np.uint64))
    s = slots(keys, cap)
    counts = np.bincount(s, minlength=cap)
    # 2048 keys over 16384 slots: a random spread puts at most 3-4 keys in any one slot
    assert counts.max() <= 4, (name, int(counts.max()))
    assert np.count_nonzero(counts) >= 0.9 * n, (name, int(np.count_nonzero(counts)))
    # linear probing: no long clusters at load 1/8
    assert longest_run(counts > 0) <= 12, name


def test_fold_is_a_bijection_on_two_words():
    # x -> x ^ (x >> 32) keeps the high word and xors it into the low one: distinct keys stay
    # distinct before the multiply (an odd multiplier is a bijection too)
    rng = np.random.default_rng(7)
    x = rng.integers(0, 2**63, size=100_000, dtype=np.int64).astype(np.uint64)
    y = x ^ (x >> np.uint64(32))
    assert np.unique(y).size == np.unique(x).size
    back = y ^ (y >> np.uint64(32))
    assert np.array_equal(back, x)
