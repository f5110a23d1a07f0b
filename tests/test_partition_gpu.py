"""vj_partition (partition_gpu) on the GPU against the oracle: exact histogram and offsets,
each bucket holding the same multiset of rows, hashes moved with their rows."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, d):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64) if a.itemsize == 8 else a.view(np.int32)).to(d)


def check_partition(vjlib, ctx, oracle, cuda, keys, pay, hashes, shift, bits, hash_algo=0, hash_bits=64):
    import torch

    n = pay.size
    kw = keys.itemsize // 4 * (keys.shape[1] if keys.ndim > 1 else 1)
    pb = pay.itemsize
    dk, dp = dev(keys, cuda), dev(pay, cuda)
    ok = torch.zeros_like(dk)
    op = torch.zeros_like(dp)
    dh = dev(hashes, cuda) if hashes is not None else None
    oh = torch.zeros_like(dh) if dh is not None else None
    bins = 1 << bits
    hh = np.zeros(bins, np.uint64)
    ho = np.zeros(bins, np.uint64)
    t = vjlib.table(dk, dp, n, kw, pb)
    ctx.partition(t, ok, op, shift, bits, hashes_in=dh, hash_bits=hash_bits, hash_algo=hash_algo, hashes_out=oh, h_hist=hh, h_off=ho)
    torch.cuda.synchronize()
    if hashes is None:
        words = np.ascontiguousarray(keys).view(np.uint32).reshape(n, kw) if n else np.zeros((0, kw), np.uint32)
        hv, _ = oracle.hash_elements(words, n, 0, kw, 32, hash_bits, hash_algo)
    else:
        hv = hashes
    want_hist, want_off, _ = oracle.partition(hv, shift, bits)
    assert np.array_equal(hh, want_hist)
    assert np.array_equal(ho, want_off)
    got_keys = ok.cpu().numpy().view(keys.dtype).reshape(keys.shape)
    got_pay = op.cpu().numpy().view(pay.dtype)
    # every bucket holds exactly its rows: the payloads are row ids, so the row placed at each
    # output position is known, and its bucket must be the bucket whose range holds it
    assert np.array_equal(np.sort(got_pay), np.sort(pay))  # a permutation of the rows
    bucket = ((hv.astype(np.uint64) >> np.uint64(shift)) & np.uint64(bins - 1)) if n else hv
    bucket_of_slot = np.repeat(np.arange(bins, dtype=np.uint64), want_hist.astype(np.int64))
    assert np.array_equal(bucket[got_pay.astype(np.int64)], bucket_of_slot)
    # the whole permutation keeps (key, payload) rows together
    order = np.argsort(pay, kind="stable")
    gorder = np.argsort(got_pay, kind="stable")
    assert np.array_equal(got_keys.reshape(n, -1)[gorder], np.ascontiguousarray(keys).reshape(n, -1)[order])
    if hashes is not None:
        got_h = oh.cpu().numpy().view(hashes.dtype)
        assert np.array_equal(got_h[gorder], hashes[order])


@pytest.mark.parametrize("bits", [1, 4, 8, 11, 12])
def test_partition_recomputed_fnv(vjlib, ctx, oracle, cuda, bits):
    rng = np.random.default_rng(bits)
    n = 300_001
    keys = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    pay = np.arange(n, dtype=np.uint64)
    check_partition(vjlib, ctx, oracle, cuda, keys, pay, None, shift=3, bits=bits)


def test_partition_given_hashes(vjlib, ctx, oracle, cuda):
    rng = np.random.default_rng(1)
    n = 100_000
    keys = rng.integers(0, 2**64, size=(n, 2), dtype=np.uint64)
    pay = np.arange(n, dtype=np.uint64)
    h64 = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    check_partition(vjlib, ctx, oracle, cuda, keys, pay, h64, shift=17, bits=9, hash_bits=64)
    h32 = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    check_partition(vjlib, ctx, oracle, cuda, keys, pay, h32, shift=5, bits=6, hash_bits=32)


def test_partition_int32_keys_and_other_hashes(vjlib, ctx, oracle, cuda):
    rng = np.random.default_rng(2)
    n = 50_000
    keys = rng.integers(0, 2**31, size=n, dtype=np.uint32)
    pay = np.arange(n, dtype=np.uint32)
    for algo, hb in [(0, 32), (3, 64), (10, 32)]:
        check_partition(vjlib, ctx, oracle, cuda, keys, pay, None, shift=0, bits=7, hash_algo=algo, hash_bits=hb)


def test_partition_skewed_and_tiny(vjlib, ctx, oracle, cuda):
    rng = np.random.default_rng(3)
    n = 40_000
    keys = np.where(rng.random(n) < 0.9, np.uint64(7), rng.integers(0, 2**64, size=n, dtype=np.uint64)).astype(np.uint64)
    pay = np.arange(n, dtype=np.uint64)
    check_partition(vjlib, ctx, oracle, cuda, keys, pay, None, shift=0, bits=8)
    for n in (1, 2, 255):
        check_partition(vjlib, ctx, oracle, cuda, keys[:n].copy(), pay[:n].copy(), None, shift=0, bits=4)
