"""vj_partition_noalloc: the radix pass for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: an engine that has given all of HBM to its own buffer
pool, or one that cannot let a cudaFree synchronise a device its other streams are using.
vj_partition_noalloc serves them: it takes no context, and the pass's working memory is a
static device array of VJ_NOALLOC_SCRATCH_BYTES instead of a context workspace.

The GPU test first makes an empty call (rows = 0), the warm-up such a caller makes before
its pool takes the device's memory: it places the library's module and static array on the
device. It then calls the entry point through the C ABI twice in a row, with different
layouts and bucket counts, so that the second call starts on the scratch contents the first
call left behind, and checks that neither call made an allocation (the library's own
allocation counter). Each result must equal what vj_partition (the context entry point)
gives for the same input: the same histogram and offsets, exactly, and each bucket holding
the same rows (the order inside a bucket is unspecified for both). This file is named to be
collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

SCRATCH_BYTES = 4 << 20  # VJ_NOALLOC_SCRATCH_BYTES
MAX_RADIX_BITS = 10  # VJ_NOALLOC_MAX_RADIX_BITS


def _dev(a, d):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64) if a.itemsize == 8 else a.view(np.int32)).to(d)


def _run(vjlib, ctx, cuda, keys, pay, hashes, hash_bits, shift, bits, noalloc):
    """One partition of (keys, pay[, hashes]) by vj_partition_noalloc or vj_partition."""
    import torch

    n = pay.size
    kw = keys.itemsize // 4 * (keys.shape[1] if keys.ndim > 1 else 1)
    dk, dp = _dev(keys, cuda), _dev(pay, cuda)
    ok, op = torch.zeros_like(dk), torch.zeros_like(dp)
    dh = _dev(hashes, cuda) if hashes is not None else None
    oh = torch.zeros_like(dh) if dh is not None else None
    bins = 1 << bits
    d_hist = torch.zeros(bins, dtype=torch.int64, device=cuda)
    d_off = torch.zeros(bins, dtype=torch.int64, device=cuda)
    h_hist = np.zeros(bins, np.uint64)
    h_off = np.zeros(bins, np.uint64)
    t = vjlib.table(dk, dp, n, kw, pay.itemsize)
    kwargs = dict(hashes_in=dh, hash_bits=hash_bits, hash_algo=0, hashes_out=oh, d_hist=d_hist, d_off=d_off, h_hist=h_hist, h_off=h_off)
    if noalloc:
        vjlib.partition_noalloc(t, ok, op, shift, bits, **kwargs)
    else:
        ctx.partition(t, ok, op, shift, bits, **kwargs)
    torch.cuda.synchronize()
    return {
        "h_hist": h_hist,
        "h_off": h_off,
        "d_hist": d_hist.cpu().numpy().view(np.uint64),
        "d_off": d_off.cpu().numpy().view(np.uint64),
        "keys": ok.cpu().numpy().view(keys.dtype).reshape(n, -1),
        "pay": op.cpu().numpy().view(pay.dtype),
        "hashes": oh.cpu().numpy().view(hashes.dtype) if oh is not None else None,
    }


def _same_partition(got, want, bits):
    # histogram and offsets: exact, on the host and on the device
    for k in ("h_hist", "h_off", "d_hist", "d_off"):
        assert np.array_equal(got[k], want[k]), k
    assert np.array_equal(got["h_hist"], got["d_hist"])
    # each bucket holds the same rows: sort both outputs by (bucket of the slot, payload)
    bucket_of_slot = np.repeat(np.arange(1 << bits), want["h_hist"].astype(np.int64))
    go = np.lexsort((got["pay"], bucket_of_slot))
    wo = np.lexsort((want["pay"], bucket_of_slot))
    assert np.array_equal(got["pay"][go], want["pay"][wo])
    assert np.array_equal(got["keys"][go], want["keys"][wo])
    if want["hashes"] is not None:
        assert np.array_equal(got["hashes"][go], want["hashes"][wo])


@pytest.mark.gpu
def test_noalloc_partition_matches_context_partition_twice(vjlib, ctx, cuda):
    import torch

    rng = np.random.default_rng(20261203)
    # warm-up: an empty table
    empty = torch.zeros(1, dtype=torch.int64, device=cuda)
    warm_hist = np.full(4, 7, np.uint64)
    vjlib.partition_noalloc(vjlib.table(empty, empty, 0, 2, 8), empty, empty, 0, 2, h_hist=warm_hist)
    assert warm_hist.tolist() == [0, 0, 0, 0]
    allocations = vjlib.allocation_count()
    # first call: 2^20 + 3 rows of one u64 key, FNV-1a recomputed from the keys, the most
    # buckets the scratch holds (so it runs with fewer work units than vj_partition)
    n1 = (1 << 20) + 3
    keys1 = rng.integers(0, 2**64, size=n1, dtype=np.uint64)
    pay1 = rng.permutation(n1).astype(np.uint64)
    first = _run(vjlib, ctx, cuda, keys1, pay1, None, 64, 3, MAX_RADIX_BITS, noalloc=True)
    # second call, straight after: another layout (two u64 key words, given u32 hashes moved
    # with their rows) and fewer buckets, on the scratch the first call left
    n2 = 70_001
    keys2 = rng.integers(0, 2**64, size=(n2, 2), dtype=np.uint64)
    pay2 = rng.permutation(n2).astype(np.uint64)
    h2 = rng.integers(0, 2**32, size=n2, dtype=np.uint64).astype(np.uint32)
    second = _run(vjlib, ctx, cuda, keys2, pay2, h2, 32, 5, 7, noalloc=True)
    assert vjlib.allocation_count() == allocations, "vj_partition_noalloc allocated"

    _same_partition(first, _run(vjlib, ctx, cuda, keys1, pay1, None, 64, 3, MAX_RADIX_BITS, noalloc=False), MAX_RADIX_BITS)
    _same_partition(second, _run(vjlib, ctx, cuda, keys2, pay2, h2, 32, 5, 7, noalloc=False), 7)
    assert int(first["h_hist"].sum()) == n1 and int(second["h_hist"].sum()) == n2


def test_noalloc_partition_rejects_more_buckets_than_its_scratch_holds(vjlib):
    # checked before any CUDA call, so this needs no GPU
    lib = vjlib.load()
    t = vjlib.VjTable(None, None, 0, 2, 8)
    h = (ctypes.c_uint64 * 4096)()
    st = lib.vj_partition_noalloc(ctypes.byref(t), None, 64, 0, None, None, None, 0, MAX_RADIX_BITS + 1, None, None, h, h, None)
    assert st == vjlib.VJ_ERR_UNSUPPORTED
    msg = vjlib.last_error()
    assert "static scratch" in msg and str(SCRATCH_BYTES) in msg
    assert lib.vj_partition_noalloc(None, None, 64, 0, None, None, None, 0, 4, None, None, None, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
