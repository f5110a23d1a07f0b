"""vj_join_host's chunked pipeline (probe side >= 2 x build side and >= 2^23 rows): pairs
from host tables into a host buffer must equal vj_join's on the same rows -- count and
order-independent digest -- for ragged chunk bounds, duplicate keys, 16 chunks, pinned and
pageable host memory, and a capacity that runs out part way."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from test_join_gpu import sort_pairs

pytestmark = pytest.mark.gpu

VJ_ERR_CAPACITY = 5


def device_join(vjlib, ctx, cuda, rk, rp, sk, sp, kw, pb):
    import torch

    drk, drp, dsk, dsp = (torch.from_numpy(a).to(cuda) for a in (rk, rp, sk, sp))
    out = torch.zeros((sk.size * 4 + 1, 2), dtype=torch.int32 if pb == 4 else torch.int64, device=cuda)
    res = ctx.join(vjlib.table(drk, drp, rk.size, kw, pb), vjlib.table(dsk, dsp, sk.size, kw, pb), out=out, capacity=out.shape[0])
    return res.count, vjlib.pairs_digest(out, res.count, pb)


def host_join(vjlib, ctx, cuda, rk, rp, sk, sp, kw, pb, capacity, pinned):
    import torch

    dt = np.uint32 if pb == 4 else np.uint64
    if pinned:
        rk, rp, sk, sp = (torch.from_numpy(a).pin_memory() for a in (rk, rp, sk, sp))
        out = torch.zeros((max(1, capacity), 2), dtype=torch.int32 if pb == 4 else torch.int64).pin_memory()
        host = out.numpy().view(dt)
    else:
        out = np.zeros((max(1, capacity), 2), dt)
        host = out
    n = ctx.join_host(vjlib.table(rk, rp, rk.shape[0], kw, pb), vjlib.table(sk, sp, sk.shape[0], kw, pb), out, capacity)
    return n, host


def digest_of_host(vjlib, cuda, host, n, pb):
    import torch

    t = torch.from_numpy(host[:n].view(np.int32 if pb == 4 else np.int64)).to(cuda)
    return vjlib.pairs_digest(t, n, pb)


@pytest.mark.parametrize("pinned", [True, False])
def test_chunked_unique_keys_ragged(vjlib, ctx, cuda, pinned):
    rng = np.random.default_rng(51)
    nr, ns = 1 << 21, (1 << 23) + 12345  # two chunks of unequal length
    rk = rng.permutation(np.arange(1, 4 * nr, 2, dtype=np.uint64))[:nr].astype(np.uint32)
    sk = rng.integers(0, 4 * nr, size=ns, dtype=np.uint64).astype(np.uint32)
    rp = np.arange(nr, dtype=np.uint32)
    sp = np.arange(ns, dtype=np.uint32)
    want = device_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4)
    n, host = host_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4, ns, pinned)
    assert n == want[0]
    assert digest_of_host(vjlib, cuda, host, n, 4) == want[1]


def test_chunked_duplicates_int64(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(52)
    nr, ns = 1 << 20, (1 << 23) + 777
    rk = rng.integers(0, 1 << 19, size=nr, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15 & ((1 << 63) - 1))
    sk = rng.integers(0, 1 << 19, size=ns, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15 & ((1 << 63) - 1))
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, _, _ = oracle.join(rk, rp, sk, sp)
    want = device_join(vjlib, ctx, cuda, rk, rp, sk, sp, 2, 8)
    assert want[0] == cnt
    n, host = host_join(vjlib, ctx, cuda, rk, rp, sk, sp, 2, 8, cnt, True)
    assert n == cnt
    assert digest_of_host(vjlib, cuda, host, n, 8) == want[1]


def test_chunked_sixteen_chunks(vjlib, ctx, cuda):
    rng = np.random.default_rng(53)
    nr, ns = 1 << 16, 1 << 26
    rk = np.arange(nr, dtype=np.uint32) * np.uint32(7)
    sk = rng.integers(0, 14 * nr, size=ns, dtype=np.uint64).astype(np.uint32)
    rp = np.arange(nr, dtype=np.uint32)
    sp = np.arange(ns, dtype=np.uint32)
    want = device_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4)
    n, host = host_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4, want[0], True)
    assert n == want[0]
    assert digest_of_host(vjlib, cuda, host, n, 4) == want[1]


def test_chunked_capacity_runs_out(vjlib, ctx, cuda):
    """Room for half the pairs: VJ_ERR_CAPACITY with the full count; then the exact count
    fits and the pairs are whole."""
    rng = np.random.default_rng(54)
    nr, ns = 1 << 21, 1 << 23
    rk = np.arange(nr, dtype=np.uint32)
    sk = rng.integers(0, 2 * nr, size=ns, dtype=np.uint64).astype(np.uint32)
    rp = np.arange(nr, dtype=np.uint32)
    sp = np.arange(ns, dtype=np.uint32)
    want = device_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4)
    half = want[0] // 2
    out = np.zeros((half, 2), np.uint32)
    need = ctypes.c_uint64(0)
    r = vjlib.table(rk, rp, nr, 1, 4)
    s = vjlib.table(sk, sp, ns, 1, 4)
    st = ctx.lib.vj_join_host(ctx.handle, ctypes.byref(r), ctypes.byref(s), None, out.ctypes.data_as(ctypes.c_void_p), half, ctypes.byref(need), None)
    assert st == VJ_ERR_CAPACITY
    assert need.value == want[0]
    n, host = host_join(vjlib, ctx, cuda, rk, rp, sk, sp, 1, 4, int(need.value), False)
    assert n == want[0]
    assert digest_of_host(vjlib, cuda, host, n, 4) == want[1]


@pytest.mark.parametrize("offset", [0, 1, 2])
def test_pinned_tables_at_any_alignment(vjlib, ctx, cuda, oracle, offset):
    """Page-locked tables starting 0, 4 or 8 bytes past a 16-byte boundary (16-, 4- and
    8-byte loads of host memory), on the unchunked path."""
    import torch

    g = oracle.gen_join(12 + offset, 4, 30_000, 120_000, 0.75)
    rk, sk = g["r_keys"], g["s_keys"]
    rp = g["r_pay"].astype(np.uint32)
    sp = g["s_pay"].astype(np.uint32)

    def pinned(a):
        t = torch.zeros(a.size + 4, dtype=torch.int32).pin_memory()
        t[offset : offset + a.size] = torch.from_numpy(a.view(np.int32))
        return t[offset : offset + a.size]

    h = [pinned(a) for a in (rk, rp, sk, sp)]
    assert h[0].data_ptr() % 16 == 4 * offset
    out = torch.zeros((120_000, 2), dtype=torch.int32).pin_memory()
    n = ctx.join_host(vjlib.table(h[0], h[1], rk.size, 1, 4), vjlib.table(h[2], h[3], sk.size, 1, 4), out, 120_000)
    cnt, want, _ = oracle.join(rk, g["r_pay"], sk, g["s_pay"])
    assert n == cnt == g["matches"]
    assert np.array_equal(sort_pairs(out[:n].numpy().view(np.uint32).astype(np.uint64)), want)


def test_chunked_small_build_side(vjlib, ctx, cuda, oracle):
    """A build side too small for a radix pass: each chunk is joined whole."""
    rng = np.random.default_rng(55)
    nr, ns = 1000, (1 << 23) + 5
    rk = rng.integers(0, 3000, size=nr, dtype=np.uint64)
    sk = rng.integers(0, 3000, size=ns, dtype=np.uint64)
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, _, _ = oracle.join(rk, rp, sk, sp)
    want = device_join(vjlib, ctx, cuda, rk, rp, sk, sp, 2, 8)
    assert want[0] == cnt
    n, host = host_join(vjlib, ctx, cuda, rk, rp, sk, sp, 2, 8, cnt, True)
    assert n == cnt
    assert digest_of_host(vjlib, cuda, host, n, 8) == want[1]
