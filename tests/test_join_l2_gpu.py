"""Joins with L2-resident tables (one radix pass, per-partition open-addressing tables in
global memory) against the oracle: every layout, duplicates, several build chunks per
partition, many partitions (table regions reused), skew, degenerate hashes (which fall back
to shared-memory tables), capacity handling and hash-carrying rows."""
from __future__ import annotations

import numpy as np
import pytest

from test_join_gpu import dev, gpu_join, key_words, sort_pairs

pytestmark = pytest.mark.gpu


def keys_of(rng, n, kw, domain):
    """n keys of kw 32-bit words drawn from `domain` distinct values."""
    base = rng.integers(0, domain, size=n, dtype=np.uint64)
    if kw == 1:
        return (base * np.uint64(2654435761) % np.uint64(2**32)).astype(np.uint32)
    cols = [(base * np.uint64(0x9E3779B97F4A7C15 + 2 * c)) ^ np.uint64(c) for c in range(kw // 2)]
    return np.stack(cols, axis=1) if kw > 2 else cols[0]


def check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, opts):
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=max(cnt, 1))
    assert count == cnt
    assert np.array_equal(sort_pairs(got), want)
    return ctx.last_profile()


@pytest.mark.parametrize("kw,pb", [(1, 4), (1, 8), (2, 4), (2, 8), (4, 4), (4, 8), (6, 4), (6, 8), (8, 4), (8, 8)])
def test_layouts_with_l2_tables(vjlib, ctx, cuda, oracle, kw, pb):
    rng = np.random.default_rng(100 + kw * 10 + pb)
    nr, ns = 20_000, 70_000
    rk = keys_of(rng, nr, kw, 30_000)  # some duplicate build keys, ~half the probe rows miss
    sk = keys_of(rng, ns, kw, 45_000)
    pt = np.uint32 if pb == 4 else np.uint64
    rp = rng.permutation(nr).astype(pt)
    sp = rng.permutation(ns).astype(pt)
    for opts in (vjlib.options(tables="l2"), vjlib.options(tables="l2", passes=1, radix_bits=(6, 0))):
        prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, opts)
        assert prof.tables == 1 and prof.fallbacks == 0 and prof.passes == 1


def test_many_partitions_reuse_table_regions(vjlib, ctx, cuda, oracle):
    # 2^9 partitions -> hundreds of seqs over a ring of 8 table regions
    rng = np.random.default_rng(7)
    nr, ns = 60_000, 150_000
    rk = rng.permutation(np.arange(nr, dtype=np.uint64) * np.uint64(0x9E3779B1) + np.uint64(17))
    sk = np.concatenate([rk[rng.integers(0, nr, size=ns // 2)], rng.integers(2**62, 2**63, size=ns - ns // 2, dtype=np.uint64)])
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2", passes=1, radix_bits=(9, 0)))
    assert prof.tables == 1 and prof.radix_bits[0] == 9


def test_several_build_chunks_per_partition(vjlib, ctx, cuda, oracle):
    # build chunks of 1024 rows: ~15 seqs per partition, each probed by all its probe rows
    rng = np.random.default_rng(8)
    nr, ns = 30_000, 90_000
    rk = rng.integers(0, 20_000, size=nr, dtype=np.uint64)
    sk = rng.integers(0, 40_000, size=ns, dtype=np.uint64)
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2", passes=1, radix_bits=(1, 0), build_rows=1000, probe_rows=700))
    assert prof.tables == 1 and prof.build_rows == 1024 and prof.probe_rows == 700


def test_duplicate_heavy_build_side_falls_back(vjlib, ctx, cuda, oracle):
    # one key 3000 times: its cluster is longer than an insert may walk
    rng = np.random.default_rng(9)
    rk = np.concatenate([np.full(3000, 77, np.uint64), rng.integers(1000, 2**40, size=5000, dtype=np.uint64)])
    sk = np.concatenate([np.full(20, 77, np.uint64), rk[3000 + rng.integers(0, 5000, size=6000)], rng.integers(2**41, 2**42, size=3000, dtype=np.uint64)])
    rp = np.arange(rk.size, dtype=np.uint64)
    sp = np.arange(sk.size, dtype=np.uint64)
    prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2"))
    assert prof.fallbacks == 1 and prof.tables == 0


def test_moderate_duplicates_stay_in_l2(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(10)
    rk = np.repeat(rng.integers(0, 2**50, size=4000, dtype=np.uint64), 8)  # 8 copies of each key
    rng.shuffle(rk)
    sk = np.concatenate([rk[rng.integers(0, rk.size, size=50_000)], rng.integers(2**51, 2**52, size=20_000, dtype=np.uint64)])
    rp = np.arange(rk.size, dtype=np.uint64)
    sp = np.arange(sk.size, dtype=np.uint64)
    prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2", passes=1, radix_bits=(3, 0)))
    assert prof.tables == 1 and prof.fallbacks == 0


def test_degenerate_hash_falls_back(vjlib, ctx, cuda, oracle):
    # custom_xor over the two words of (a ^ c) << 32 | a is c for every row
    rng = np.random.default_rng(3)
    a = rng.integers(0, 2**32, size=3000, dtype=np.uint64)
    rk = ((a ^ np.uint64(0xBEEF)) << np.uint64(32)) | a
    sk = rk[rng.integers(0, 3000, size=8000)]
    rp = np.arange(3000, dtype=np.uint64)
    sp = np.arange(8000, dtype=np.uint64)
    prof = check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(hash_algo=1, tables="l2"))
    assert prof.fallbacks == 1


def test_skewed_probe_side_l2(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(5)
    nr, ns = 50_000, 400_000
    rk = rng.permutation(np.arange(1, nr + 1, dtype=np.uint64) * np.uint64(0x9E3779B1))
    sk = rk[np.minimum(rng.zipf(1.3, size=ns), nr) - 1]
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2", passes=1, radix_bits=(5, 0)))


def test_empty_partitions_and_sides(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(11)
    # few rows over 2^10 partitions: most partitions are empty on one side
    rk = rng.integers(0, 2**64, size=300, dtype=np.uint64)
    sk = np.concatenate([rk[:100], rng.integers(0, 2**64, size=200, dtype=np.uint64)])
    rp = np.arange(300, dtype=np.uint64)
    sp = np.arange(300, dtype=np.uint64)
    check(vjlib, ctx, cuda, oracle, rk, rp, sk, sp, vjlib.options(tables="l2", passes=1, radix_bits=(10, 0)))
    # no matches at all
    check(vjlib, ctx, cuda, oracle, rk, rp, sk[100:], sp[100:], vjlib.options(tables="l2"))


def test_owned_output_growth_and_capacity_error_l2(vjlib, ctx, cuda, oracle):
    import torch

    rng = np.random.default_rng(12)
    rk = rng.integers(0, 300, size=6000, dtype=np.uint64)  # ~20 copies per key: more pairs than |S|
    sk = rng.integers(0, 300, size=5000, dtype=np.uint64)
    rp = np.arange(6000, dtype=np.uint64)
    sp = np.arange(5000, dtype=np.uint64)
    cnt, want, dig = oracle.join(rk, rp, sk, sp)
    assert cnt > 5000
    opts = vjlib.options(tables="l2")
    res = ctx.join(vjlib.table(dev(rk, cuda), dev(rp, cuda), 6000, 2, 8), vjlib.table(dev(sk, cuda), dev(sp, cuda), 5000, 2, 8), opts)
    assert res.owned == 1 and res.count == cnt
    assert np.array_equal(sort_pairs(vjlib.device_to_numpy(res.pairs, 2 * res.count, np.uint64)), want)
    ctx.free(res)
    out = torch.zeros((10, 2), dtype=torch.int64, device=cuda)
    with pytest.raises(vjlib.VjError) as e:
        ctx.join(vjlib.table(dev(rk, cuda), dev(rp, cuda), 6000, 2, 8), vjlib.table(dev(sk, cuda), dev(sp, cuda), 5000, 2, 8), opts, out=out, capacity=10)
    assert e.value.status == vjlib.VJ_ERR_CAPACITY


@pytest.mark.parametrize("hb", [32, 64])
def test_join_with_hashes_on_l2_tables(vjlib, ctx, cuda, oracle, hb):
    """Rows that carry the caller's hashes (build_probe) through both table kinds: the
    shared-memory default, and L2 tables through vj_join on the same rows' keys."""
    import torch

    rng = np.random.default_rng(13 + hb)
    nr, ns = 1 << 21, 1 << 22
    rk = rng.permutation(np.arange(nr, dtype=np.uint64)) * np.uint64(0x9E3779B97F4A7C15)
    sk = np.concatenate([rk[rng.integers(0, nr, size=ns // 2)], rng.integers(0, 2**64, size=ns // 2, dtype=np.uint64) | np.uint64(1)])
    rk = rk & ~np.uint64(1)  # build keys even, misses odd
    sk[: ns // 2] &= ~np.uint64(1)
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    words_r = rk.view(np.uint32).reshape(nr, 2)
    words_s = sk.view(np.uint32).reshape(ns, 2)
    rh, _ = oracle.hash_elements(words_r, nr, 0, 2, 32, hb, "fnv")
    sh, _ = oracle.hash_elements(words_s, ns, 0, 2, 32, hb, "fnv")
    cnt, _, dig = oracle.join(rk, rp, sk, sp, want_pairs=False)
    out = torch.zeros((cnt, 2), dtype=torch.int64, device=cuda)
    t_r = vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, 2, 8)
    t_s = vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, 2, 8)
    n = ctx.build_probe(t_r, t_s, r_hashes=dev(rh, cuda), s_hashes=dev(sh, cuda), hash_bits=hb, out=out, capacity=cnt)
    assert n == cnt
    assert vjlib.pairs_digest(out, n, 8) == dig
    res = ctx.join(t_r, t_s, vjlib.options(hash_bits=hb, tables="l2"), out=out, capacity=cnt)
    assert res.count == cnt and ctx.last_profile().tables == 1
    assert vjlib.pairs_digest(out, res.count, 8) == dig
