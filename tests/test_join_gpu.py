"""vj_join / vj_build_probe / vj_join_host on the GPU against the oracle and the reference's
own join_cpu results (golden). Output equality = match count + the sorted pair list; at
full benchmark sizes = count + order-independent digest against the generator's truth."""
from __future__ import annotations

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, d):
    import torch

    a = np.ascontiguousarray(a)
    if a.size == 0:
        return torch.zeros(1, dtype=torch.int64, device=d)
    return torch.from_numpy(a.view(np.int64) if a.itemsize == 8 else a.view(np.int32)).to(d)


def key_words(keys):
    return keys.itemsize // 4 * (keys.shape[1] if keys.ndim > 1 else 1)


def gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts=None, capacity=None):
    """Join through the C ABI into a caller buffer; returns sorted [M, 2] u64 pairs."""
    import torch

    kw = key_words(rk) if rk.size else key_words(sk)
    pb = rp.itemsize
    nr, ns = rp.size, sp.size
    cap = capacity if capacity is not None else max(1, ns)
    out = torch.zeros((cap, 2), dtype=torch.int64 if pb == 8 else torch.int32, device=cuda)
    res = ctx.join(vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, kw, pb), vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, kw, pb), opts, out=out, capacity=cap)
    torch.cuda.synchronize()
    got = out[: res.count].cpu().numpy().view(np.uint64 if pb == 8 else np.uint32).astype(np.uint64)
    return res.count, got


def sort_pairs(p):
    p = np.asarray(p, dtype=np.uint64).reshape(-1, 2)
    if p.shape[0] > 1:
        p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return p


def test_golden_reference_join_cpu_cases(vjlib, ctx, cuda, join_cases):
    meta = json.loads(bytes(join_cases["meta"]).decode())
    for name, m in meta.items():
        rk = join_cases[f"{name}_r_keys"]
        sk = join_cases[f"{name}_s_keys"]
        want = join_cases[f"{name}_pairs"]
        rp = np.arange(1, m["nr"] + 1, dtype=np.uint64)
        sp = np.arange(1, m["ns"] + 1, dtype=np.uint64)
        for opts in (None, vjlib.options(passes=1, radix_bits=(4, 0)), vjlib.options(passes=2, radix_bits=(3, 2), build_rows=32)):
            count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=max(1, m["matches"]))
            assert count == m["matches"], name
            assert np.array_equal(sort_pairs(got), want), name


@pytest.mark.parametrize("kw,pb", [(1, 4), (1, 8), (2, 4), (2, 8), (4, 8), (6, 4), (8, 8)])
def test_random_layouts_vs_oracle(vjlib, ctx, cuda, oracle, kw, pb):
    rng = np.random.default_rng(kw * 10 + pb)
    nr, ns = 20_000, 70_000
    cols = max(1, kw // 2)
    kt = np.uint32 if kw == 1 else np.uint64
    dom = 30_000 if kw <= 2 else 6
    rk = rng.integers(0, dom, size=(nr, cols)).astype(kt)
    sk = rng.integers(0, dom, size=(ns, cols)).astype(kt)
    if cols == 1:
        rk, sk = rk[:, 0].copy(), sk[:, 0].copy()
    pt = np.uint32 if pb == 4 else np.uint64
    rp = rng.permutation(nr).astype(pt)
    sp = rng.permutation(ns).astype(pt)
    cnt, want, _ = oracle.join(rk, rp.astype(np.uint64), sk, sp.astype(np.uint64))
    for opts in (None, vjlib.options(passes=0), vjlib.options(passes=1, radix_bits=(6, 0)), vjlib.options(passes=2, radix_bits=(5, 4))):
        count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=max(1, cnt))
        assert count == cnt, opts
        assert np.array_equal(sort_pairs(got), want)


def test_cross_product_chunks_small_tables(vjlib, ctx, cuda, oracle):
    # build partitions larger than one table: (build chunk x probe chunk) work items
    rng = np.random.default_rng(7)
    nr, ns = 5_000, 9_000
    rk = rng.integers(0, 700, size=nr, dtype=np.uint64)
    sk = rng.integers(0, 700, size=ns, dtype=np.uint64)
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    for opts in (vjlib.options(passes=0, build_rows=64, probe_rows=500), vjlib.options(passes=1, radix_bits=(2, 0), build_rows=128, probe_rows=1000)):
        count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=cnt)
        assert count == cnt
        assert np.array_equal(sort_pairs(got), want)


def test_degenerate_hash_one_partition(vjlib, ctx, cuda, oracle):
    # custom_xor over the two words of (a ^ c) << 32 | a is c for every row
    rng = np.random.default_rng(3)
    a = rng.integers(0, 2**32, size=3000, dtype=np.uint64)
    rk = ((a ^ np.uint64(0xBEEF)) << np.uint64(32)) | a
    sk = rk[rng.integers(0, 3000, size=8000)]
    rp = np.arange(3000, dtype=np.uint64)
    sp = np.arange(8000, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, vjlib.options(hash_algo=1, passes=2, radix_bits=(4, 4)), capacity=cnt)
    assert count == cnt == 8000
    assert np.array_equal(sort_pairs(got), want)


@pytest.mark.parametrize("pattern", ["high_word", "equal_halves", "top_bits", "stride_2p20", "int32_high", "wide_last_word"])
def test_patterned_keys_vs_oracle(vjlib, ctx, cuda, oracle, pattern):
    # Keys whose differences sit in few bits: the probe's table slots come from a
    # multiplicative mix of the key (not of its hash), so such key sets must still find
    # every match, whatever the partitioning.
    rng = np.random.default_rng(11)
    n = 12_000
    i = rng.permutation(n).astype(np.uint64) + np.uint64(1)
    if pattern == "high_word":
        rk = i << np.uint64(32)
    elif pattern == "equal_halves":
        rk = (i << np.uint64(32)) | i
    elif pattern == "top_bits":
        rk = i << np.uint64(50)
    elif pattern == "stride_2p20":
        rk = i << np.uint64(20)
    elif pattern == "int32_high":
        rk = (i << np.uint64(18)).astype(np.uint32)
    else:  # 16-byte keys equal but for the last word
        rk = np.zeros((n, 2), dtype=np.uint64)
        rk[:, 0] = np.uint64(0x0123456789ABCDEF)
        rk[:, 1] = i << np.uint64(40)
    pick = rng.integers(0, n, size=3 * n)
    sk = rk[pick].copy()
    miss = rng.random(3 * n) < 0.3  # 30 % of the probe rows get a key outside R
    if rk.ndim == 1:
        sk[miss] = sk[miss] + rk.dtype.type(1)
    else:
        sk[miss, 0] = sk[miss, 0] + np.uint64(1)
    rp = np.arange(n, dtype=np.uint64)
    sp = np.arange(3 * n, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    for opts in (None, vjlib.options(passes=0), vjlib.options(passes=1, radix_bits=(3, 0))):
        count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=max(1, cnt))
        assert count == cnt, (pattern, opts)
        assert np.array_equal(sort_pairs(got), want), (pattern, opts)


def test_skewed_probe_side(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(5)
    nr, ns = 50_000, 400_000
    rk = rng.permutation(np.arange(1, nr + 1, dtype=np.uint64) * np.uint64(0x9E3779B1))
    ranks = np.minimum(rng.zipf(1.3, size=ns), nr) - 1
    sk = rk[ranks]
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, capacity=cnt)
    assert count == cnt == ns
    assert np.array_equal(sort_pairs(got), want)


def test_duplicate_build_keys_grow_library_output(vjlib, ctx, cuda, oracle):
    import torch

    rng = np.random.default_rng(6)
    nr, ns = 4000, 6000
    rk = rng.integers(0, 50, size=nr, dtype=np.uint64)  # ~80 duplicates per key
    sk = rng.integers(0, 50, size=ns, dtype=np.uint64)
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, want, dig = oracle.join(rk, rp, sk, sp)
    assert cnt > ns
    # library-owned output: starts at |S| pairs and is grown to the exact count
    res = ctx.join(vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, 2, 8), vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, 2, 8))
    assert res.owned == 1 and res.count == cnt
    got = vjlib.device_to_numpy(res.pairs, 2 * res.count, np.uint64)
    assert np.array_equal(sort_pairs(got), want)
    assert vjlib.pairs_digest(res.pairs, res.count, 8) == dig
    ctx.free(res)
    # caller buffer too small: VJ_ERR_CAPACITY and the needed count
    out = torch.zeros((100, 2), dtype=torch.int64, device=cuda)
    with pytest.raises(vjlib.VjError) as e:
        ctx.join(vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, 2, 8), vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, 2, 8), out=out, capacity=100)
    assert e.value.status == vjlib.VJ_ERR_CAPACITY


def test_probe_shapes_vs_oracle(vjlib, ctx, cuda, oracle):
    """Probe block sizes, table loads and build/probe chunk sizes (several items per
    partition, items with more probe rows than one round) give the oracle's pairs."""
    rng = np.random.default_rng(12)
    nr, ns = 40_000, 300_000
    rk = rng.permutation(np.arange(nr, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
    pick = rng.integers(0, 2 * nr, size=ns)
    sk = np.where(pick < nr, rk[np.minimum(pick, nr - 1)], pick.astype(np.uint64) + np.uint64(1 << 40))
    rp = np.arange(nr, dtype=np.uint64)
    sp = np.arange(ns, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    for opts in (
        vjlib.options(probe_threads=64),
        vjlib.options(probe_threads=288),
        vjlib.options(probe_threads=1024, table_load_pct=25),
        vjlib.options(table_load_pct=12),
        vjlib.options(passes=1, radix_bits=(3, 0), build_rows=512, probe_rows=20_000),
        vjlib.options(passes=2, radix_bits=(2, 2), probe_rows=9000),
    ):
        count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, opts, capacity=cnt)
        assert count == cnt, vjlib.options_dict(opts)
        assert np.array_equal(sort_pairs(got), want), vjlib.options_dict(opts)


def test_device_flag_reaches_the_status(vjlib, ctx, cuda, oracle):
    """A flag a kernel sets in the join's error word (here planted by the test option, as a
    bounded wait that ran out would set it) comes back as VJ_ERR_DEVICE, and the next join
    on the same context is clean again."""
    rng = np.random.default_rng(4)
    rk = rng.integers(0, 2**40, size=5000, dtype=np.uint64)
    sk = rk[rng.integers(0, 5000, size=20000)]
    rp = np.arange(5000, dtype=np.uint64)
    sp = np.arange(20000, dtype=np.uint64)
    with pytest.raises(vjlib.VjError) as e:
        gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, vjlib.options(test_device_flag=True), capacity=20000)
    assert e.value.status == vjlib.VJ_ERR_DEVICE
    assert "flags 20" in str(e.value)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    count, got = gpu_join(vjlib, ctx, cuda, rk, rp, sk, sp, capacity=20000)
    assert count == cnt and np.array_equal(sort_pairs(got), want)


def test_l2_tables_flag_refused(vjlib, ctx, cuda):
    one = np.array([5], np.uint64)
    with pytest.raises(vjlib.VjError) as e:
        gpu_join(vjlib, ctx, cuda, one, one, one, one, vjlib.options(tables="l2"))
    assert e.value.status == vjlib.VJ_ERR_UNSUPPORTED


def test_empty_and_single(vjlib, ctx, cuda):
    e = np.zeros(0, np.uint64)
    one = np.array([5], np.uint64)
    assert gpu_join(vjlib, ctx, cuda, e, e, one, one)[0] == 0
    assert gpu_join(vjlib, ctx, cuda, one, one, e, e)[0] == 0
    count, got = gpu_join(vjlib, ctx, cuda, one, np.array([9], np.uint64), one, np.array([4], np.uint64))
    assert count == 1 and got.tolist() == [[9, 4]]


def test_join_host_buffers(vjlib, ctx, cuda, oracle):
    import torch

    g = oracle.gen_join(11, 4, 30_000, 120_000, 0.75)
    rk, sk = g["r_keys"], g["s_keys"]
    rp = g["r_pay"].astype(np.uint32)
    sp = g["s_pay"].astype(np.uint32)
    out = np.zeros((120_000, 2), np.uint32)
    n = ctx.join_host(vjlib.table(rk, rp, rk.size, 1, 4), vjlib.table(sk, sp, sk.size, 1, 4), out, 120_000)
    cnt, want, _ = oracle.join(rk, g["r_pay"], sk, g["s_pay"])
    assert n == cnt == g["matches"]
    assert np.array_equal(sort_pairs(out[:n].astype(np.uint64)), want)
    torch.cuda.synchronize()


def test_build_probe_with_and_without_hashes(vjlib, ctx, cuda, oracle):
    import torch

    rng = np.random.default_rng(8)
    nr, ns = 3000, 10_000
    rk = rng.integers(0, 4000, size=nr, dtype=np.uint64)
    sk = rng.integers(0, 4000, size=ns, dtype=np.uint64)
    rp = np.arange(1, nr + 1, dtype=np.uint64)
    sp = np.arange(1, ns + 1, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    out = torch.zeros((max(cnt, 1), 2), dtype=torch.int64, device=cuda)
    t_r = vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, 2, 8)
    t_s = vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, 2, 8)
    n = ctx.build_probe(t_r, t_s, out=out, capacity=cnt)
    assert n == cnt
    assert np.array_equal(sort_pairs(out[:n].cpu().numpy().view(np.uint64)), want)
    # with hashes: rows match only when hash and keys agree; equal keys from hash_func agree
    for hb in (32, 64):
        rh, _ = oracle.hash_elements(rk.view(np.uint32), nr, 0, 1, 64, hb, "fnv")
        sh, _ = oracle.hash_elements(sk.view(np.uint32), ns, 0, 1, 64, hb, "fnv")
        out.zero_()
        n = ctx.build_probe(t_r, t_s, r_hashes=dev(rh, cuda), s_hashes=dev(sh, cuda), hash_bits=hb, out=out, capacity=cnt)
        assert n == cnt
        assert np.array_equal(sort_pairs(out[:n].cpu().numpy().view(np.uint64)), want)
    # hashes that disagree for equal keys suppress those matches (hash test of probe_kernel)
    rh = np.arange(nr, dtype=np.uint64)
    sh = np.full(ns, 2**63, dtype=np.uint64)
    assert ctx.build_probe(t_r, t_s, r_hashes=dev(rh, cuda), s_hashes=dev(sh, cuda), hash_bits=64, out=out, capacity=cnt) == 0
    # count only
    assert ctx.build_probe(t_r, t_s, out=None, capacity=0) == cnt


def test_build_probe_partitioned_with_hashes(vjlib, ctx, cuda, oracle):
    # tables large enough that build_and_probe partitions them: the probe reads row-contiguous
    # rows that carry their hash (key and hash loaded, the payload read when a row matches)
    import torch

    rng = np.random.default_rng(9)
    nr, ns = 60_000, 200_000
    rk = rng.integers(0, 80_000, size=nr, dtype=np.uint64)
    sk = rng.integers(0, 80_000, size=ns, dtype=np.uint64)
    rp = np.arange(1, nr + 1, dtype=np.uint64)
    sp = np.arange(1, ns + 1, dtype=np.uint64)
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    out = torch.zeros((max(cnt, 1), 2), dtype=torch.int64, device=cuda)
    t_r = vjlib.table(dev(rk, cuda), dev(rp, cuda), nr, 2, 8)
    t_s = vjlib.table(dev(sk, cuda), dev(sp, cuda), ns, 2, 8)
    for hb in (32, 64):
        rh, _ = oracle.hash_elements(rk.view(np.uint32), nr, 0, 1, 64, hb, "fnv")
        sh, _ = oracle.hash_elements(sk.view(np.uint32), ns, 0, 1, 64, hb, "fnv")
        out.zero_()
        n = ctx.build_probe(t_r, t_s, r_hashes=dev(rh, cuda), s_hashes=dev(sh, cuda), hash_bits=hb, out=out, capacity=cnt)
        assert n == cnt, hb
        assert np.array_equal(sort_pairs(out[:n].cpu().numpy().view(np.uint64)), want), hb


def test_generator_matches_oracle(vjlib, cuda, oracle):
    import torch

    for kb, pb in ((4, 4), (8, 8)):
        nr, ns = 10_000, 40_000
        thr = oracle.match_threshold(0.5)
        kt = torch.int32 if kb == 4 else torch.int64
        pt = torch.int32 if pb == 4 else torch.int64
        rk = torch.zeros(nr, dtype=kt, device=cuda)
        sk = torch.zeros(ns, dtype=kt, device=cuda)
        rp = torch.zeros(nr, dtype=pt, device=cuda)
        sp = torch.zeros(ns, dtype=pt, device=cuda)
        vjlib.generate_join(42, kb, pb, nr, ns, thr, rk, rp, sk, sp)
        torch.cuda.synchronize()
        g = oracle.gen_join(42, kb, nr, ns, 0.5)
        kdt = np.uint32 if kb == 4 else np.uint64
        assert np.array_equal(rk.cpu().numpy().view(kdt), g["r_keys"])
        assert np.array_equal(sk.cpu().numpy().view(kdt), g["s_keys"])
        assert np.array_equal(sp.cpu().numpy().astype(np.uint64) if pb == 4 else sp.cpu().numpy().view(np.uint64), g["s_pay"])
        assert vjlib.generate_join_expect(42, nr, ns, thr) == oracle.gen_join_expect(42, nr, ns, 0.5)


@pytest.mark.parametrize("tables", ["auto", "shared"])
@pytest.mark.parametrize(
    "name,kb,pb,nr,ns,ratio",
    [
        ("int32 FK join 2^20 x 2^22", 4, 4, 1 << 20, 1 << 22, 1.0),
        ("int64 50% join 2^27 x 2^29", 8, 8, 1 << 27, 1 << 29, 0.5),
    ],
)
def test_full_size_count_and_digest(vjlib, ctx, cuda, name, kb, pb, nr, ns, ratio, tables):
    """Benchmark sizes: count and order-independent digest equal the generator's truth,
    with the planner's choice of tables and with each kind forced."""
    import torch

    thr = int(round(ratio * (1 << 32)))
    kt = torch.int32 if kb == 4 else torch.int64
    pt = torch.int32 if pb == 4 else torch.int64
    rk = torch.empty(nr, dtype=kt, device=cuda)
    sk = torch.empty(ns, dtype=kt, device=cuda)
    rp = torch.empty(nr, dtype=pt, device=cuda)
    sp = torch.empty(ns, dtype=pt, device=cuda)
    vjlib.generate_join(42, kb, pb, nr, ns, thr, rk, rp, sk, sp)
    want = vjlib.generate_join_expect(42, nr, ns, thr)
    cap = want[0]
    out = torch.empty((cap, 2), dtype=pt, device=cuda)
    opts = vjlib.options(tables=tables)
    res = ctx.join(vjlib.table(rk, rp, nr, kb // 4, pb), vjlib.table(sk, sp, ns, kb // 4, pb), opts, out=out, capacity=cap)
    assert res.count == want[0], name
    assert ctx.last_profile().tables == 0
    assert vjlib.pairs_digest(out, res.count, pb) == (want[1], want[2]), name
    del rk, sk, rp, sp, out
    torch.cuda.empty_cache()
