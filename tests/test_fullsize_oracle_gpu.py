"""Full-size joins of the benchmark shapes against the CPU oracle's own join.

The GPU joins the tables through the C ABI; the tables are then copied to the host and the
oracle (oracle/vj_oracle.c: multithreaded radix-partitioned chained-table join, the
reference's build/probe restated in C) joins them again. Count and the order-independent
pair digest (sum and xor of a 64-bit mix per pair) must agree -- the reference's verify
contract (src/join_benchmark.cu:97-148) without materialising 2^28 sorted pairs.

  - 2^27 x 2^29 int64 join, 50 % match (the headline benchmark join);
  - 2^26 unique x 2^28 Zipf(1.0) int64 skew join;
  - 4096 int32 joins in one vj_join_batch call, |R_i| log-uniform over [2^10, 2^20],
    |S_i| = 4 |R_i|, 75 % match: every join against its own oracle join.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_u64(t):
    return t.cpu().numpy().view(np.uint64)


def test_2p27_x_2p29_int64_join_vs_oracle(vjlib, ctx, cuda, oracle):
    import torch

    nr, ns, seed = 1 << 27, 1 << 29, 42
    thr = oracle.match_threshold(0.5)
    rk = torch.empty(nr, dtype=torch.int64, device=cuda)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int64, device=cuda)
    sp = torch.empty_like(sk)
    vjlib.generate_join(seed, 8, 8, nr, ns, thr, rk, rp, sk, sp)
    out = torch.empty((ns, 2), dtype=torch.int64, device=cuda)
    res = ctx.join(vjlib.table(rk, rp, nr, 2, 8), vjlib.table(sk, sp, ns, 2, 8), None, out=out, capacity=ns)
    got = (res.count, *vjlib.pairs_digest(out, res.count, 8))
    del out
    torch.cuda.empty_cache()
    cnt, _, dig = oracle.join(host_u64(rk), host_u64(rp), host_u64(sk), host_u64(sp), want_pairs=False)
    assert got == (cnt, *dig)
    assert cnt == oracle.gen_join_expect(seed, nr, ns, 0.5)[0]


def test_2p26_x_2p28_zipf_skew_join_vs_oracle(vjlib, ctx, cuda, oracle):
    import torch

    nr, ns = 1 << 26, 1 << 28
    rk = torch.empty(nr, dtype=torch.int64, device=cuda)
    rp = torch.empty_like(rk)
    one_k = torch.empty(1, dtype=torch.int64, device=cuda)
    one_p = torch.empty(1, dtype=torch.int64, device=cuda)
    vjlib.generate_join(42, 8, 8, nr, 1, 0, rk, rp, one_k, one_p)  # unique R keys, payload = row id
    # Zipf(1.0) ranks by inverse CDF in double precision; rank r -> a random build row
    gen = torch.Generator(device=cuda)
    gen.manual_seed(42)
    w = 1.0 / torch.arange(1, nr + 1, dtype=torch.float64, device=cuda)
    cdf = torch.cumsum(w, 0)
    cdf /= cdf[-1].clone()
    del w
    perm = torch.randperm(nr, generator=gen, device=cuda)
    ridx = torch.empty(ns, dtype=torch.int64, device=cuda)
    step = 1 << 25
    for a in range(0, ns, step):
        u = torch.rand(step, dtype=torch.float64, generator=gen, device=cuda)
        ridx[a : a + step] = perm[torch.clamp(torch.searchsorted(cdf, u), max=nr - 1)]
    del cdf, perm
    sk = rk[ridx]
    del ridx
    sp = torch.arange(ns, dtype=torch.int64, device=cuda)
    out = torch.empty((ns, 2), dtype=torch.int64, device=cuda)
    res = ctx.join(vjlib.table(rk, rp, nr, 2, 8), vjlib.table(sk, sp, ns, 2, 8), None, out=out, capacity=ns)
    got = (res.count, *vjlib.pairs_digest(out, res.count, 8))
    del out
    torch.cuda.empty_cache()
    cnt, _, dig = oracle.join(host_u64(rk), host_u64(rp), host_u64(sk), host_u64(sp), want_pairs=False)
    assert cnt == ns
    assert got == (cnt, *dig)


def test_4096_batched_int32_joins_vs_oracle(vjlib, ctx, cuda, oracle):
    import torch

    joins, seed = 4096, 42
    rng = np.random.default_rng(seed)
    r_sizes = np.exp(rng.uniform(np.log(2.0**10), np.log(2.0**20), size=joins)).astype(np.int64)
    s_sizes = 4 * r_sizes
    r_off = np.concatenate([[0], np.cumsum(r_sizes)]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.int64)
    nr, ns = int(r_off[-1]), int(s_off[-1])
    rk = torch.empty(nr, dtype=torch.int32, device=cuda)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int32, device=cuda)
    sp = torch.empty_like(sk)
    thr = oracle.match_threshold(0.75)
    for j in range(joins):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        vjlib.generate_join(seed + j, 4, 4, b - a, d - c, thr, rk[a:b], rp[a:b], sk[c:d], sp[c:d])
    pairs = torch.empty((ns, 2), dtype=torch.int32, device=cuda)  # join j may emit |S_j| pairs
    counts = torch.zeros(joins, dtype=torch.int64, device=cuda)
    status = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    d_r = torch.from_numpy(r_off).to(cuda)
    d_s = torch.from_numpy(s_off).to(cuda)
    ctx.join_batch(vjlib.table(rk, rp, nr, 1, 4), vjlib.table(sk, sp, ns, 1, 4), joins, d_r, d_s, pairs, d_s, ns, counts, status, max_build_rows=int(r_sizes.max()))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got_counts = counts.cpu().numpy()
    got = [(int(got_counts[j]), *vjlib.pairs_digest(pairs[int(s_off[j]) :], int(got_counts[j]), 4)) for j in range(joins)]
    del pairs
    h_rk = rk.cpu().numpy().view(np.uint32)
    h_sk = sk.cpu().numpy().view(np.uint32)
    h_rp = rp.cpu().numpy().view(np.uint32).astype(np.uint64)
    h_sp = sp.cpu().numpy().view(np.uint32).astype(np.uint64)

    def one(j):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        cnt, _, dig = oracle.join(h_rk[a:b], h_rp[a:b], h_sk[c:d], h_sp[c:d], hash_bits=32, threads=1, want_pairs=False)
        return (cnt, *dig)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        want = list(ex.map(one, range(joins)))
    bad = [j for j in range(joins) if got[j] != want[j]]
    assert not bad, f"{len(bad)} joins differ from the oracle, first {bad[:5]}"
