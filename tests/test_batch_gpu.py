"""vj_join_batch: many independent joins in one fused, persistent launch (or, with
VJ_JOIN_BATCH_LAUNCHES, the same phases as separate launches). Every join's pairs must
equal the oracle's (small joins) and vj_join's on the same rows (larger ones), in its own
output range; per-join capacities, out-of-range offsets, CUDA-graph replay and the graph's
single kernel node included."""
from __future__ import annotations

import numpy as np
import pytest

from test_join_gpu import dev, sort_pairs

pytestmark = pytest.mark.gpu


def make_batch(rng, joins, max_r, key_dtype, dup_domain=None):
    """Concatenated build/probe rows of `joins` joins; payloads are global row ids."""
    r_sizes = np.where(rng.random(joins) < 0.1, 0, rng.integers(1, max_r + 1, size=joins))
    s_sizes = np.where(rng.random(joins) < 0.1, 0, rng.integers(1, 4 * max_r + 1, size=joins))
    rks, sks = [], []
    for j in range(joins):
        dom = dup_domain or 4 * max(1, int(r_sizes[j]))
        base = rng.integers(0, 2**30 if key_dtype == np.uint32 else 2**62, dtype=np.uint64)
        rks.append((base + rng.integers(0, dom, size=r_sizes[j], dtype=np.uint64)).astype(key_dtype))
        sks.append((base + rng.integers(0, dom, size=s_sizes[j], dtype=np.uint64)).astype(key_dtype))
    r_off = np.concatenate([[0], np.cumsum(r_sizes)]).astype(np.uint64)
    s_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.uint64)
    rk = np.concatenate(rks)
    sk = np.concatenate(sks)
    pt = np.uint32 if key_dtype == np.uint32 else np.uint64
    return rk, np.arange(rk.size, dtype=pt), sk, np.arange(sk.size, dtype=pt), r_off, s_off


def oracle_per_join(oracle, rk, rp, sk, sp, r_off, s_off):
    wants = []
    for j in range(r_off.size - 1):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        if b > a and d > c:
            cnt, want, _ = oracle.join(rk[a:b], rp[a:b], sk[c:d], sp[c:d])
        else:
            cnt, want = 0, np.zeros((0, 2), np.uint64)
        wants.append((cnt, want))
    return wants


def run_batch(vjlib, ctx, cuda, rk, rp, sk, sp, r_off, s_off, caps, max_r=0, opts=None):
    import torch

    joins = r_off.size - 1
    kw = rk.itemsize // 4
    pb = rp.itemsize
    p_off = np.concatenate([[0], np.cumsum(caps)]).astype(np.uint64)
    total = int(p_off[-1])
    pairs = torch.zeros((max(1, total), 2), dtype=torch.int64 if pb == 8 else torch.int32, device=cuda)
    counts = torch.zeros(joins, dtype=torch.int64, device=cuda)
    status = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    t_r = vjlib.table(dev(rk, cuda), dev(rp, cuda), rk.size, kw, pb)
    t_s = vjlib.table(dev(sk, cuda), dev(sp, cuda), sk.size, kw, pb)
    ctx.join_batch(t_r, t_s, joins, dev(r_off, cuda), dev(s_off, cuda), pairs, dev(p_off, cuda), total, counts, status, max_build_rows=max_r, opts=opts)
    torch.cuda.synchronize()
    out = pairs.cpu().numpy().view(np.uint64 if pb == 8 else np.uint32).astype(np.uint64)
    return counts.cpu().numpy().view(np.uint64), out, p_off, int(status.cpu().numpy()[0])


@pytest.mark.parametrize("launches", [False, True], ids=["fused", "launches"])
@pytest.mark.parametrize("key_dtype", [np.uint32, np.uint64])
def test_batch_matches_oracle_per_join(vjlib, ctx, cuda, oracle, key_dtype, launches):
    rng = np.random.default_rng(31 if key_dtype == np.uint32 else 32)
    rk, rp, sk, sp, r_off, s_off = make_batch(rng, 60, 3000, key_dtype)
    wants = oracle_per_join(oracle, rk, rp, sk, sp, r_off, s_off)
    caps = np.array([max(1, w[0]) for w in wants], np.uint64)
    opts = vjlib.options(batch_launches=True) if launches else None
    counts, out, p_off, status = run_batch(vjlib, ctx, cuda, rk, rp, sk, sp, r_off, s_off, caps, max_r=3000, opts=opts)
    assert ctx.last_profile().kernel_launches == 1 if not launches else ctx.last_profile().kernel_launches > 1
    assert status == 0
    for j, (cnt, want) in enumerate(wants):
        assert counts[j] == cnt, j
        assert np.array_equal(sort_pairs(out[int(p_off[j]) : int(p_off[j]) + cnt]), want), j


def test_batch_duplicates_pass_choices(vjlib, ctx, cuda, oracle):
    # duplicate keys on both sides; joins large enough for a radix pass over the batch
    rng = np.random.default_rng(33)
    rk, rp, sk, sp, r_off, s_off = make_batch(rng, 24, 40_000, np.uint64, dup_domain=5000)
    wants = oracle_per_join(oracle, rk, rp, sk, sp, r_off, s_off)
    caps = np.array([max(1, w[0]) for w in wants], np.uint64)
    variants = (None, vjlib.options(passes=1, radix_bits=(6, 0)), vjlib.options(passes=0), vjlib.options(passes=1, radix_bits=(6, 0), batch_launches=True), vjlib.options(passes=0, batch_launches=True))
    for opts in variants:
        counts, out, p_off, status = run_batch(vjlib, ctx, cuda, rk, rp, sk, sp, r_off, s_off, caps, max_r=40_000, opts=opts)
        assert status == 0
        for j, (cnt, want) in enumerate(wants):
            assert counts[j] == cnt, j
            assert np.array_equal(sort_pairs(out[int(p_off[j]) : int(p_off[j]) + cnt]), want), j


def _generated_batch(vjlib, cuda, seed0, r_sizes, ratio):
    """Joins from the seeded generator (int32 keys and payloads), concatenated per side."""
    import torch

    s_sizes = 4 * r_sizes
    r_off = np.concatenate([[0], np.cumsum(r_sizes)]).astype(np.uint64)
    s_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.uint64)
    rk = torch.empty(int(r_off[-1]), dtype=torch.int32, device=cuda)
    rp = torch.empty_like(rk)
    sk = torch.empty(int(s_off[-1]), dtype=torch.int32, device=cuda)
    sp = torch.empty_like(sk)
    thr = int(ratio * (1 << 32))
    for j in range(r_sizes.size):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        vjlib.generate_join(seed0 + j, 4, 4, b - a, d - c, thr, rk[a:b], rp[a:b], sk[c:d], sp[c:d])
    return rk, rp, sk, sp, r_off, s_off, s_sizes, thr


def test_batch_equals_sequential_joins(vjlib, ctx, cuda):
    """300 joins, log-uniform sizes 2^6..2^16, 75% match: per-join count and digest equal
    vj_join's on the same rows and the generator's expectation."""
    import torch

    rng = np.random.default_rng(34)
    r_sizes = np.exp(rng.uniform(np.log(64), np.log(65536), size=300)).astype(np.int64)
    rk, rp, sk, sp, r_off, s_off, s_sizes, thr = _generated_batch(vjlib, cuda, 1000, r_sizes, 0.75)
    p_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.uint64)
    pairs = torch.zeros((int(p_off[-1]), 2), dtype=torch.int32, device=cuda)
    counts = torch.zeros(r_sizes.size, dtype=torch.int64, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    t_r = vjlib.table(rk, rp, rk.numel(), 1, 4)
    t_s = vjlib.table(sk, sp, sk.numel(), 1, 4)
    ctx.join_batch(t_r, t_s, r_sizes.size, dev(r_off, cuda), dev(s_off, cuda), pairs, dev(p_off, cuda), int(p_off[-1]), counts, status, max_build_rows=int(r_sizes.max()))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = counts.cpu().numpy()
    one = torch.zeros((int(s_sizes.max()), 2), dtype=torch.int32, device=cuda)
    for j in range(r_sizes.size):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        res = ctx.join(vjlib.table(rk[a:b], rp[a:b], b - a, 1, 4), vjlib.table(sk[c:d], sp[c:d], d - c, 1, 4), out=one, capacity=d - c)
        assert got[j] == res.count, j
        assert vjlib.pairs_digest(pairs[int(p_off[j]) :], res.count, 4) == vjlib.pairs_digest(one, res.count, 4), j
        assert res.count == vjlib.generate_join_expect(1000 + j, b - a, d - c, thr)[0]


def test_batch_per_join_capacity_and_bad_offsets(vjlib, ctx, cuda, oracle):
    rng = np.random.default_rng(35)
    rk, rp, sk, sp, r_off, s_off = make_batch(rng, 8, 500, np.uint64, dup_domain=50)
    wants = [w[0] for w in oracle_per_join(oracle, rk, rp, sk, sp, r_off, s_off)]
    # join 3 gets room for 5 pairs only: its count is still the full count, the others whole
    caps = np.array([max(1, w) for w in wants], np.uint64)
    caps[3] = 5
    counts, out, p_off, status = run_batch(vjlib, ctx, cuda, rk, rp, sk, sp, r_off, s_off, caps, max_r=500)
    assert status == 0
    assert [int(c) for c in counts] == wants
    # decreasing build offsets: clamped into range and reported in the status word
    bad = r_off.copy()
    bad[2], bad[3] = r_off[3] + 7, r_off[2]
    counts, out, p_off, status = run_batch(vjlib, ctx, cuda, rk, rp, sk, sp, bad, s_off, caps, max_r=500)
    assert status & 16


def test_batch_replays_in_a_cuda_graph(vjlib, ctx, cuda):
    import torch

    rng = np.random.default_rng(36)
    r_sizes = rng.integers(1000, 20000, size=64)
    rk, rp, sk, sp, r_off, s_off, s_sizes, thr = _generated_batch(vjlib, cuda, 7000, r_sizes, 0.75)
    p_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.uint64)
    pairs = torch.zeros((int(p_off[-1]), 2), dtype=torch.int32, device=cuda)
    counts = torch.zeros(r_sizes.size, dtype=torch.int64, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    t_r = vjlib.table(rk, rp, rk.numel(), 1, 4)
    t_s = vjlib.table(sk, sp, sk.numel(), 1, 4)
    d_r, d_s, d_p = dev(r_off, cuda), dev(s_off, cuda), dev(p_off, cuda)
    args = (t_r, t_s, int(r_sizes.size), d_r, d_s, pairs, d_p, int(p_off[-1]), counts, status)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    ctx.join_batch(*args, max_build_rows=int(r_sizes.max()), stream=stream)  # grows the workspace
    torch.cuda.synchronize()
    first = counts.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        ctx.join_batch(*args, max_build_rows=int(r_sizes.max()), stream=stream)
    counts.zero_()
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(counts, first) and int(status.item()) == 0
    for j in range(r_sizes.size):
        want = vjlib.generate_join_expect(7000 + j, int(r_sizes[j]), int(s_sizes[j]), thr)
        assert int(counts[j].item()) == want[0]
        assert vjlib.pairs_digest(pairs[int(p_off[j]) :], want[0], 4) == (want[1], want[2]), j


def test_batch_graph_holds_one_kernel_node(vjlib, ctx, cuda):
    """A batch captured from a stream is one kernel node (the fused launch; the rest are
    memsets and the status copy); replayed, every join equals the generator's expectation.
    The separate-launch form of the same batch is many kernel nodes."""
    import ctypes

    import torch

    try:
        rt = ctypes.CDLL("libcudart.so.13")
    except OSError:
        pytest.skip("libcudart.so.13 not loadable")
    rng = np.random.default_rng(37)
    r_sizes = np.exp(rng.uniform(np.log(2.0**10), np.log(2.0**16), size=200)).astype(np.int64)
    rk, rp, sk, sp, r_off, s_off, s_sizes, thr = _generated_batch(vjlib, cuda, 9000, r_sizes, 0.75)
    p_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.uint64)
    pairs = torch.zeros((int(p_off[-1]), 2), dtype=torch.int32, device=cuda)
    counts = torch.zeros(r_sizes.size, dtype=torch.int64, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    t_r = vjlib.table(rk, rp, rk.numel(), 1, 4)
    t_s = vjlib.table(sk, sp, sk.numel(), 1, 4)
    args = (t_r, t_s, int(r_sizes.size), dev(r_off, cuda), dev(s_off, cuda), pairs, dev(p_off, cuda), int(p_off[-1]), counts, status)
    stream = torch.cuda.Stream()
    h = ctypes.c_void_p(stream.cuda_stream)

    def kernel_nodes(opts):
        ctx.join_batch(*args, max_build_rows=int(r_sizes.max()), opts=opts, stream=stream)  # grows the workspace
        torch.cuda.synchronize()
        graph = ctypes.c_void_p()
        assert rt.cudaStreamBeginCapture(h, 0) == 0
        ctx.join_batch(*args, max_build_rows=int(r_sizes.max()), opts=opts, stream=stream)
        assert rt.cudaStreamEndCapture(h, ctypes.byref(graph)) == 0
        n = ctypes.c_size_t(0)
        assert rt.cudaGraphGetNodes(graph, None, ctypes.byref(n)) == 0
        nodes = (ctypes.c_void_p * n.value)()
        assert rt.cudaGraphGetNodes(graph, nodes, ctypes.byref(n)) == 0
        kinds = []
        for nd in nodes:
            t = ctypes.c_int(-1)
            assert rt.cudaGraphNodeGetType(ctypes.c_void_p(nd), ctypes.byref(t)) == 0
            kinds.append(t.value)
        exe = ctypes.c_void_p()
        assert rt.cudaGraphInstantiate(ctypes.byref(exe), graph, ctypes.c_ulonglong(0)) == 0
        counts.zero_()
        status.fill_(-1)
        torch.cuda.synchronize()
        for _ in range(2):
            assert rt.cudaGraphLaunch(exe, h) == 0
        assert rt.cudaStreamSynchronize(h) == 0
        rt.cudaGraphExecDestroy(exe)
        rt.cudaGraphDestroy(graph)
        assert int(status.item()) == 0
        for j in range(r_sizes.size):
            want = vjlib.generate_join_expect(9000 + j, int(r_sizes[j]), int(s_sizes[j]), thr)
            assert int(counts[j].item()) == want[0], j
            assert vjlib.pairs_digest(pairs[int(p_off[j]) :], want[0], 4) == (want[1], want[2]), j
        return kinds.count(0)  # cudaGraphNodeTypeKernel

    assert kernel_nodes(None) == 1
    assert kernel_nodes(vjlib.options(batch_launches=True)) >= 5
