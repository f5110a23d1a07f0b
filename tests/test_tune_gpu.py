"""The autotuner: candidate plans agree on the result, the winner is kept per shape class
and used by later automatic joins of that class (same pairs), and the cache survives a
save / load round trip into another context."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tables(vjlib, cuda, nr, ns, seed):
    import torch

    rk = torch.empty(nr, dtype=torch.int64, device=cuda)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int64, device=cuda)
    sp = torch.empty_like(sk)
    thr = 1 << 31
    vjlib.generate_join(seed, 8, 8, nr, ns, thr, rk, rp, sk, sp)
    return vjlib.table(rk, rp, nr, 2, 8), vjlib.table(sk, sp, ns, 2, 8), vjlib.generate_join_expect(seed, nr, ns, thr)


def test_tune_then_automatic_join_uses_it(vjlib, cuda, tmp_path):
    import torch

    nr, ns = 1 << 21, 1 << 23
    r, s, want = _tables(vjlib, cuda, nr, ns, 11)
    out = torch.empty((ns, 2), dtype=torch.int64, device=cuda)
    ctx = vjlib.Context(0)
    try:
        ctx.set_profiling(True)
        best, ms = ctx.tune(r, s, out, ns)
        assert ms > 0
        res = ctx.join(r, s, None, out=out, capacity=ns)  # automatic: the tuned plan
        prof = ctx.last_profile()
        assert res.count == want[0] and vjlib.pairs_digest(out, res.count, 8) == (want[1], want[2])
        if best.flags & vjlib.VJ_JOIN_FIXED_PASSES:
            assert prof.passes == best.passes
            assert prof.radix_bits[0] == best.radix_bits[0]
        path = tmp_path / "tune.txt"
        ctx.tune_save(str(path))
        text = path.read_text()
        assert text.count("\n") == 2  # header + one entry
    finally:
        ctx.close()
    # a fresh context loads the cache and plans the same way
    ctx2 = vjlib.Context(0)
    try:
        ctx2.set_profiling(True)
        ctx2.tune_load(str(path))
        res = ctx2.join(r, s, None, out=out, capacity=ns)
        assert res.count == want[0] and vjlib.pairs_digest(out, res.count, 8) == (want[1], want[2])
        if best.flags & vjlib.VJ_JOIN_FIXED_PASSES:
            assert ctx2.last_profile().radix_bits[0] == best.radix_bits[0]
        # another shape class is not affected: a much smaller join plans on its own
        r3, s3, want3 = _tables(vjlib, cuda, 1 << 12, 1 << 14, 12)
        res3 = ctx2.join(r3, s3, None, out=out, capacity=ns)
        assert res3.count == want3[0]
    finally:
        ctx2.close()


def test_tune_load_rejects_a_malformed_file(vjlib, cuda, tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("not a tuning line\n")
    ctx = vjlib.Context(0)
    try:
        with pytest.raises(vjlib.VjError) as e:
            ctx.tune_load(str(bad))
        assert e.value.status == vjlib.VJ_ERR_INVALID_ARGUMENT
    finally:
        ctx.close()


def _lg(x):
    b = 0
    while (1 << b) < x:
        b += 1
    return b


def test_tuned_plan_reaches_batched_joins_and_server_requests(vjlib, cuda, tmp_path):
    """A tuning entry (here loaded from a cache file, so that its plan is known) changes the
    plan of vj_join_batch -- keyed by the batch's largest join -- and of a server request
    whose slots share the cache; the results stay those of the untuned plans."""
    import torch

    # batch: 8 int64 joins of 2^14 .. 2^16 build rows, |S| = 4 |R|
    sizes = [1 << (14 + (j % 3)) for j in range(8)]
    r_off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    s_off = 4 * r_off
    nr, ns = int(r_off[-1]), int(s_off[-1])
    rk = torch.empty(nr, dtype=torch.int64, device=cuda)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int64, device=cuda)
    sp = torch.empty_like(sk)
    for j in range(8):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        vjlib.generate_join(100 + j, 8, 8, b - a, d - c, 1 << 31, rk[a:b], rp[a:b], sk[c:d], sp[c:d])
    t_r, t_s = vjlib.table(rk, rp, nr, 2, 8), vjlib.table(sk, sp, ns, 2, 8)
    d_r, d_s = torch.from_numpy(r_off).to(cuda), torch.from_numpy(s_off).to(cuda)
    max_r = max(sizes)

    def batch(ctx):
        pairs = torch.zeros((ns, 2), dtype=torch.int64, device=cuda)
        counts = torch.zeros(8, dtype=torch.int64, device=cuda)
        status = torch.full((1,), -1, dtype=torch.int32, device=cuda)
        ctx.join_batch(t_r, t_s, 8, d_r, d_s, pairs, d_s, ns, counts, status, max_build_rows=max_r)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        c = counts.cpu().numpy()
        return [(int(c[j]), *vjlib.pairs_digest(pairs[int(s_off[j]) :], int(c[j]), 8)) for j in range(8)], ctx.last_profile()

    plain = vjlib.Context(0)
    try:
        want, prof0 = batch(plain)
    finally:
        plain.close()
    # a plan the planner would not pick: one pass of 3 bits, 256-row tables
    key = f"2 8 {_lg(max_r)} {_lg(max_r * 4 + 1)} 0 64"
    path = tmp_path / "plan.txt"
    path.write_text(f"{key} | 1 1 3 0 256 0 0 0 | 1.0\n")
    tuned = vjlib.Context(0)
    try:
        tuned.tune_load(str(path))
        got, prof1 = batch(tuned)
        assert got == want
        assert (prof1.passes, prof1.radix_bits[0], prof1.build_rows) == (1, 3, 256)
        assert (prof0.radix_bits[0], prof0.build_rows) != (3, 256)
    finally:
        tuned.close()

    # server: a request of a 2^16 x 2^18 join with the slots sharing a cache for its class
    r, s, exp = _tables(vjlib, cuda, 1 << 16, 1 << 18, 21)
    path2 = tmp_path / "plan2.txt"
    path2.write_text(f"2 8 16 18 0 64 | 1 1 3 0 256 0 0 0 | 1.0\n")
    src = vjlib.Context(0)
    srv = vjlib.Server(0, 0, 2)
    try:
        out = torch.zeros((1 << 18, 2), dtype=torch.int64, device=cuda)
        res0 = srv.wait(srv.submit(r, s, out, 1 << 18))
        assert res0.status == 0 and res0.count == exp[0]
        src.tune_load(str(path2))
        srv.share_tuning(src)
        res1 = srv.wait(srv.submit(r, s, out, 1 << 18))
        assert res1.status == 0 and res1.count == exp[0]
        assert vjlib.pairs_digest(out, res1.count, 8) == (exp[1], exp[2])
        assert (res1.passes, res1.radix_bits[0], res1.build_rows) == (1, 3, 256)
        assert (res0.radix_bits[0], res0.build_rows) != (3, 256)
    finally:
        srv.close()
        src.close()
