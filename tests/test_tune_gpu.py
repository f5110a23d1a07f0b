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
