"""The join server: requests of mixed sizes submitted together run concurrently in slots
under a memory budget; every result must equal the same join run alone through vj_join
(count and order-independent digest), the budget must hold, and a request larger than the
whole budget is refused."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_requests(vjlib, cuda, n, seed, lo=10, hi=20):
    import torch

    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        nr = int(np.exp(rng.uniform(np.log(2.0**lo), np.log(2.0**hi))))
        ns = int(rng.integers(2, 9)) * nr
        thr = int(rng.uniform(0.1, 1.0) * (1 << 32))
        rk = torch.empty(nr, dtype=torch.int64, device=cuda)
        rp = torch.empty_like(rk)
        sk = torch.empty(ns, dtype=torch.int64, device=cuda)
        sp = torch.empty_like(sk)
        vjlib.generate_join(seed * 1000 + i, 8, 8, nr, ns, thr, rk, rp, sk, sp)
        out = torch.empty((ns, 2), dtype=torch.int64, device=cuda)
        reqs.append((vjlib.table(rk, rp, nr, 2, 8), vjlib.table(sk, sp, ns, 2, 8), out, ns, seed * 1000 + i, thr))
    return reqs


def test_results_same_alone_and_in_the_mix(vjlib, ctx, cuda):
    import torch

    reqs = make_requests(vjlib, cuda, 24, 5)
    budget = 8 << 30
    srv = vjlib.Server(0, budget, 4)
    try:
        ids = [srv.submit(r, s, out, cap) for (r, s, out, cap, _, _) in reqs]
        results = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st.completed == 24 and st.peak_bytes <= budget
    assert st.peak_running >= 2  # requests overlapped on the device
    alone = torch.empty((max(q[3] for q in reqs), 2), dtype=torch.int64, device=cuda)
    for (r, s, out, cap, seed, thr), res in zip(reqs, results):
        assert res.status == 0
        assert res.submit_s <= res.start_s <= res.finish_s
        one = ctx.join(r, s, out=alone, capacity=cap)
        assert res.count == one.count == vjlib.generate_join_expect(seed, r.rows, s.rows, thr)[0]
        assert vjlib.pairs_digest(out, res.count, 8) == vjlib.pairs_digest(alone, one.count, 8)


def test_budget_admission_and_refusal(vjlib, cuda):
    reqs = make_requests(vjlib, cuda, 10, 6, lo=18, hi=20)
    budget = 1 << 30
    srv = vjlib.Server(0, budget, 4)
    try:
        ids = [srv.submit(r, s, out, cap) for (r, s, out, cap, _, _) in reqs]
        results = [srv.wait(i) for i in ids]
        st = srv.stats()
        # a join needing more than the whole budget is refused at submission
        big = make_requests(vjlib, cuda, 1, 7, lo=24, hi=24)[0]
        with pytest.raises(vjlib.VjError) as e:
            srv.submit(big[0], big[1], big[2], big[3])
        assert e.value.status == vjlib.VJ_ERR_BUDGET
    finally:
        srv.close()
    assert all(res.status == 0 for res in results)
    assert st.peak_bytes <= budget
    for (r, s, out, cap, seed, thr), res in zip(reqs, results):
        want = vjlib.generate_join_expect(seed, r.rows, s.rows, thr)
        assert res.count == want[0] and vjlib.pairs_digest(out, res.count, 8) == (want[1], want[2])


def test_capacity_error_is_per_request(vjlib, cuda):
    reqs = make_requests(vjlib, cuda, 3, 8, lo=12, hi=14)
    srv = vjlib.Server(0, 0, 2)
    try:
        r, s, out, cap, seed, thr = reqs[1]
        want = vjlib.generate_join_expect(seed, r.rows, s.rows, thr)[0]
        ids = [srv.submit(reqs[0][0], reqs[0][1], reqs[0][2], reqs[0][3]), srv.submit(r, s, out, 1), srv.submit(reqs[2][0], reqs[2][1], reqs[2][2], reqs[2][3])]
        res = [srv.wait(i) for i in ids]
    finally:
        srv.close()
    assert res[1].status == vjlib.VJ_ERR_CAPACITY and res[1].count == want
    assert res[0].status == 0 and res[2].status == 0
