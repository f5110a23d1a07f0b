"""Benchmark of the GB300 hash join (one JSON line on rank 0).

Workload (the reference's headline join shape): build R = 2^27 rows, probe S = 2^29 rows,
int64 keys and int64 payloads (payload = row id), R keys unique uniform 64-bit values,
half of the S keys drawn from R and half from a disjoint range, FNV-1a 64 hash, two radix
passes. A step is one vj_join of the device-resident tables into a device pair buffer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--small]

value   (|R|+|S|) * steps * ranks / max-over-ranks time, CUDA events on the join stream
e2e     the same through vj_join_host with pinned HOST tables and a HOST pair buffer
        (host->device copies of R and S and the device->host copy of the pairs inside)
roofline  the dominant kernel: algorithmic bytes per launch / its event-timed duration
cpu_baseline  the CPU oracle (multithreaded radix hash join) on a bounded sample
--impl reference  times the reference's CPU join path (the oracle port of it) on the host

N > 1 runs independent replicas, one per GPU (the join is single-GPU; weak scaling).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import re
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "vectorized-join_gb300"

METRIC = "join tuples/sec (|R|+|S|) and % of HBM roofline on 1 GB300; p50/p99 per-join latency"
UNIT = "tuples/s"
SEED = 42
LATENCY_SAMPLES = 30  # joins behind the p50/p99 latency figures


def _import(path: Path, name: str):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def workload(shift: int) -> dict:
    lr, ls = 27 - shift, 29 - shift
    return {
        "workload": f"int64 equi-join 2^{lr} x 2^{ls}, 50% match, FNV-1a 64, 2 radix passes",
        "r_rows": 1 << lr,
        "s_rows": 1 << ls,
        "key_bytes": 8,
        "payload_bytes": 8,
        "match_ratio": 0.5,
        "hash": "fnv1a-64",
        "l2_policy": "inputs (%.1f GiB) larger than the 126 MB L2; no flush needed" % (((1 << lr) + (1 << ls)) * 16 / 2**30),
    }


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def cpu_baseline(oracle, small: bool, budget_s: float = 12.0) -> dict:
    """Oracle join (all host threads) on a bounded sample of the same workload shape."""
    lr, ls = (19, 21) if small else (22, 24)
    nr, ns = 1 << lr, 1 << ls
    g = oracle.gen_join(SEED, 8, nr, ns, 0.5)
    threads = os.cpu_count() or 1
    runs, t_total = 0, 0.0
    while t_total < budget_s and runs < 50:
        t0 = time.perf_counter()
        cnt, _, _ = oracle.join(g["r_keys"], g["r_pay"], g["s_keys"], g["s_pay"], radix_bits=12, threads=threads, want_pairs=False)
        t_total += time.perf_counter() - t0
        runs += 1
        assert cnt == g["matches"]
    return {
        "value": (nr + ns) * runs / t_total,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"2^{lr} x 2^{ls} rows of the same int64 50%-match workload (1/{(1 << 27) // nr} of each side), {runs} joins, {t_total:.1f} s",
    }


def profiled_traffic(kernel: str):
    """`traffic-per-launch-at-full-size: <kernel> <bytes>` from the summaries in profiles/."""
    pat = re.compile(r"^traffic-per-launch-at-full-size:\s+(\w+)\s+(\d+)\s*$", re.M)
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for name, val in pat.findall(f.read_text()):
            if name == kernel:
                return int(val)
    return None


def max_over_ranks(value: float, device) -> float:
    """The largest `value` over all ranks (the slowest rank's time); `value` itself at N=1."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank_step: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return units_per_rank_step * steps * world / (max_ms / 1000.0)


def run_reference(args, cfg) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    oracle = _import(ROOT / "oracle" / "oracle.py", "vj_oracle")
    oracle.build()
    lr, ls = (19, 21) if args.small else (22, 24)
    nr, ns = 1 << lr, 1 << ls
    g = oracle.gen_join(SEED, 8, nr, ns, 0.5)
    threads = os.cpu_count() or 1

    def step():
        cnt, _, _ = oracle.join(g["r_keys"], g["r_pay"], g["s_keys"], g["s_pay"], radix_bits=12, threads=threads, want_pairs=False)
        assert cnt == g["matches"]

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = (nr + ns) * args.steps / dt
    sample = f"each step joins 2^{lr} x 2^{ls} rows of the same workload (CPU radix hash join restating the reference's algorithm, {threads} threads)"
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1000 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "data": "synthetic (seeded generator)",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own CPU join (join_cpu) is a nested loop; its radix/chained-table algorithm runs here as the C oracle port on all host threads",
    }
    print(json.dumps(line), flush=True)


def run_e2e(args, ctx, vj, torch, stream, dev, world, rk, rp, sk, sp, nr, ns, m, w, w_p):
    """The same join through vj_join_host: pinned host tables in, pinned host pairs out."""
    import torch.distributed as dist

    n = nr + ns
    torch.cuda.empty_cache()
    h_rk = torch.empty(nr, dtype=torch.int64, pin_memory=True)
    h_rp = torch.empty(nr, dtype=torch.int64, pin_memory=True)
    h_sk = torch.empty(ns, dtype=torch.int64, pin_memory=True)
    h_sp = torch.empty(ns, dtype=torch.int64, pin_memory=True)
    h_rk.copy_(rk)
    h_rp.copy_(rp)
    h_sk.copy_(sk)
    h_sp.copy_(sp)
    torch.cuda.synchronize()
    h_out = torch.empty((m, 2), dtype=torch.int64, pin_memory=True)
    th_r = vj.table(h_rk, h_rp, nr, 2, 8)
    th_s = vj.table(h_sk, h_sp, ns, 2, 8)
    got = ctx.join_host(th_r, th_s, h_out, m, stream=stream)  # warm-up (allocates the staging buffer)
    assert got == m
    torch.cuda.synchronize()
    e_steps = max(1, args.e2e_steps)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(e_steps + 1)]
    if world > 1:
        dist.barrier()
    evs[0].record(stream)
    for i in range(e_steps):
        got = ctx.join_host(th_r, th_s, h_out, m, stream=stream)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    assert got == m
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(e_steps)]
    e2e_ms = max_over_ranks(evs[0].elapsed_time(evs[-1]), dev)
    q = sorted(per)
    return {
        "value": job_rate(n, e_steps, world, e2e_ms),
        "unit": UNIT,
        "h2d_bytes_per_step": n * w,
        "d2h_bytes_per_step": m * 2 * w_p,
        "ms_per_step": e2e_ms / e_steps,
        "steps": e_steps,
        "step_ms": {"min": q[0], "p50": q[len(q) // 2], "max": q[-1], "stdev": statistics.pstdev(per)},
        "api": "vj_join_host (pinned host tables in, pinned host pairs out)",
    }


# ---------------------------------------------------------------- other workloads
#
# `--workload` selects one of the other measured shapes; each prints one JSON line with the
# same base keys. The default (the 2^27 x 2^29 int64 join) is the headline.


def _timed(torch, stream, fn, steps: int, warmup: int):
    """Per-step device times (ms) of fn() with CUDA events on `stream`, after warm-up."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for i in range(steps):
        fn()
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    return [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]


def _latency(ms: list) -> dict:
    q = sorted(ms)
    return {"p50": q[len(q) // 2], "p99": q[min(len(q) - 1, int(round(0.99 * (len(q) - 1))))], "min": q[0], "max": q[-1]}


def _base_line(metric, value, unit, steps, warmup, ms, dtype, cfg, hib=True):
    return {
        "metric": metric,
        "value": value,
        "unit": unit,
        "n_gpus": 1,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": ms,
        "higher_is_better": hib,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": dtype,
        "data": "synthetic (seeded, generated on the device)",
        "config": cfg,
    }


def run_small_join(args) -> None:
    """int32 keys and payloads, R = 2^20 unique keys, S = 2^22 drawn from R (100% match),
    FNV-1a 32, one radix pass of 8 bits. The working set (~42 MB) fits in L2."""
    import torch

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")
    oracle = _import(ROOT / "oracle" / "oracle.py", "vj_oracle")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nr, ns = 1 << 20, 1 << 22
    thr = 1 << 32
    rk = torch.empty(nr, dtype=torch.int32, device=dev)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int32, device=dev)
    sp = torch.empty_like(sk)
    vj.generate_join(SEED, 4, 4, nr, ns, thr, rk, rp, sk, sp)
    expect = vj.generate_join_expect(SEED, nr, ns, thr)
    out = torch.empty((expect[0], 2), dtype=torch.int32, device=dev)
    ctx = vj.Context(0)
    ctx.set_profiling(True)
    t_r, t_s = vj.table(rk, rp, nr, 1, 4), vj.table(sk, sp, ns, 1, 4)
    opts = vj.options(hash_bits=32, passes=1, radix_bits=(8, 0))
    stream = torch.cuda.current_stream()
    res = ctx.join(t_r, t_s, opts, out=out, capacity=expect[0], stream=stream)
    assert res.count == expect[0] and vj.pairs_digest(out, res.count, 4) == (expect[1], expect[2])
    steps = max(args.steps, 30)
    sampler = ClockSampler(0)
    sampler.start()
    ms = _timed(torch, stream, lambda: ctx.join(t_r, t_s, opts, out=out, capacity=expect[0], stream=stream), steps, args.warmup)
    clocks = sampler.stop()
    t = sum(ms) / len(ms)
    n = nr + ns
    b_alg = n * (1 * (4 + 2 * 8) + 8) + expect[0] * 2 * 4
    peak, src = measured_peak()
    cfg = {"workload": "int32 FK join 2^20 x 2^22, 100% match, FNV-1a 32, 1 radix pass of 8 bits", "r_rows": nr, "s_rows": ns, "l2_policy": "working set ~42 MB fits in L2: L2, not HBM, bounds it"}
    line = _base_line(METRIC, n / (t / 1000), UNIT, steps, args.warmup, t, "int32", cfg)
    line["join_roofline"] = {"bytes_alg_per_join": b_alg, "achieved": b_alg / (t / 1000) / 1e9, "peak": peak, "unit": "GB/s", "frac": b_alg / (t / 1000) / 1e9 / peak, "peak_source": src}
    line["latency_ms"] = _latency(ms)
    line["stages_ms"] = ctx.last_profile().as_dict()
    line["clocks"] = clocks
    # the oracle on the host cores, same inputs
    g = oracle.gen_join(SEED, 4, nr, ns, 1.0)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    runs = 0
    while time.perf_counter() - t0 < 5.0:
        cnt, _, _ = oracle.join(g["r_keys"], g["r_pay"], g["s_keys"], g["s_pay"], hash_bits=32, radix_bits=8, threads=threads, want_pairs=False)
        runs += 1
    assert cnt == expect[0]
    dt = time.perf_counter() - t0
    line["cpu_baseline"] = {"value": n * runs / dt, "unit": UNIT, "cores": threads, "kind": "port", "sample": f"the full workload, {runs} joins in {dt:.1f} s"}
    print(json.dumps(line), flush=True)


def run_skew_join(args) -> None:
    """R = 2^26 unique int64 keys, S = 2^28 keys drawn Zipf(s = 1.0) over R's keys: the heavy
    hitters crowd a few partitions and probe chains."""
    import torch

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nr, ns = 1 << 26, 1 << 28
    rk = torch.empty(nr, dtype=torch.int64, device=dev)
    rp = torch.empty_like(rk)
    dummy_k = torch.empty(1, dtype=torch.int64, device=dev)
    dummy_p = torch.empty(1, dtype=torch.int64, device=dev)
    vj.generate_join(SEED, 8, 8, nr, 1, 0, rk, rp, dummy_k, dummy_p)  # unique R keys, payload = row id
    # Zipf(1.0) ranks by inverse CDF (double precision); rank r -> a random build row
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    w = 1.0 / torch.arange(1, nr + 1, dtype=torch.float64, device=dev)
    cdf = torch.cumsum(w, 0)
    cdf /= cdf[-1].clone()
    del w
    perm = torch.randperm(nr, generator=gen, device=dev)
    ridx = torch.empty(ns, dtype=torch.int64, device=dev)
    chunk = 1 << 25
    for a in range(0, ns, chunk):
        u = torch.rand(chunk, dtype=torch.float64, generator=gen, device=dev)
        ridx[a : a + chunk] = perm[torch.clamp(torch.searchsorted(cdf, u), max=nr - 1)]
    del cdf, perm
    sk = rk[ridx]
    sp = torch.arange(ns, dtype=torch.int64, device=dev)
    want = torch.stack([rp[ridx], sp], dim=1).contiguous()
    want_digest = vj.pairs_digest(want, ns, 8)
    del want, ridx
    out = torch.empty((ns, 2), dtype=torch.int64, device=dev)
    ctx = vj.Context(0)
    ctx.set_profiling(True)
    t_r, t_s = vj.table(rk, rp, nr, 2, 8), vj.table(sk, sp, ns, 2, 8)
    stream = torch.cuda.current_stream()
    res = ctx.join(t_r, t_s, None, out=out, capacity=ns, stream=stream)
    assert res.count == ns and vj.pairs_digest(out, res.count, 8) == want_digest
    sampler = ClockSampler(0)
    sampler.start()
    ms = _timed(torch, stream, lambda: ctx.join(t_r, t_s, None, out=out, capacity=ns, stream=stream), args.steps, args.warmup)
    clocks = sampler.stop()
    prof = ctx.last_profile().as_dict()
    t = sum(ms) / len(ms)
    n = nr + ns
    b_alg = n * (2 * (8 + 2 * 16) + 16) + ns * 2 * 8
    peak, src = measured_peak()
    cfg = {"workload": "int64 skew join 2^26 unique x 2^28 Zipf(1.0) over R, 100% match, FNV-1a 64, 2 radix passes", "r_rows": nr, "s_rows": ns, "l2_policy": "inputs (5 GiB) larger than L2"}
    line = _base_line(METRIC, n / (t / 1000), UNIT, args.steps, args.warmup, t, "int64", cfg)
    line["join_roofline"] = {"bytes_alg_per_join": b_alg, "achieved": b_alg / (t / 1000) / 1e9, "peak": peak, "unit": "GB/s", "frac": b_alg / (t / 1000) / 1e9 / peak, "peak_source": src}
    line["latency_ms"] = _latency(ms)
    line["stages_ms"] = prof
    line["clocks"] = clocks
    print(json.dumps(line), flush=True)


def run_batch_join(args) -> None:
    """4096 independent int32 joins, |R_i| log-uniform over [2^10, 2^20], |S_i| = 4 |R_i|,
    75% of S_i drawn from R_i (per-join seed = 42 + i): one vj_join_batch call (one fused,
    persistent launch) replayed from a CUDA graph, against the same batch as separate
    launches (VJ_JOIN_BATCH_LAUNCHES) and the same 4096 joins as sequential vj_join calls."""
    import numpy as np
    import torch

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    joins = 4096 >> args.shift  # --shift: smaller profiling cases (fewer, smaller joins)
    rng = np.random.default_rng(SEED)
    r_sizes = np.exp(rng.uniform(np.log(2.0**10), np.log(2.0 ** (20 - args.shift)), size=joins)).astype(np.int64)
    s_sizes = 4 * r_sizes
    r_off = np.concatenate([[0], np.cumsum(r_sizes)]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum(s_sizes)]).astype(np.int64)
    nr, ns = int(r_off[-1]), int(s_off[-1])
    rk = torch.empty(nr, dtype=torch.int32, device=dev)
    rp = torch.empty_like(rk)
    sk = torch.empty(ns, dtype=torch.int32, device=dev)
    sp = torch.empty_like(sk)
    thr = int(round(0.75 * (1 << 32)))
    for j in range(joins):
        a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
        vj.generate_join(SEED + j, 4, 4, b - a, d - c, thr, rk[a:b], rp[a:b], sk[c:d], sp[c:d])
    want = [vj.generate_join_expect(SEED + j, int(r_sizes[j]), int(s_sizes[j]), thr) for j in range(joins)]
    m = sum(w[0] for w in want)
    p_off = s_off.copy()  # join j may emit up to |S_j| pairs (unique build keys)
    pairs = torch.empty((ns, 2), dtype=torch.int32, device=dev)
    counts = torch.zeros(joins, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    d_r = torch.from_numpy(r_off).to(dev)
    d_s = torch.from_numpy(s_off).to(dev)
    d_p = torch.from_numpy(p_off).to(dev)
    ctx = vj.Context(0)
    t_r, t_s = vj.table(rk, rp, nr, 1, 4), vj.table(sk, sp, ns, 1, 4)
    stream = torch.cuda.Stream()
    def graph_of(opts):
        call = lambda: ctx.join_batch(t_r, t_s, joins, d_r, d_s, pairs, d_p, ns, counts, status, max_build_rows=int(r_sizes.max()), opts=opts, stream=stream)
        call()  # grows the workspace outside the capture
        torch.cuda.synchronize()
        launches = ctx.last_profile().kernel_launches
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            call()
        counts.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        got = counts.cpu().numpy()
        for j in range(joins):
            assert got[j] == want[j][0], j
            assert vj.pairs_digest(pairs[int(p_off[j]) :], int(got[j]), 4) == (want[j][1], want[j][2]), j
        return g, launches

    g_sep, launches_sep = graph_of(vj.options(batch_launches=True))
    ms_sep = _timed(torch, torch.cuda.current_stream(), g_sep.replay, args.steps, args.warmup)
    del g_sep
    g, launches_fused = graph_of(None)
    sampler = ClockSampler(0)
    sampler.start()
    ms = _timed(torch, torch.cuda.current_stream(), g.replay, args.steps, args.warmup)  # replay() launches on the current stream
    clocks = sampler.stop()
    t_batch = sum(ms) / len(ms)
    # the same joins back to back through vj_join (each synchronises to return its count)
    seq_stream = torch.cuda.current_stream()

    def sequential():
        for j in range(joins):
            a, b, c, d = int(r_off[j]), int(r_off[j + 1]), int(s_off[j]), int(s_off[j + 1])
            res = ctx.join(vj.table(rk[a:b], rp[a:b], b - a, 1, 4), vj.table(sk[c:d], sp[c:d], d - c, 1, 4), out=pairs[c:d], capacity=d - c, stream=seq_stream)
            assert res.count == want[j][0]

    sequential()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(seq_stream)
    sequential()
    e1.record(seq_stream)
    torch.cuda.synchronize()
    t_seq = e0.elapsed_time(e1)
    n = nr + ns
    b_alg = n * (1 * (4 + 2 * 8) + 8) + m * 2 * 4
    peak, src = measured_peak()
    cfg = {
        "workload": f"batched join: {joins} int32 joins, |R_i| log-uniform [2^10, 2^{20 - args.shift}], |S_i| = 4|R_i|, 75% match, one vj_join_batch in a CUDA graph",
        "joins": joins,
        "r_rows": nr,
        "s_rows": ns,
        "l2_policy": "inputs (%.1f GiB) larger than L2" % (n * 8 / 2**30),
    }
    line = _base_line(METRIC, n / (t_batch / 1000), UNIT, args.steps, args.warmup, t_batch, "int32", cfg)
    line["join_roofline"] = {"bytes_alg_per_join": b_alg, "achieved": b_alg / (t_batch / 1000) / 1e9, "peak": peak, "unit": "GB/s", "frac": b_alg / (t_batch / 1000) / 1e9 / peak, "peak_source": src, "passes": 1}
    line["latency_ms"] = _latency(ms)
    line["gpu_launches"] = launches_fused
    line["separate_launches"] = {"ms": sum(ms_sep) / len(ms_sep), "value": n / (sum(ms_sep) / len(ms_sep) / 1000), "unit": UNIT, "kernel_launches": launches_sep, "api": "the same vj_join_batch with VJ_JOIN_BATCH_LAUNCHES, in a CUDA graph"}
    line["sequential"] = {"ms": t_seq, "value": n / (t_seq / 1000), "unit": UNIT, "api": "4096 vj_join calls back to back"}
    line["speedup_vs_sequential"] = t_seq / t_batch
    line["matches"] = m
    line["clocks"] = clocks
    print(json.dumps(line), flush=True)


def run_serve(args) -> None:
    """Serving loop: 120 join requests, int64 keys, |R| log-uniform over [2^12, 2^24],
    |S| = U{2..8} |R|, match ratio U[0.1, 1.0], probe keys uniform or Zipf(0.8) over R
    (50/50), arriving as a Poisson process; the server admits them into 4 slots under a
    150 GB budget. Compared with the serialized loop (one slot) on the same arrivals; every
    request's pairs digest must be the same in both."""
    import numpy as np
    import torch

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(SEED)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    n_req = 120
    reqs = []
    tuples = 0
    for i in range(n_req):
        nr = int(np.exp(rng.uniform(np.log(2.0**12), np.log(2.0**24))))
        ns = int(rng.integers(2, 9)) * nr
        ratio = float(rng.uniform(0.1, 1.0))
        zipf = bool(rng.random() < 0.5)
        rk = torch.empty(nr, dtype=torch.int64, device=dev)
        rp = torch.empty_like(rk)
        sk = torch.empty(ns, dtype=torch.int64, device=dev)
        sp = torch.empty_like(sk)
        vj.generate_join(SEED + i, 8, 8, nr, ns, int(ratio * (1 << 32)), rk, rp, sk, sp)
        if zipf:  # hits drawn Zipf(0.8) over R (inverse of the continuous CDF), misses random
            u = torch.rand(ns, dtype=torch.float64, generator=gen, device=dev)
            rank = torch.floor(((nr ** 0.2 - 1.0) * u + 1.0) ** 5.0).to(torch.int64).clamp_(1, nr) - 1
            perm = torch.randperm(nr, generator=gen, device=dev)
            hit = torch.rand(ns, generator=gen, device=dev) < ratio
            miss = torch.randint(-(2**62), 2**62, (ns,), generator=gen, device=dev, dtype=torch.int64)
            sk = torch.where(hit, rk[perm[rank]], miss)
            del u, rank, perm, hit, miss
        out = torch.empty((ns, 2), dtype=torch.int64, device=dev)
        reqs.append((vj.table(rk, rp, nr, 2, 8), vj.table(sk, sp, ns, 2, 8), out, ns))
        tuples += nr + ns
    torch.cuda.synchronize()

    def serve(slots: int, arrivals):
        srv = vj.Server(0, 150 << 30, slots)
        try:
            t0 = time.perf_counter()
            ids = []
            for (r, s_, out, cap), at in zip(reqs, arrivals):
                while time.perf_counter() - t0 < at:
                    pass
                ids.append(srv.submit(r, s_, out, cap))
            res = [srv.wait(i) for i in ids]
            st = srv.stats()
        finally:
            srv.close()
        assert all(x.status == 0 for x in res)
        lat = sorted((x.finish_s - x.submit_s) * 1000 for x in res)
        span = max(x.finish_s for x in res) - min(x.submit_s for x in res)
        digests = [vj.pairs_digest(q[2], x.count, 8) for q, x in zip(reqs, res)]
        return {
            "tuples_per_s": tuples / span,
            "makespan_s": span,
            "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))], "max": lat[-1]},
            "peak_running": st.peak_running,
            "peak_gb": st.peak_bytes / 1e9,
        }, [x.count for x in res], digests

    zero = [0.0] * n_req
    serve(4, zero)  # warm-up: contexts, workspaces, module loading
    sat_ser, counts_ser, dig_ser = serve(1, zero)
    sat_srv, counts_srv, dig_srv = serve(4, zero)
    assert counts_ser == counts_srv and dig_ser == dig_srv, "a result differs between the serialized loop and the server"
    mu = n_req / sat_ser["makespan_s"]  # serialized service rate, requests / s
    loads = []
    sampler = ClockSampler(0)
    sampler.start()
    for frac in (0.5, 0.9, 2.0):
        lam = frac * mu
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=n_req))
        arrivals -= arrivals[0]
        srv_r, c1, d1 = serve(4, arrivals)
        ser_r, c2, d2 = serve(1, arrivals)
        assert c1 == counts_ser and c2 == counts_ser and d1 == dig_ser and d2 == dig_ser
        loads.append({"offered_load_of_serial_rate": frac, "rate_req_per_s": lam, "server": srv_r, "serialized": ser_r})
    clocks = sampler.stop()
    cfg = {
        "workload": "serving loop: 120 int64 join requests, |R| log-uniform [2^12, 2^24], |S| = U{2..8}|R|, match U[0.1,1], keys uniform or Zipf(0.8), Poisson arrivals, 150 GB budget, 4 slots",
        "requests": n_req,
        "tuples": tuples,
        "l2_policy": "request tables (%.1f GiB in all) larger than L2" % (tuples * 16 / 2**30),
    }
    line = _base_line(METRIC, sat_srv["tuples_per_s"], UNIT, 1, 1, sat_srv["makespan_s"] * 1000, "int64", cfg)
    line["saturation"] = {"server": sat_srv, "serialized": sat_ser, "speedup": sat_ser["makespan_s"] / sat_srv["makespan_s"]}
    line["loads"] = loads
    line["clocks"] = clocks
    print(json.dumps(line), flush=True)


def run_hash_bench(args) -> None:
    """hash_func over 2^30 keys of 8, 16 and 32 uniform random bytes, FNV-1a 64 and the
    custom hash (custom_xor_hw), 64-bit chunks. Bytes = n * (key bytes + 8)."""
    import numpy as np
    import torch

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")
    oracle = _import(ROOT / "oracle" / "oracle.py", "vj_oracle")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n = 1 << (30 - args.shift)  # --shift: smaller profiling cases
    peak, src = measured_peak()
    stream = torch.cuda.current_stream()
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    results = []
    sampler = ClockSampler(0)
    sampler.start()
    for eb in (8, 16, 32):
        keys = torch.randint(-(2**62), 2**62, (n * eb // 8,), dtype=torch.int64, generator=gen, device=dev)
        hashes = torch.empty(n, dtype=torch.int64, device=dev)
        for algo in ("fnv", "custom_xor_hw"):
            call = lambda: vj.hash(keys, n, 0, eb // 8, 64, 64, algo, hashes, stream=stream)
            call()
            torch.cuda.synchronize()
            k = 4096
            words = keys[: k * eb // 8].cpu().numpy().view(np.uint32).reshape(k, eb // 4)
            want, _ = oracle.hash_elements(words, k, 0, eb // 8, 64, 64, algo)
            assert np.array_equal(hashes[:k].cpu().numpy().view(np.uint64), want.astype(np.uint64)), (eb, algo)
            ms = _timed(torch, stream, call, args.steps, args.warmup)
            t = sum(ms) / len(ms)
            gbs = n * (eb + 8) / (t / 1000) / 1e9
            results.append({"key_bytes": eb, "algo": algo, "ms": t, "GB/s": gbs, "frac": gbs / peak, "keys_per_s": n / (t / 1000)})
        del keys, hashes
        torch.cuda.empty_cache()
    clocks = sampler.stop()
    head = next(r for r in results if r["key_bytes"] == 16 and r["algo"] == "fnv")
    cfg = {"workload": f"hash 2^{30 - args.shift} keys x {{8,16,32}} B, FNV-1a 64 and custom_xor_hw, 64-bit chunks", "keys": n, "l2_policy": "inputs larger than L2"}
    line = _base_line("hash throughput (bytes read + written / s) on 1 GB300", head["GB/s"], "GB/s", args.steps, args.warmup, head["ms"], "u64", cfg)
    line["roofline"] = {"kernel": "hash_kernel", "bound": "hbm", "achieved": head["GB/s"], "peak": peak, "unit": "GB/s", "frac": head["frac"], "traffic": None, "peak_source": src}
    line["cases"] = results
    line["clocks"] = clocks
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="1/8 size workload (quick checks), same as --shift 3")
    ap.add_argument("--shift", type=int, default=0, help="divide both table sizes by 2^shift (profiling cases)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="time the planner's own plan, without the autotuner")
    ap.add_argument("--workload", default="join", choices=["join", "join-small", "join-skew", "join-batch", "serve", "hash"], help="join: the 2^27 x 2^29 int64 join (default); the others print their own line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "ours" and args.workload != "join":
        {"join-small": run_small_join, "join-skew": run_skew_join, "join-batch": run_batch_join, "serve": run_serve, "hash": run_hash_bench}[args.workload](args)
        return
    if args.small:
        args.shift = max(args.shift, 3)
    args.small = args.shift > 0
    cfg = workload(args.shift)
    if args.impl == "reference":
        run_reference(args, cfg)
        return

    import numpy as np
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    graft = _import(ROOT / "__graft_entry__.py", "graft_entry")
    graft.build()
    vj = _import(PKG / "vj.py", "vj")

    nr, ns = cfg["r_rows"], cfg["s_rows"]
    thr = int(round(cfg["match_ratio"] * (1 << 32)))
    seed = SEED + rank
    rk = torch.empty(nr, dtype=torch.int64, device=dev)
    rp = torch.empty(nr, dtype=torch.int64, device=dev)
    sk = torch.empty(ns, dtype=torch.int64, device=dev)
    sp = torch.empty(ns, dtype=torch.int64, device=dev)
    vj.generate_join(seed, 8, 8, nr, ns, thr, rk, rp, sk, sp)
    expect = vj.generate_join_expect(seed, nr, ns, thr)
    cap = ns
    out = torch.empty((cap, 2), dtype=torch.int64, device=dev)
    ctx = vj.Context(local)
    ctx.set_profiling(True)
    t_r = vj.table(rk, rp, nr, 2, 8)
    t_s = vj.table(sk, sp, ns, 2, 8)
    stream = torch.cuda.current_stream()

    # the autotuner picks the plan (radix split, table size, table kind) for this shape
    # class before the timed region; the timed joins are automatic and use it
    tuned_opts, tuned_ms = (None, None) if args.no_tune else ctx.tune(t_r, t_s, out, cap, stream=stream)

    def step():
        return ctx.join(t_r, t_s, None, out=out, capacity=cap, stream=stream)

    for _ in range(args.warmup):
        res = step()
    # correctness of the benchmarked configuration: count + digest against the generator
    assert res.count == expect[0], (res.count, expect)
    assert vj.pairs_digest(out, res.count, 8) == (expect[1], expect[2]), "digest mismatch"

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    events = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    profiles = []
    events[0].record(stream)
    for i in range(args.steps):
        res = step()
        events[i + 1].record(stream)
        profiles.append(ctx.last_profile().as_dict())
    torch.cuda.synchronize()
    clocks = sampler.stop()
    step_ms = [events[i].elapsed_time(events[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(events[0].elapsed_time(events[-1]), dev)
    if world > 1:
        dist.barrier()
    value = job_rate(nr + ns, args.steps, world, total_ms)

    # p50/p99 over at least LATENCY_SAMPLES joins: the timed steps, then more joins after
    # the timed region (they do not enter `value`)
    lat_ms = list(step_ms)
    extra = max(0, LATENCY_SAMPLES - args.steps)
    if extra:
        lev = [torch.cuda.Event(enable_timing=True) for _ in range(extra + 1)]
        lev[0].record(stream)
        for i in range(extra):
            step()
            lev[i + 1].record(stream)
        torch.cuda.synchronize()
        lat_ms += [lev[i].elapsed_time(lev[i + 1]) for i in range(extra)]

    # ---- roofline of the dominant kernel (stage events recorded by the library)
    peak, peak_src = measured_peak()
    w_k, w_p = cfg["key_bytes"], cfg["payload_bytes"]
    w = w_k + w_p
    n = nr + ns
    m = expect[0]
    prof0 = profiles[0]
    passes = prof0["passes"]

    def avg(key, idx=None):
        vals = [p[key][idx] if idx is not None else p[key] for p in profiles]
        return sum(vals) / len(vals)

    kernels = {}
    for p in range(passes):
        # pass 1 counts keys; a second pass counts the 2-byte buckets pass 1 wrote per row
        kernels[f"histogram_kernel (pass {p + 1})"] = (avg("ms_histogram", p), n * (w_k if p == 0 else 2))
        kernels[f"scatter_kernel (pass {p + 1})"] = (avg("ms_scatter", p), n * 2 * w)
    kernels["probe_kernel"] = (avg("ms_probe"), n * w + m * 2 * w_p)
    # dominant kernel kind by total time per join
    kinds = {}
    for name, (ms, byts) in kernels.items():
        kind = name.split(" ")[0]
        kinds.setdefault(kind, []).append((ms, byts))
    dom_kind = max(kinds, key=lambda k: sum(x[0] for x in kinds[k]))
    launches = kinds[dom_kind]
    ms_per_launch = sum(x[0] for x in launches) / len(launches)
    bytes_per_launch = sum(x[1] for x in launches) / len(launches)
    achieved = bytes_per_launch / (ms_per_launch / 1000.0) / 1e9
    # DRAM bytes per launch of this kernel from the committed ncu summary of the same build
    # (captured at 1/8 size and scaled by rows); only the full-size workload has one
    traffic = profiled_traffic(dom_kind) if args.shift == 0 and not args.small else None
    roofline = {
        "kernel": dom_kind,
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": traffic,
        "peak_source": peak_src,
        "launches_per_step": len(launches),
        "bytes_per_launch": bytes_per_launch,
        "ms_per_launch": ms_per_launch,
    }
    b_alg = n * (passes * (w_k + 2 * w) + w) + m * 2 * w_p
    ms_step = total_ms / args.steps
    join_roofline = {
        "bytes_alg_per_join": b_alg,
        "achieved": b_alg / (ms_step / 1000.0) / 1e9,
        "peak": peak,
        "unit": "GB/s",
        "frac": b_alg / (ms_step / 1000.0) / 1e9 / peak,
        "formula": "(|R|+|S|)*(P*(w_k+2w)+w) + M*2*w_p",
    }
    stages = {name: round(ms, 4) for name, (ms, _) in kernels.items()}
    stages["total_profiled"] = avg("ms_total")

    # ---- end to end through the C ABI with host buffers
    del out
    e2e = None
    if args.no_e2e:
        del rk, rp, sk, sp
    else:
        e2e = run_e2e(args, ctx, vj, torch, stream, dev, world, rk, rp, sk, sp, nr, ns, m, w, w_p)
        del rk, rp, sk, sp

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        oracle = _import(ROOT / "oracle" / "oracle.py", "vj_oracle")
        oracle.build()
        cpu = cpu_baseline(oracle, args.small)

    cfg = dict(cfg)
    cfg["radix_passes"] = passes
    cfg["radix_bits"] = prof0["radix_bits"][:passes]
    cfg["build_rows_per_table"] = prof0["build_rows"]
    cfg["parallelism"] = "replicas" if world > 1 else "single GPU"
    cfg["tables"] = prof0.get("tables")
    if tuned_opts is not None:
        cfg["tuned_plan"] = vj.options_dict(tuned_opts)
        cfg["tuner_best_ms"] = tuned_ms
    lat = sorted(lat_ms)

    def pct(q):
        k = min(len(lat) - 1, max(0, int(round(q * (len(lat) - 1)))))
        return lat[k]

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int64",
            "data": "synthetic (seeded counter-based generator; R unique u64 keys, S half from R, half from a disjoint range)",
            "config": cfg,
            "roofline": roofline,
            "join_roofline": join_roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(sum(p["kernel_launches"] for p in profiles)),
            "clocks": clocks,
            "latency_ms": {"p50": pct(0.5), "p99": pct(0.99), "min": lat[0], "max": lat[-1], "samples": len(lat)},
            "stages_ms": stages,
            "matches": m,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
