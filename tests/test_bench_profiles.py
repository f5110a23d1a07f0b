"""bench.py's roofline `traffic` comes from the committed ncu summaries in profiles/: each
dominant-kernel candidate has a per-launch DRAM figure at full size, close to its
algorithmic bytes (2^27 + 2^29 int64 rows, 2^28 pairs)."""
from __future__ import annotations

import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_lines_match_algorithmic_bytes():
    bench = load_bench()
    n, w, w_p, m = (1 << 27) + (1 << 29), 16, 8, 1 << 28
    scatter = bench.profiled_traffic("scatter_kernel")
    probe = bench.profiled_traffic("probe_kernel")
    hist = bench.profiled_traffic("histogram_kernel")
    assert scatter and probe and hist
    # scatter: read and write every row once per pass
    assert 0.95 <= scatter / (n * 2 * w) <= 1.3
    # probe: read both sides' partitioned rows once, write the pairs
    assert 0.95 <= probe / (n * w + m * 2 * w_p) <= 1.3
    # histogram: mean of pass 1 (8-byte keys) and pass 2 (u16 bucket ids)
    assert 0.9 <= hist / (n * (8 + 2) / 2) <= 1.3
    assert bench.profiled_traffic("no_such_kernel") is None
