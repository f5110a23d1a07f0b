"""Generates the committed golden fixtures of tests/golden/ (run in a container that has the
reference sources, after oracle/ref_build.sh):

    python tests/golden/make_golden.py

hash_kat.npz   Known-answer vectors of all 13 hash algorithms x hash bits {32, 64} x chunk
               bits {8, 32, 64, 128} over fixed byte patterns (zeros, 0xFF, a byte ramp that
               covers the sign-extended char path, alternating words) and seeded random
               bytes, for several element sizes and chunk offsets. Values come from the
               CPU oracle; every element whose value does not depend on an out-of-range
               shift is also checked against the reference's own kernel source run as host
               code (oracle/_ref/ref_hash_host_*), and the script stops on any difference.
               `ub_*` marks the elements that rest on the shift clamp (pinned on the GPU by
               oracle/ref_gpu_check.py).
join_cases.npz Small join inputs (u64 key columns + u64 primary keys, like db_table) with
               the sorted (r_pk, s_pk) pairs the reference's JoinProvider::join_cpu
               produces (oracle/_ref/ref_join_cpu): duplicates on both sides, empty sides,
               no matches, multi-column keys.
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
N_ELEMS = 48

# element sizes in bytes tried for each chunk width (must be multiples of the chunk size)
ELEMENT_BYTES = {8: [1, 3, 8, 16, 32], 32: [4, 8, 12, 16, 32], 64: [8, 16, 24, 32], 128: [16, 32, 48]}


def pattern_bytes(nbytes_per_elem: int, n: int, seed: int) -> np.ndarray:
    """n elements: [zeros, 0xFF, byte ramp, alternating words, random ...]."""
    total = n * nbytes_per_elem
    rng = np.random.default_rng(seed)
    buf = rng.integers(0, 256, size=total, dtype=np.uint8)
    e = nbytes_per_elem
    buf[0:e] = 0
    buf[e : 2 * e] = 0xFF
    buf[2 * e : 3 * e] = (np.arange(e) * 37 + 0x80) & 0xFF
    ramp = np.arange(8 * e, dtype=np.int64) & 0xFF
    buf[3 * e : 11 * e] = ramp
    alt = np.frombuffer(np.array([0xAAAAAAAA, 0x55555555] * (e + 1), dtype=np.uint32).tobytes(), dtype=np.uint8)
    buf[11 * e : 12 * e] = alt[:e]
    small = rng.integers(0, 4, size=4 * e, dtype=np.uint8)
    buf[12 * e : 16 * e] = small  # small lane values keep the *_shift offsets in range
    return buf


def make_hash_kat(tmp: Path) -> dict:
    arrays = {}
    manifest = []
    checked = unpinned = 0
    for cb in (8, 32, 64, 128):
        cbytes = cb // 8
        for eb in ELEMENT_BYTES[cb]:
            ec = eb // cbytes
            inp = pattern_bytes(eb, N_ELEMS, seed=1000 * cb + eb)
            arrays[f"in_c{cb}_e{eb}"] = inp
            for off in sorted({0, 1, ec // 2}):
                if off > ec:
                    continue
                for hb in (32, 64):
                    for algo in O.ALGORITHMS:
                        h, ub = O.hash_elements(inp, N_ELEMS, off, ec, cb, hb, algo)
                        ref = O.ref_hash_host(algo, inp, N_ELEMS, off, ec, cb, hb, tmp)
                        if ref is None:
                            raise SystemExit("oracle/_ref is not built; run oracle/ref_build.sh first")
                        bad = (h != ref) & ~ub
                        if bad.any():
                            raise SystemExit(f"oracle differs from the reference source: hb={hb} cb={cb} eb={eb} off={off} {algo} at {np.nonzero(bad)[0][:5]}")
                        checked += int((~ub).sum())
                        unpinned += int(ub.sum())
                        key = f"h{hb}_c{cb}_e{eb}_o{off}_{algo}"
                        arrays[key] = h
                        if ub.any():
                            arrays["ub_" + key] = ub.astype(np.uint8)
                        manifest.append([hb, cb, eb, off, algo])
    arrays["manifest"] = np.frombuffer(json.dumps(manifest).encode(), dtype=np.uint8)
    np.savez_compressed(OUT / "hash_kat.npz", **arrays)
    return {"cases": len(manifest), "elements_checked_against_reference_source": checked, "elements_on_shift_clamp": unpinned}


def make_join_cases(tmp: Path) -> dict:
    rng = np.random.default_rng(20240611)
    cases = {}
    specs = [
        # (name, nr, ns, columns, key domain)
        ("fk_small", 200, 800, 1, None),
        ("dups_both", 300, 1200, 1, 40),
        ("dups_heavy", 64, 2000, 1, 3),
        ("multi2", 256, 1024, 2, 5),
        ("multi3", 128, 700, 3, 3),
        ("multi4", 100, 300, 4, 2),
        ("no_match", 150, 400, 1, None),
        ("empty_r", 0, 100, 1, 10),
        ("empty_s", 100, 0, 1, 10),
        ("single", 1, 1, 1, 1),
        ("extreme_values", 50, 200, 1, None),
    ]
    meta = {}
    for name, nr, ns, cols, dom in specs:
        if name == "fk_small":
            rk = rng.permutation(np.arange(10**6, dtype=np.uint64))[:nr].reshape(nr, 1)
            sk = rk[rng.integers(0, nr, size=ns)]
        elif name == "no_match":
            rk = rng.integers(0, 2**40, size=(nr, cols), dtype=np.uint64)
            sk = rng.integers(2**41, 2**42, size=(ns, cols), dtype=np.uint64)
        elif name == "extreme_values":
            vals = np.array([0, 1, 2**32 - 1, 2**32, 2**63, 2**64 - 1, 0xFFFFFFFF00000000, 0x00000000FFFFFFFF], dtype=np.uint64)
            rk = vals[rng.integers(0, vals.size, size=nr)].reshape(nr, 1)
            sk = vals[rng.integers(0, vals.size, size=ns)].reshape(ns, 1)
        else:
            rk = rng.integers(0, dom, size=(nr, cols), dtype=np.uint64)
            sk = rng.integers(0, dom, size=(ns, cols), dtype=np.uint64)
        rpk = np.arange(1, nr + 1, dtype=np.uint64)  # primary keys as the reference generates them
        spk = np.arange(1, ns + 1, dtype=np.uint64)
        ref = O.ref_join_cpu(rk, rpk, sk, spk, tmp)
        if ref is None:
            raise SystemExit("oracle/_ref is not built; run oracle/ref_build.sh first")
        cnt, pairs, _ = O.join(rk, rpk, sk, spk, threads=4)
        if cnt != len(ref) or not np.array_equal(pairs, ref):
            raise SystemExit(f"oracle join differs from the reference join_cpu on {name}")
        cases[f"{name}_r_keys"] = np.ascontiguousarray(rk)
        cases[f"{name}_s_keys"] = np.ascontiguousarray(sk)
        cases[f"{name}_pairs"] = ref
        meta[name] = {"nr": nr, "ns": ns, "columns": cols, "matches": int(len(ref))}
    cases["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT / "join_cases.npz", **cases)
    return meta


def main():
    O.build()
    with tempfile.TemporaryDirectory() as d:
        tmp = Path(d)
        print("hash_kat:", make_hash_kat(tmp))
        print("join_cases:", make_join_cases(tmp))


if __name__ == "__main__":
    main()
