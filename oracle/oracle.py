"""ctypes loader for the CPU oracle (oracle/vj_oracle.c).

TEST INFRASTRUCTURE ONLY: tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module as the checker. Nothing in the library imports it.

The oracle restates the reference's hash kernels (src/hash/hash.cu:84-505), its radix
partition (src/join/join_provider.cu:315-380) and its chained-table build/probe
(src/join/join_provider.cu:382-442) in C; see the header of vj_oracle.c.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

# Same order as the reference dispatcher, src/hash/hash.cu:515-541.
ALGORITHMS = [
    "fnv",
    "custom_xor",
    "custom_xor_shift",
    "custom_xor_hw",
    "custom_mult_xor_shift",
    "custom_n_mult_xor_shift",
    "custom_mult_xor_hw",
    "custom_mult",
    "custom_mult_shift",
    "custom_mult_hw",
    "custom_add",
    "custom_add_shift",
    "custom_add_hw",
]
SHIFT_ALGORITHMS = {"custom_xor_shift", "custom_add_shift", "custom_mult_shift", "custom_mult_xor_shift", "custom_n_mult_xor_shift"}


def build(force: bool = False) -> Path:
    """Compile vj_oracle.c into liboracle.so (gcc, plain C, portable flags)."""
    src = HERE / "vj_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        tmp = LIB_PATH.with_suffix(".so.tmp%d" % os.getpid())
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref(reference_root: str | None) -> bool:
    """Build oracle/_ref from the reference sources under reference_root (the checkout of
    vgerber/vectorized-join) when they are there. Returns True when the reference checkers
    exist afterwards."""
    if reference_root and Path(reference_root, "src", "hash", "hash.cu").exists():
        subprocess.check_call(["bash", str(HERE / "ref_build.sh"), reference_root])
    return (REF_DIR / "ref_join_cpu").exists()


_lib = None

u64 = ctypes.c_uint64
vp = ctypes.c_void_p
i32 = ctypes.c_int


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.vjo_hash_element.restype = u64
        L.vjo_hash_element.argtypes = [vp, i32, i32, i32, i32, i32, vp]
        L.vjo_hash.restype = None
        L.vjo_hash.argtypes = [vp, u64, i32, i32, i32, i32, i32, vp, vp]
        L.vjo_partition.restype = None
        L.vjo_partition.argtypes = [vp, i32, u64, i32, i32, vp, vp, vp]
        L.vjo_pair_digest.restype = u64
        L.vjo_pair_digest.argtypes = [u64, u64]
        L.vjo_join.restype = u64
        L.vjo_join.argtypes = [vp, vp, u64, vp, vp, u64, i32, i32, i32, i32, i32, vp, u64, vp, vp]
        L.vjo_join_nested.restype = u64
        L.vjo_join_nested.argtypes = [vp, vp, u64, vp, vp, u64, i32, vp, u64]
        L.vjo_sort_pairs.restype = None
        L.vjo_sort_pairs.argtypes = [vp, u64]
        L.vjo_rng.restype = u64
        L.vjo_rng.argtypes = [u64, u64, u64]
        L.vjo_ukey64.restype = u64
        L.vjo_ukey64.argtypes = [u64, u64]
        L.vjo_ukey31.restype = ctypes.c_uint32
        L.vjo_ukey31.argtypes = [u64, u64]
        L.vjo_gen_join.restype = u64
        L.vjo_gen_join.argtypes = [u64, i32, u64, u64, u64, vp, vp, vp, vp, vp]
        L.vjo_gen_join_expect.restype = u64
        L.vjo_gen_join_expect.argtypes = [u64, u64, u64, u64, vp, vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(vp)


def algo_id(name: str) -> int:
    return ALGORITHMS.index(name)


def hash_elements(elements: np.ndarray, n: int, chunk_offset: int, element_chunks: int, chunk_bits: int, hash_bits: int, algo: str | int):
    """hash_func over a byte buffer (src/hash/hash.cu:507-557). Returns (hashes, ub) where
    ub marks elements whose value depends on an out-of-range shift."""
    algo = algo_id(algo) if isinstance(algo, str) else int(algo)
    buf = np.ascontiguousarray(elements).view(np.uint8)
    need = n * element_chunks * (chunk_bits // 8)
    assert buf.size >= need, (buf.size, need)
    out = np.zeros(n, dtype=np.uint64 if hash_bits == 64 else np.uint32)
    ub = np.zeros(n, dtype=np.uint8)
    lib().vjo_hash(_ptr(buf), n, chunk_offset, element_chunks, chunk_bits, hash_bits, algo, _ptr(out), _ptr(ub))
    return out, ub.astype(bool)


def partition(hashes: np.ndarray, radix_shift: int, radix_bits: int):
    """One radix pass (src/join/join_provider.cu:610-661): (histogram, offsets, stable perm)."""
    hashes = np.ascontiguousarray(hashes)
    hb = 64 if hashes.dtype == np.uint64 else 32
    bins = 1 << radix_bits
    hist = np.zeros(bins, np.uint64)
    offs = np.zeros(bins, np.uint64)
    perm = np.zeros(max(1, hashes.size), np.uint64)
    lib().vjo_partition(_ptr(hashes), hb, hashes.size, radix_shift, radix_bits, _ptr(hist), _ptr(offs), _ptr(perm))
    return hist, offs, perm[: hashes.size]


def _key_words(keys: np.ndarray) -> tuple[np.ndarray, int]:
    """Keys as rows of 32-bit words: u32 [n] -> kw 1, u64 [n] -> kw 2, u64 [n, c] -> kw 2c."""
    keys = np.ascontiguousarray(keys)
    n = keys.shape[0]
    kw = keys.itemsize // 4 * (keys.shape[1] if keys.ndim > 1 else 1)
    words = keys.view(np.uint32).reshape(n, kw) if n else np.zeros((0, kw), np.uint32)
    return np.ascontiguousarray(words), kw


def join(r_keys, r_pay, s_keys, s_pay, hash_bits=64, algo="fnv", radix_bits=8, threads=None, want_pairs=True):
    """Multiset equi-join (build R, probe S). Returns (count, pairs sorted [M, 2] u64 or None,
    (digest_sum, digest_xor))."""
    rw, kw = _key_words(r_keys)
    sw, kw2 = _key_words(s_keys)
    assert kw == kw2
    r_pay = np.ascontiguousarray(r_pay, dtype=np.uint64)
    s_pay = np.ascontiguousarray(s_pay, dtype=np.uint64)
    if threads is None:
        threads = os.cpu_count() or 1
    algo = algo_id(algo) if isinstance(algo, str) else int(algo)
    ds = ctypes.c_uint64(0)
    dx = ctypes.c_uint64(0)
    L = lib()
    count = L.vjo_join(_ptr(rw), _ptr(r_pay), rw.shape[0], _ptr(sw), _ptr(s_pay), sw.shape[0], kw, hash_bits, algo, radix_bits, threads, None, 0, ctypes.byref(ds), ctypes.byref(dx))
    pairs = None
    if want_pairs:
        pairs = np.zeros((max(1, count), 2), np.uint64)
        count2 = L.vjo_join(_ptr(rw), _ptr(r_pay), rw.shape[0], _ptr(sw), _ptr(s_pay), sw.shape[0], kw, hash_bits, algo, radix_bits, threads, _ptr(pairs), count, None, None)
        assert count2 == count
        pairs = pairs[:count]
    return int(count), pairs, (int(ds.value), int(dx.value))


def join_nested(r_keys, r_pay, s_keys, s_pay):
    """The literal nested-loop algorithm of join_cpu (src/join/join_provider.cuh:249-282)."""
    rw, kw = _key_words(r_keys)
    sw, _ = _key_words(s_keys)
    r_pay = np.ascontiguousarray(r_pay, dtype=np.uint64)
    s_pay = np.ascontiguousarray(s_pay, dtype=np.uint64)
    L = lib()
    m = L.vjo_join_nested(_ptr(rw), _ptr(r_pay), rw.shape[0], _ptr(sw), _ptr(s_pay), sw.shape[0], kw, None, 0)
    pairs = np.zeros((max(1, m), 2), np.uint64)
    L.vjo_join_nested(_ptr(rw), _ptr(r_pay), rw.shape[0], _ptr(sw), _ptr(s_pay), sw.shape[0], kw, _ptr(pairs), m)
    return sort_pairs(pairs[:m])


def sort_pairs(pairs: np.ndarray) -> np.ndarray:
    pairs = np.ascontiguousarray(pairs, dtype=np.uint64).reshape(-1, 2)
    if pairs.shape[0] > 1:
        order = np.lexsort((pairs[:, 1], pairs[:, 0]))
        pairs = np.ascontiguousarray(pairs[order])
    return pairs


def pair_digest(r: np.ndarray, s: np.ndarray) -> tuple[int, int]:
    """(sum, xor) of the per-pair digest over arrays of payloads (numpy restatement of
    vjo_pair_digest, checked against the C one in the tests)."""
    def fmix(z):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))

    r = np.asarray(r, dtype=np.uint64)
    s = np.asarray(s, dtype=np.uint64)
    with np.errstate(over="ignore"):
        d = fmix(r ^ fmix(s + np.uint64(0x9E3779B97F4A7C15)))
    return int(np.sum(d, dtype=np.uint64)), int(np.bitwise_xor.reduce(d)) if d.size else 0


def match_threshold(ratio: float) -> int:
    """Probe row j matches when (rng >> 32) < threshold."""
    return int(round(min(max(ratio, 0.0), 1.0) * (1 << 32)))


def gen_join(seed: int, key_bytes: int, nr: int, ns: int, match_ratio: float):
    """Seeded join workload (see vjo_gen_join). Returns dict with r_keys, r_pay, s_keys,
    s_pay (u64 payloads = row ids), r_of_s and the match count."""
    kt = np.uint64 if key_bytes == 8 else np.uint32
    rk = np.zeros(max(1, nr), kt)
    sk = np.zeros(max(1, ns), kt)
    rp = np.zeros(max(1, nr), np.uint64)
    sp = np.zeros(max(1, ns), np.uint64)
    ros = np.zeros(max(1, ns), np.uint64)
    m = lib().vjo_gen_join(seed, key_bytes, nr, ns, match_threshold(match_ratio), _ptr(rk), _ptr(rp), _ptr(sk), _ptr(sp), _ptr(ros))
    return dict(r_keys=rk[:nr], r_pay=rp[:nr], s_keys=sk[:ns], s_pay=sp[:ns], r_of_s=ros[:ns], matches=int(m))


def gen_join_expect(seed: int, nr: int, ns: int, match_ratio: float):
    """(count, digest_sum, digest_xor) of the join of gen_join's tables, without joining."""
    ds = ctypes.c_uint64(0)
    dx = ctypes.c_uint64(0)
    m = lib().vjo_gen_join_expect(seed, nr, ns, match_threshold(match_ratio), ctypes.byref(ds), ctypes.byref(dx))
    return int(m), int(ds.value), int(dx.value)


# ------------------------------------------------------------------ reference checkers


def ref_hash_host(algo: str, elements: np.ndarray, n: int, chunk_offset: int, element_chunks: int, chunk_bits: int, hash_bits: int, tmpdir: Path) -> np.ndarray | None:
    """Run the reference's own hash kernel source as host code (oracle/_ref); None if absent."""
    exe = REF_DIR / f"ref_hash_host_h{hash_bits}_c{chunk_bits}"
    if not exe.exists():
        return None
    tmpdir = Path(tmpdir)
    fin = tmpdir / "ref_in.bin"
    fout = tmpdir / "ref_out.bin"
    np.ascontiguousarray(elements).view(np.uint8)[: n * element_chunks * chunk_bits // 8].tofile(fin)
    subprocess.check_call([str(exe), algo, str(n), str(chunk_offset), str(element_chunks), str(fin), str(fout)])
    return np.fromfile(fout, dtype=np.uint64 if hash_bits == 64 else np.uint32, count=n)


def ref_join_cpu(r_cols: np.ndarray, r_pk: np.ndarray, s_cols: np.ndarray, s_pk: np.ndarray, tmpdir: Path) -> np.ndarray | None:
    """The reference's JoinProvider::join_cpu on host db_tables (u64 key columns, u64 pks).
    Returns the sorted [M, 2] pairs or None if the checker is absent."""
    exe = REF_DIR / "ref_join_cpu"
    if not exe.exists():
        return None
    r_cols = np.ascontiguousarray(r_cols, dtype=np.uint64)
    s_cols = np.ascontiguousarray(s_cols, dtype=np.uint64)
    r_cols = r_cols if r_cols.ndim == 2 else r_cols.reshape(-1, 1)
    s_cols = s_cols if s_cols.ndim == 2 else s_cols.reshape(-1, 1)
    cc = max(r_cols.shape[1], s_cols.shape[1])
    tmpdir = Path(tmpdir)
    fin = tmpdir / "ref_join_in.bin"
    fout = tmpdir / "ref_join_out.bin"
    with open(fin, "wb") as f:
        np.array([cc, r_pk.size, s_pk.size], np.uint64).tofile(f)
        r_cols.tofile(f)
        np.ascontiguousarray(r_pk, np.uint64).tofile(f)
        s_cols.tofile(f)
        np.ascontiguousarray(s_pk, np.uint64).tofile(f)
    subprocess.check_call([str(exe), str(fin), str(fout)])
    raw = np.fromfile(fout, dtype=np.uint64)
    m = int(raw[0])
    return sort_pairs(raw[1 : 1 + 2 * m].reshape(m, 2))
