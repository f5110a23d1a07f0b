"""The reference's C++ API names (include/vj_compat.hpp), compiled into a driver that calls
them like the reference's own drivers, checked against the CPU oracle."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA = Path("/usr/local/cuda")


def build_driver(tmp: Path, hash_bits: int, chunk_bits: int) -> Path:
    exe = tmp / f"compat_driver_h{hash_bits}_c{chunk_bits}"
    lib = ROOT / "vectorized-join_gb300" / "lib"
    cmd = [
        "g++",
        "-std=c++17",
        "-O1",
        f"-DHASH_BITS={hash_bits}",
        f"-DHASH_CHUNK_BITS={chunk_bits}",
        "-I",
        str(ROOT / "include"),
        "-I",
        str(CUDA / "include"),
        str(ROOT / "tests" / "compat" / "compat_driver.cpp"),
        "-o",
        str(exe),
        "-L",
        str(lib),
        "-lvj",
        f"-Wl,-rpath,{lib}",
        "-L",
        str(CUDA / "lib64"),
        "-lcudart",
        f"-Wl,-rpath,{CUDA / 'lib64'}",
    ]
    subprocess.check_call(cmd)
    return exe


def test_compat_header_compiles(vjlib, tmp_path):
    # compile only (no GPU needed): every reference name resolves against libvj.so
    build_driver(tmp_path, 64, 64)


@pytest.mark.gpu
@pytest.mark.parametrize("hash_bits,chunk_bits", [(64, 64), (32, 32)])
def test_compat_driver_matches_oracle(vjlib, cuda, oracle, tmp_path, hash_bits, chunk_bits):
    exe = build_driver(tmp_path, hash_bits, chunk_bits)
    rng = np.random.default_rng(hash_bits + chunk_bits)
    cc, nr, ns = 2, 3000, 12000
    rk = rng.integers(0, 40, size=(nr, cc), dtype=np.uint64)
    sk = rng.integers(0, 40, size=(ns, cc), dtype=np.uint64)
    rp = np.arange(1, nr + 1, dtype=np.uint64)
    sp = np.arange(1, ns + 1, dtype=np.uint64)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([cc, nr, ns], np.uint64).tofile(f)
        rk.tofile(f)
        rp.tofile(f)
        sk.tofile(f)
        sp.tofile(f)
    subprocess.check_call([str(exe), str(fin), str(fout)])
    raw = np.fromfile(fout, dtype=np.uint64)
    rec, i = {}, 1
    while i < raw.size:
        tag, n = int(raw[i]), int(raw[i + 1])
        rec[tag] = raw[i + 2 : i + 2 + n]
        i += 2 + n
    flags = rec[9]
    assert flags[0] == 0  # hash_func status
    assert flags[1] == vjlib.VJ_ERR_INVALID_ARGUMENT  # unknown algorithm "xor_hw"
    assert flags[2] == 0  # partition_gpu status
    assert flags[3] == 0 and flags[4] == 0 and flags[6] == 0
    # hashes
    words = np.ascontiguousarray(rk).view(np.uint32)
    want_h, _ = oracle.hash_elements(words, nr, 0, cc * 8 // (chunk_bits // 8), chunk_bits, hash_bits, "fnv")
    assert np.array_equal(rec[1], want_h.astype(np.uint64))
    # partition: exact histogram/offsets, bucket multisets, hashes moved with their rows
    hist, offs, _ = oracle.partition(want_h, 4, 6)
    assert np.array_equal(rec[2], hist) and np.array_equal(rec[3], offs)
    bucket = (want_h.astype(np.uint64) >> np.uint64(4)) & np.uint64(63)
    for b in range(64):
        lo, hi = int(offs[b]), int(offs[b] + hist[b])
        assert np.array_equal(np.sort(rec[4][lo:hi]), np.sort(rp[bucket == b]))
    moved = rec[5][np.argsort(rec[4])]
    assert np.array_equal(moved, want_h.astype(np.uint64))
    # joins
    cnt, want, _ = oracle.join(rk, rp, sk, sp)
    assert flags[5] == cnt
    for tag in (6, 7, 8):
        got = rec[tag].reshape(-1, 2)
        got = got[np.lexsort((got[:, 1], got[:, 0]))]
        assert got.shape[0] == cnt, tag
        assert np.array_equal(got, want), tag
