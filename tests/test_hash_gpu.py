"""vj_hash on the GPU against the golden vectors and the oracle (bit-exact)."""
from __future__ import annotations

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(a: np.ndarray, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)


def run_hash(vjlib, dev, data: np.ndarray, n, off, ec, cb, hb, algo, byte_offset=0):
    import torch

    buf = to_dev(np.concatenate([np.zeros(byte_offset, np.uint8), data.view(np.uint8)]), dev)
    out = torch.zeros(max(n, 1), dtype=torch.int64 if hb == 64 else torch.int32, device=dev)
    vjlib.hash(buf.data_ptr() + byte_offset, n, off, ec, cb, hb, algo, out)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint64 if hb == 64 else np.uint32)[:n]


def test_golden_vectors_bit_exact(vjlib, cuda, hash_kat):
    manifest = json.loads(bytes(hash_kat["manifest"]).decode())
    for hb, cb, eb, off, algo in manifest:
        inp = hash_kat[f"in_c{cb}_e{eb}"]
        want = hash_kat[f"h{hb}_c{cb}_e{eb}_o{off}_{algo}"]
        got = run_hash(vjlib, cuda, inp, want.size, off, eb // (cb // 8), cb, hb, algo)
        assert np.array_equal(got, want), (hb, cb, eb, off, algo, np.nonzero(got != want)[0][:5])


@pytest.mark.parametrize("eb", [8, 16, 32])
@pytest.mark.parametrize("algo", ["fnv", "custom_xor_hw", "custom_mult_xor_shift", "custom_add_hw"])
def test_vector_paths_vs_oracle(vjlib, cuda, oracle, eb, algo):
    n = 70001  # not a multiple of the unrolled block step
    data = np.random.default_rng(eb).integers(0, 256, size=n * eb, dtype=np.uint8)
    for cb in (8, 32, 64, 128):
        if eb % (cb // 8):
            continue
        ec = eb // (cb // 8)
        for hb in (32, 64):
            want, _ = oracle.hash_elements(data, n, 0, ec, cb, hb, algo)
            got = run_hash(vjlib, cuda, data, n, 0, ec, cb, hb, algo)
            assert np.array_equal(got, want), (cb, hb)


def test_generic_path_offsets_and_odd_sizes(vjlib, cuda, oracle):
    rng = np.random.default_rng(2)
    for cb, ec, off in [(8, 3, 0), (8, 7, 2), (32, 5, 1), (64, 3, 2), (128, 3, 1), (64, 2, 1), (32, 8, 5)]:
        n = 5003
        data = rng.integers(0, 256, size=n * ec * cb // 8, dtype=np.uint8)
        for algo in ("fnv", "custom_mult_hw", "custom_n_mult_xor_shift", "custom_xor_shift"):
            want, _ = oracle.hash_elements(data, n, off, ec, cb, 64, algo)
            got = run_hash(vjlib, cuda, data, n, off, ec, cb, 64, algo)
            assert np.array_equal(got, want), (cb, ec, off, algo)


def test_unaligned_base_uses_generic_path(vjlib, cuda, oracle):
    # 8-byte elements starting 4 bytes past a 16-byte boundary (chunk 32 alignment only)
    n = 3001
    data = np.random.default_rng(4).integers(0, 256, size=n * 8, dtype=np.uint8)
    want, _ = oracle.hash_elements(data, n, 0, 2, 32, 64, "fnv")
    got = run_hash(vjlib, cuda, data, n, 0, 2, 32, 64, "fnv", byte_offset=4)
    assert np.array_equal(got, want)


def test_misaligned_chunk_rejected(vjlib, cuda):
    import torch

    buf = torch.zeros(64, dtype=torch.uint8, device=cuda)
    out = torch.zeros(4, dtype=torch.int64, device=cuda)
    with pytest.raises(vjlib.VjError) as e:
        vjlib.hash(buf.data_ptr() + 4, 2, 0, 1, 64, 64, "fnv", out)
    assert e.value.status == vjlib.VJ_ERR_INVALID_ARGUMENT
