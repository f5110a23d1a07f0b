"""The reference's own hash kernels (src/hash/hash.cu compiled unchanged for sm_103a by
oracle/ref_build.sh) run on the GPU against the golden known-answer vectors
(tests/golden/hash_kat.npz), which the library's kernels are checked against in
test_hash_gpu.py. This pins the golden values of the *_shift variants whose shift amounts
fall outside [0, hash bits) -- undefined in C++, so only the reference's compiled code can
say what they are. The cubins are built where the reference sources are; without them the
test is skipped (tests/golden/ref_gpu_check.json is the record of a run on a GB300)."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_reference_hash_kernels_give_the_golden_vectors(cuda):
    spec = importlib.util.spec_from_file_location("ref_gpu_check", ROOT / "oracle" / "ref_gpu_check.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ref_gpu_check"] = mod
    spec.loader.exec_module(mod)
    cubins = [mod.REF / f"ref_h{hb}_c{cb}.cubin" for hb in (32, 64) for cb in (8, 32, 64, 128)]
    if not all(p.exists() for p in cubins):
        pytest.skip("reference cubins absent (oracle/_ref is built where the reference sources are)")
    assert mod.run(None) == 0
