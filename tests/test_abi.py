"""CPU tests of the C ABI boundary: the library loads, exports every function include/vj.h
declares, and validates arguments without touching a GPU."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "vj.h").read_text()
    return sorted(set(re.findall(r"^VJ_API\s+[\w\s\*]+?\b(vj_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(vjlib):
    names = declared_functions()
    assert len(names) >= 18
    lib = vjlib.load()
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(vjlib.EXPORTS) == names


def test_version_and_strings(vjlib):
    lib = vjlib.load()
    assert lib.vj_version() >= 10000
    assert lib.vj_status_string(0) == b"ok"
    assert lib.vj_status_string(vjlib.VJ_ERR_CAPACITY) == b"output capacity too small"


def test_algorithm_names_round_trip(vjlib):
    lib = vjlib.load()
    for i, name in enumerate(vjlib.ALGORITHMS):
        assert lib.vj_hash_algo_id(name.encode()) == i
        assert lib.vj_hash_algo_name(i) == name.encode()
    # the reference launches nothing for an unknown name (hash.cu:515-541); here it is -1
    assert lib.vj_hash_algo_id(b"custom") == -1
    assert lib.vj_hash_algo_id(b"xor_hw") == -1
    assert lib.vj_hash_algo_name(13) is None


def test_hash_argument_validation_without_gpu(vjlib):
    lib = vjlib.load()
    # n == 0 is a no-op
    assert lib.vj_hash(None, 0, 0, 1, 64, 64, 0, None, None) == 0
    assert lib.vj_hash(None, 10, 0, 1, 64, 64, 99, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert "unknown algorithm" in vjlib.last_error()
    assert lib.vj_hash(None, 10, 0, 1, 16, 64, 0, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_hash(None, 10, 0, 1, 64, 48, 0, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_hash(None, 10, 0, 40000, 64, 64, 0, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_hash(None, 10, 0, 1, 64, 64, 0, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert "null" in vjlib.last_error()


def test_join_argument_validation_without_gpu(vjlib):
    lib = vjlib.load()
    t = vjlib.VjTable(None, None, 0, 2, 8)
    res = vjlib.VjResult()
    assert lib.vj_join(None, ctypes.byref(t), ctypes.byref(t), None, ctypes.byref(res), None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    bad = vjlib.VjTable(None, None, 0, 3, 8)
    # null context is reported first
    assert lib.vj_join(None, ctypes.byref(bad), ctypes.byref(t), None, ctypes.byref(res), None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_result_free(None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_pairs_digest(None, 0, 3, None, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_generate_join(1, 3, 8, 1, 1, 0, None, None, None, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_ctx_destroy(None) == 0
    assert lib.vj_ctx_memory_in_use(None) == 0


def test_host_batch_and_tune_argument_validation_without_gpu(vjlib):
    lib = vjlib.load()
    t = vjlib.VjTable(None, None, 0, 2, 8)
    n = ctypes.c_uint64(7)
    # null context / count are reported before any device work
    assert lib.vj_join_host(None, ctypes.byref(t), ctypes.byref(t), None, None, 0, ctypes.byref(n), None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_join_host(None, ctypes.byref(t), ctypes.byref(t), None, None, 0, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_join_batch(None, ctypes.byref(t), ctypes.byref(t), 1, None, None, 0, None, None, None, 0, None, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert lib.vj_tune(None, ctypes.byref(t), ctypes.byref(t), None, None, 0, 0, None, None, None) == vjlib.VJ_ERR_INVALID_ARGUMENT
    assert "null" in vjlib.last_error()


def test_join_options_round_trip(vjlib):
    o = vjlib.options(passes=2, radix_bits=(8, 9), build_rows=1024, tables="shared")
    d = vjlib.options_dict(o)
    assert d["tables"] == "shared" and d["passes"] == 2 and d["radix_bits"] == [8, 9] and d["build_rows"] == 1024
    a = vjlib.options_dict(vjlib.options())
    assert a["tables"] == "auto" and a["passes"] == "auto"
    assert vjlib.options_dict(vjlib.options(tables="l2"))["tables"] == "l2"
    t = vjlib.options_dict(vjlib.options(probe_threads=256, table_load_pct=25, probe_rows=4096))
    assert t["probe_threads"] == 256 and t["table_load_pct"] == 25 and t["probe_rows"] == 4096
    assert ctypes.sizeof(vjlib.VjJoinOptions) == 56  # include/vj.h layout (unchanged by table_load_pct)
    assert vjlib.options(test_device_flag=True).flags == vjlib.VJ_JOIN_TEST_DEVICE_FLAG
    assert vjlib.allocation_count() >= 0
