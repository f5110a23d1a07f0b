"""ctypes binding of lib/libvj.so (the C ABI of include/vj.h) for tests and benchmarks.

Device buffers are passed as raw pointers or as torch CUDA tensors (torch provides device
memory and streams only; every computation runs in the library's kernels). There is no
CPU fallback: importing this module without the built library raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libvj.so"

VJ_OK = 0
VJ_ERR_INVALID_ARGUMENT = 1
VJ_ERR_UNSUPPORTED = 2
VJ_ERR_CUDA = 3
VJ_ERR_OUT_OF_MEMORY = 4
VJ_ERR_CAPACITY = 5
VJ_ERR_DEVICE = 6
VJ_ERR_BUDGET = 7
VJ_JOIN_FIXED_PASSES = 1
VJ_JOIN_SHARED_TABLES = 2
VJ_JOIN_L2_TABLES = 4
VJ_JOIN_TEST_DEVICE_FLAG = 1 << 16
VJ_JOIN_BATCH_LAUNCHES = 1 << 17

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

# Every symbol include/vj.h declares.
EXPORTS = [
    "vj_version",
    "vj_allocation_count",
    "vj_status_string",
    "vj_last_error",
    "vj_hash_algo_id",
    "vj_hash_algo_name",
    "vj_hash",
    "vj_ctx_create",
    "vj_ctx_destroy",
    "vj_ctx_memory_in_use",
    "vj_ctx_trim",
    "vj_ctx_set_profiling",
    "vj_ctx_last_profile",
    "vj_partition",
    "vj_partition_noalloc",
    "vj_build_probe",
    "vj_join",
    "vj_join_batch",
    "vj_tune",
    "vj_tune_save",
    "vj_tune_load",
    "vj_server_create",
    "vj_server_submit",
    "vj_server_wait",
    "vj_server_stats_get",
    "vj_server_destroy",
    "vj_server_share_tuning",
    "vj_join_host",
    "vj_result_free",
    "vj_pairs_digest",
    "vj_generate_join",
    "vj_generate_join_expect",
]


class VjTable(ctypes.Structure):
    _fields_ = [
        ("keys", ctypes.c_void_p),
        ("payloads", ctypes.c_void_p),
        ("rows", ctypes.c_uint64),
        ("key_words", ctypes.c_int32),
        ("payload_bytes", ctypes.c_int32),
    ]


class VjJoinOptions(ctypes.Structure):
    _fields_ = [
        ("hash_algo", ctypes.c_int32),
        ("hash_bits", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("passes", ctypes.c_int32),
        ("radix_bits", ctypes.c_int32 * 2),
        ("build_rows", ctypes.c_int32),
        ("probe_rows", ctypes.c_int32),
        ("probe_threads", ctypes.c_int32),
        ("probe_sub_rows", ctypes.c_int32),
        ("table_load_pct", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 3),
    ]


def options_dict(o: "VjJoinOptions") -> dict:
    return {
        "tables": "l2" if o.flags & VJ_JOIN_L2_TABLES else ("shared" if o.flags & VJ_JOIN_SHARED_TABLES else "auto"),
        "passes": o.passes if o.flags & VJ_JOIN_FIXED_PASSES else "auto",
        "radix_bits": [o.radix_bits[0], o.radix_bits[1]],
        "build_rows": o.build_rows,
        "probe_rows": o.probe_rows,
        "probe_threads": o.probe_threads,
        "table_load_pct": o.table_load_pct,
    }


class VjResult(ctypes.Structure):
    _fields_ = [
        ("pairs", ctypes.c_void_p),
        ("count", ctypes.c_uint64),
        ("capacity", ctypes.c_uint64),
        ("owned", ctypes.c_int32),
        ("payload_bytes", ctypes.c_int32),
    ]


class VjProfile(ctypes.Structure):
    _fields_ = [
        ("passes", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int32),
        ("radix_bits", ctypes.c_int32 * 2),
        ("build_rows", ctypes.c_uint32),
        ("probe_rows", ctypes.c_uint32),
        ("ms_histogram", ctypes.c_float * 2),
        ("ms_scatter", ctypes.c_float * 2),
        ("ms_plan", ctypes.c_float * 2),
        ("ms_probe", ctypes.c_float),
        ("ms_total", ctypes.c_float),
        ("rows", ctypes.c_uint64 * 2),
        ("matches", ctypes.c_uint64),
        ("tables", ctypes.c_int32),
        ("fallbacks", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {
            "passes": self.passes,
            "kernel_launches": self.kernel_launches,
            "radix_bits": list(self.radix_bits),
            "build_rows": self.build_rows,
            "probe_rows": self.probe_rows,
            "ms_histogram": list(self.ms_histogram),
            "ms_scatter": list(self.ms_scatter),
            "ms_plan": list(self.ms_plan),
            "ms_probe": self.ms_probe,
            "ms_total": self.ms_total,
            "rows": list(self.rows),
            "matches": self.matches,
            "tables": "l2" if self.tables == 1 else "shared",
            "fallbacks": self.fallbacks,
        }


class VjRequestResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("slot", ctypes.c_int32),
        ("count", ctypes.c_uint64),
        ("submit_s", ctypes.c_double),
        ("start_s", ctypes.c_double),
        ("finish_s", ctypes.c_double),
        ("passes", ctypes.c_int32),
        ("radix_bits", ctypes.c_int32 * 2),
        ("build_rows", ctypes.c_uint32),
    ]


class VjServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("peak_bytes", ctypes.c_uint64),
        ("budget", ctypes.c_uint64),
        ("peak_running", ctypes.c_int32),
        ("slots", ctypes.c_int32),
    ]


class VjError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"vj status {status}: {message}")
        self.status = status


_lib = None
vp = ctypes.c_void_p
u64 = ctypes.c_uint64
i32 = ctypes.c_int


def load() -> ctypes.CDLL:
    """Load lib/libvj.so (built by build.py / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() first (no CPU fallback exists)")
        L = ctypes.CDLL(str(LIB_PATH))
        L.vj_version.restype = i32
        L.vj_allocation_count.restype = u64
        L.vj_allocation_count.argtypes = []
        L.vj_status_string.restype = ctypes.c_char_p
        L.vj_status_string.argtypes = [i32]
        L.vj_last_error.restype = ctypes.c_size_t
        L.vj_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.vj_hash_algo_id.restype = i32
        L.vj_hash_algo_id.argtypes = [ctypes.c_char_p]
        L.vj_hash_algo_name.restype = ctypes.c_char_p
        L.vj_hash_algo_name.argtypes = [i32]
        L.vj_hash.restype = i32
        L.vj_hash.argtypes = [vp, u64, i32, i32, i32, i32, i32, vp, vp]
        L.vj_ctx_create.restype = i32
        L.vj_ctx_create.argtypes = [i32, u64, ctypes.POINTER(vp)]
        L.vj_ctx_destroy.restype = i32
        L.vj_ctx_destroy.argtypes = [vp]
        L.vj_ctx_memory_in_use.restype = u64
        L.vj_ctx_memory_in_use.argtypes = [vp]
        L.vj_ctx_trim.restype = i32
        L.vj_ctx_trim.argtypes = [vp]
        L.vj_ctx_set_profiling.restype = i32
        L.vj_ctx_set_profiling.argtypes = [vp, i32]
        L.vj_ctx_last_profile.restype = i32
        L.vj_ctx_last_profile.argtypes = [vp, ctypes.POINTER(VjProfile)]
        L.vj_partition.restype = i32
        L.vj_partition.argtypes = [vp, ctypes.POINTER(VjTable), vp, i32, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp]
        L.vj_partition_noalloc.restype = i32
        L.vj_partition_noalloc.argtypes = [ctypes.POINTER(VjTable), vp, i32, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp]
        L.vj_build_probe.restype = i32
        L.vj_build_probe.argtypes = [vp, ctypes.POINTER(VjTable), vp, ctypes.POINTER(VjTable), vp, i32, i32, vp, u64, ctypes.POINTER(u64), vp]
        L.vj_join.restype = i32
        L.vj_join.argtypes = [vp, ctypes.POINTER(VjTable), ctypes.POINTER(VjTable), ctypes.POINTER(VjJoinOptions), ctypes.POINTER(VjResult), vp]
        L.vj_join_batch.restype = i32
        L.vj_join_batch.argtypes = [vp, ctypes.POINTER(VjTable), ctypes.POINTER(VjTable), ctypes.c_uint32, vp, vp, u64, ctypes.POINTER(VjJoinOptions), vp, vp, u64, vp, vp, vp]
        L.vj_server_create.restype = i32
        L.vj_server_create.argtypes = [i32, u64, i32, ctypes.POINTER(vp)]
        L.vj_server_submit.restype = i32
        L.vj_server_submit.argtypes = [vp, ctypes.POINTER(VjTable), ctypes.POINTER(VjTable), ctypes.POINTER(VjJoinOptions), vp, u64, ctypes.POINTER(u64)]
        L.vj_server_wait.restype = i32
        L.vj_server_wait.argtypes = [vp, u64, ctypes.POINTER(VjRequestResult)]
        L.vj_server_stats_get.restype = i32
        L.vj_server_stats_get.argtypes = [vp, ctypes.POINTER(VjServerStats)]
        L.vj_server_share_tuning.restype = i32
        L.vj_server_share_tuning.argtypes = [vp, vp]
        L.vj_server_destroy.restype = i32
        L.vj_server_destroy.argtypes = [vp]
        L.vj_tune.restype = i32
        L.vj_tune.argtypes = [vp, ctypes.POINTER(VjTable), ctypes.POINTER(VjTable), ctypes.POINTER(VjJoinOptions), vp, u64, i32, ctypes.POINTER(VjJoinOptions), ctypes.POINTER(ctypes.c_float), vp]
        L.vj_tune_save.restype = i32
        L.vj_tune_save.argtypes = [vp, ctypes.c_char_p]
        L.vj_tune_load.restype = i32
        L.vj_tune_load.argtypes = [vp, ctypes.c_char_p]
        L.vj_join_host.restype = i32
        L.vj_join_host.argtypes = [vp, ctypes.POINTER(VjTable), ctypes.POINTER(VjTable), ctypes.POINTER(VjJoinOptions), vp, u64, ctypes.POINTER(u64), vp]
        L.vj_result_free.restype = i32
        L.vj_result_free.argtypes = [vp, ctypes.POINTER(VjResult)]
        L.vj_pairs_digest.restype = i32
        L.vj_pairs_digest.argtypes = [vp, u64, i32, ctypes.POINTER(u64), ctypes.POINTER(u64), vp]
        L.vj_generate_join.restype = i32
        L.vj_generate_join.argtypes = [u64, i32, i32, u64, u64, u64, vp, vp, vp, vp, vp]
        L.vj_generate_join_expect.restype = i32
        L.vj_generate_join_expect.argtypes = [u64, u64, u64, u64, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(u64), vp]
        _lib = L
    return _lib


_cudart = None


def device_to_numpy(src_ptr: int, count: int, dtype) -> "np.ndarray":
    """Copy `count` elements of `dtype` from a device pointer (e.g. a library-owned result)."""
    import numpy as np

    global _cudart
    if _cudart is None:
        load()
        _cudart = ctypes.CDLL("libcudart.so.13")
        _cudart.cudaMemcpy.restype = ctypes.c_int
        _cudart.cudaMemcpy.argtypes = [vp, vp, ctypes.c_size_t, ctypes.c_int]
    out = np.empty(count, dtype=dtype)
    if count:
        rc = _cudart.cudaMemcpy(out.ctypes.data, src_ptr, out.nbytes, 2)  # device to host
        if rc != 0:
            raise RuntimeError(f"cudaMemcpy failed: {rc}")
    return out


def allocation_count() -> int:
    """vj_allocation_count: allocations the library has made in this process."""
    return int(load().vj_allocation_count())


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().vj_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != VJ_OK:
        raise VjError(status, last_error())


def ptr(x) -> int | None:
    """Device/host pointer of a torch tensor, numpy array or int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(type(x))


def stream_handle(stream=None) -> int | None:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def table(keys, payloads, rows: int, key_words: int, payload_bytes: int) -> VjTable:
    """A vj_table view. The view keeps `keys` and `payloads` alive: a view of temporaries
    would otherwise point at memory the allocator hands out again."""
    t = VjTable(ptr(keys), ptr(payloads), rows, key_words, payload_bytes)
    t._refs = (keys, payloads)
    return t


def options(hash_algo: int = 0, hash_bits: int = 0, passes: int | None = None, radix_bits=(0, 0), build_rows: int = 0, probe_rows: int = 0, probe_threads: int = 0, table_load_pct: int = 0, tables: str = "auto", test_device_flag: bool = False, batch_launches: bool = False) -> VjJoinOptions:
    """Join options; tables: "auto" or "shared" (shared-memory tables; "l2" is refused by the
    library with VJ_ERR_UNSUPPORTED). batch_launches: vj_join_batch as separate launches
    instead of one fused launch."""
    o = VjJoinOptions()
    o.hash_algo = hash_algo
    o.hash_bits = hash_bits
    o.flags = {"auto": 0, "shared": VJ_JOIN_SHARED_TABLES, "l2": VJ_JOIN_L2_TABLES}[tables]
    if test_device_flag:
        o.flags |= VJ_JOIN_TEST_DEVICE_FLAG
    if batch_launches:
        o.flags |= VJ_JOIN_BATCH_LAUNCHES
    if passes is not None:
        o.flags |= VJ_JOIN_FIXED_PASSES
        o.passes = passes
    o.radix_bits[0] = radix_bits[0]
    o.radix_bits[1] = radix_bits[1]
    o.build_rows = build_rows
    o.probe_rows = probe_rows
    o.probe_threads = probe_threads
    o.table_load_pct = table_load_pct
    return o


class Context:
    """vj_ctx wrapper."""

    def __init__(self, device: int = 0, budget: int = 0):
        self.lib = load()
        h = vp()
        check(self.lib.vj_ctx_create(device, budget, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            check(self.lib.vj_ctx_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_profiling(self, enabled: bool) -> None:
        check(self.lib.vj_ctx_set_profiling(self.handle, int(enabled)))

    def last_profile(self) -> VjProfile:
        p = VjProfile()
        check(self.lib.vj_ctx_last_profile(self.handle, ctypes.byref(p)))
        return p

    def memory_in_use(self) -> int:
        return int(self.lib.vj_ctx_memory_in_use(self.handle))

    def join(self, r: VjTable, s: VjTable, opts: VjJoinOptions | None = None, out=None, capacity: int = 0, stream=None) -> VjResult:
        res = VjResult()
        if out is not None:
            res.pairs = ptr(out)
            res.capacity = capacity
        check(self.lib.vj_join(self.handle, ctypes.byref(r), ctypes.byref(s), ctypes.byref(opts) if opts else None, ctypes.byref(res), stream_handle(stream)))
        return res

    def free(self, res: VjResult) -> None:
        check(self.lib.vj_result_free(self.handle, ctypes.byref(res)))

    def join_batch(self, r: VjTable, s: VjTable, joins: int, r_offsets, s_offsets, pairs, pair_offsets, pair_capacity: int, counts, status=None, max_build_rows: int = 0, opts: VjJoinOptions | None = None, stream=None) -> None:
        """vj_join_batch: `joins` independent joins in one launch sequence (asynchronous).
        Offsets, counts and status are device arrays (u64 offsets of joins + 1 entries)."""
        check(
            self.lib.vj_join_batch(
                self.handle, ctypes.byref(r), ctypes.byref(s), joins, ptr(r_offsets), ptr(s_offsets), max_build_rows, ctypes.byref(opts) if opts else None, ptr(pairs), ptr(pair_offsets), pair_capacity,
                ptr(counts), ptr(status), stream_handle(stream)
            )
        )

    def tune(self, r: VjTable, s: VjTable, out, capacity: int, base: VjJoinOptions | None = None, max_candidates: int = 0, stream=None) -> tuple[VjJoinOptions, float]:
        """vj_tune: the fastest plan for this join's shape class (kept in the context)."""
        best = VjJoinOptions()
        ms = ctypes.c_float(0)
        check(self.lib.vj_tune(self.handle, ctypes.byref(r), ctypes.byref(s), ctypes.byref(base) if base else None, ptr(out), capacity, max_candidates, ctypes.byref(best), ctypes.byref(ms), stream_handle(stream)))
        return best, float(ms.value)

    def tune_save(self, path: str) -> None:
        check(self.lib.vj_tune_save(self.handle, str(path).encode()))

    def tune_load(self, path: str) -> None:
        check(self.lib.vj_tune_load(self.handle, str(path).encode()))

    def join_host(self, r: VjTable, s: VjTable, out, capacity: int, opts: VjJoinOptions | None = None, stream=None) -> int:
        n = u64(0)
        check(self.lib.vj_join_host(self.handle, ctypes.byref(r), ctypes.byref(s), ctypes.byref(opts) if opts else None, ptr(out), capacity, ctypes.byref(n), stream_handle(stream)))
        return int(n.value)

    def build_probe(self, r: VjTable, s: VjTable, r_hashes=None, s_hashes=None, hash_bits: int = 64, out=None, capacity: int = 0, stream=None) -> int:
        n = u64(0)
        st = self.lib.vj_build_probe(self.handle, ctypes.byref(r), ptr(r_hashes), ctypes.byref(s), ptr(s_hashes), hash_bits, 0, ptr(out), capacity, ctypes.byref(n), stream_handle(stream))
        if st == VJ_ERR_CAPACITY:
            return int(n.value)
        check(st)
        return int(n.value)

    def partition(self, t: VjTable, keys_out, pay_out, radix_shift: int, radix_bits: int, hashes_in=None, hash_bits: int = 64, hash_algo: int = 0, hashes_out=None, d_hist=None, d_off=None, h_hist=None, h_off=None, stream=None) -> None:
        check(
            self.lib.vj_partition(
                self.handle, ctypes.byref(t), ptr(hashes_in), hash_bits, hash_algo, ptr(keys_out), ptr(pay_out), ptr(hashes_out), radix_shift, radix_bits, ptr(d_hist), ptr(d_off), ptr(h_hist), ptr(h_off), stream_handle(stream)
            )
        )


def partition_noalloc(t: VjTable, keys_out, pay_out, radix_shift: int, radix_bits: int, hashes_in=None, hash_bits: int = 64, hash_algo: int = 0, hashes_out=None, d_hist=None, d_off=None, h_hist=None, h_off=None, stream=None) -> None:
    """vj_partition_noalloc on the current device: Context.partition without a context, for
    callers that cannot allocate device memory (its scratch is a static device array)."""
    check(
        load().vj_partition_noalloc(
            ctypes.byref(t), ptr(hashes_in), hash_bits, hash_algo, ptr(keys_out), ptr(pay_out), ptr(hashes_out), radix_shift, radix_bits, ptr(d_hist), ptr(d_off), ptr(h_hist), ptr(h_off), stream_handle(stream)
        )
    )


def hash(d_in, n: int, chunk_offset: int, element_chunks: int, chunk_bits: int, hash_bits: int, algo: int | str, d_out, stream=None) -> None:
    if isinstance(algo, str):
        algo = ALGORITHMS.index(algo)
    check(load().vj_hash(ptr(d_in), n, chunk_offset, element_chunks, chunk_bits, hash_bits, algo, ptr(d_out), stream_handle(stream)))


def pairs_digest(d_pairs, count: int, payload_bytes: int, stream=None) -> tuple[int, int]:
    s = u64(0)
    x = u64(0)
    check(load().vj_pairs_digest(ptr(d_pairs), count, payload_bytes, ctypes.byref(s), ctypes.byref(x), stream_handle(stream)))
    return int(s.value), int(x.value)


def generate_join(seed: int, key_bytes: int, payload_bytes: int, nr: int, ns: int, match_threshold: int, rk, rp, sk, sp, stream=None) -> None:
    check(load().vj_generate_join(seed, key_bytes, payload_bytes, nr, ns, match_threshold, ptr(rk), ptr(rp), ptr(sk), ptr(sp), stream_handle(stream)))


def generate_join_expect(seed: int, nr: int, ns: int, match_threshold: int, stream=None) -> tuple[int, int, int]:
    c = u64(0)
    s = u64(0)
    x = u64(0)
    check(load().vj_generate_join_expect(seed, nr, ns, match_threshold, ctypes.byref(c), ctypes.byref(s), ctypes.byref(x), stream_handle(stream)))
    return int(c.value), int(s.value), int(x.value)


class Server:
    """vj_server wrapper: submit joins of device tables, wait for their results."""

    def __init__(self, device: int = 0, budget: int = 0, slots: int = 4):
        self.lib = load()
        h = vp()
        check(self.lib.vj_server_create(device, budget, slots, ctypes.byref(h)))
        self.handle = h
        self._keep: dict[int, tuple] = {}

    def submit(self, r: VjTable, s: VjTable, out, capacity: int, opts: VjJoinOptions | None = None) -> int:
        rid = u64(0)
        check(self.lib.vj_server_submit(self.handle, ctypes.byref(r), ctypes.byref(s), ctypes.byref(opts) if opts else None, ptr(out), capacity, ctypes.byref(rid)))
        self._keep[int(rid.value)] = (r, s, out, opts)  # buffers live until the wait
        return int(rid.value)

    def wait(self, rid: int) -> VjRequestResult:
        res = VjRequestResult()
        check(self.lib.vj_server_wait(self.handle, rid, ctypes.byref(res)))
        self._keep.pop(rid, None)
        return res

    def share_tuning(self, ctx: "Context") -> None:
        """vj_server_share_tuning: the slots use ctx's tuning cache."""
        check(self.lib.vj_server_share_tuning(self.handle, ctx.handle))

    def stats(self) -> VjServerStats:
        st = VjServerStats()
        check(self.lib.vj_server_stats_get(self.handle, ctypes.byref(st)))
        return st

    def close(self) -> None:
        if self.handle:
            check(self.lib.vj_server_destroy(self.handle))
            self.handle = None
