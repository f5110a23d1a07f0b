"""Runs the reference's own hash kernels on the GPU and compares them with the golden
known-answer vectors (tests/golden/hash_kat.npz). Test infrastructure only.

The kernels come from oracle/_ref/ref_h{HB}_c{CB}.cubin: src/hash/hash.cu of the reference,
compiled unchanged for sm_103a by oracle/ref_build.sh (one cubin per HASH_BITS /
HASH_CHUNK_BITS pair). They are loaded with the CUDA driver API through ctypes and
launched with the reference dispatcher's grid (hash.cu:508-509: 256 threads,
max(n / 256, 1) blocks; custom_n_mult_xor_shift gets rounds = 2, hash.cu:526).

This pins every golden vector to the reference's compiled code on the GPU, including the
elements whose value rests on a *_shift variant's out-of-range shift amount.

    python oracle/ref_gpu_check.py [--out FILE.json]

Exit status 0 when every vector matches, 1 on a mismatch, 2 when the cubins are absent.
"""
from __future__ import annotations

import ctypes
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = HERE / "_ref"

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


def mangled(algo: str, hb: int, cb: int) -> str:
    """Itanium-mangled name of the reference kernel `hash_<algo>(index_t, short, short,
    [short,] chunk_t *, hash_t *)`."""
    name = "hash_fnv" if algo == "fnv" else "hash_" + algo
    chunk = {8: "Pc", 32: "P5uint1", 64: "P5uint2", 128: "P5uint4"}[cb]
    hsh = "Py" if hb == 64 else "Pj"
    shorts = "sss" if algo == "custom_n_mult_xor_shift" else "ss"
    return f"_Z{len(name)}{name}y{shorts}{chunk}{hsh}"


class Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self._check(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.dev = dev
        self.ctx = ctx
        self.modules = {}

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def module(self, path: Path):
        if path not in self.modules:
            mod = ctypes.c_void_p()
            self._check(self.cu.cuModuleLoad(ctypes.byref(mod), str(path).encode()), f"cuModuleLoad({path.name})")
            self.modules[path] = mod
        return self.modules[path]

    def function(self, mod, name: str):
        fn = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), mod, name.encode()), f"cuModuleGetFunction({name})")
        return fn

    def alloc(self, nbytes: int) -> ctypes.c_uint64:
        p = ctypes.c_uint64()
        self._check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 16))), "cuMemAlloc")
        return p

    def free(self, p):
        self.cu.cuMemFree_v2(p)

    def htod(self, dst, arr: np.ndarray):
        arr = np.ascontiguousarray(arr)
        self._check(self.cu.cuMemcpyHtoD_v2(dst, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes)), "cuMemcpyHtoD")

    def dtoh(self, arr: np.ndarray, src):
        self._check(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data_as(ctypes.c_void_p), src, ctypes.c_size_t(arr.nbytes)), "cuMemcpyDtoH")

    def launch(self, fn, grid: int, block: int, args: list):
        holders = []
        ptrs = (ctypes.c_void_p * len(args))()
        for i, a in enumerate(args):
            holders.append(a)
            ptrs[i] = ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
        self._check(self.cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, None, ptrs, None), "cuLaunchKernel")
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


def run(out_path: Path | None) -> int:
    cubins = {(hb, cb): REF / f"ref_h{hb}_c{cb}.cubin" for hb in (32, 64) for cb in (8, 32, 64, 128)}
    if not all(p.exists() for p in cubins.values()):
        print("reference cubins not present (oracle/_ref is built where the reference sources are)")
        return 2
    kat = np.load(ROOT / "tests" / "golden" / "hash_kat.npz")
    manifest = json.loads(bytes(kat["manifest"]).decode())
    drv = Driver()
    total = mismatched = clamp_checked = 0
    failures = []
    for hb, cb, eb, off, algo in manifest:
        inp = kat[f"in_c{cb}_e{eb}"]
        key = f"h{hb}_c{cb}_e{eb}_o{off}_{algo}"
        want = kat[key]
        n = want.size
        ec = eb // (cb // 8)
        mod = drv.module(cubins[(hb, cb)])
        fn = drv.function(mod, mangled(algo, hb, cb))
        d_in = drv.alloc(inp.nbytes)
        d_out = drv.alloc(n * hb // 8)
        drv.htod(d_in, inp)
        threads = 256
        blocks = max(n // threads, 1)
        args = [ctypes.c_uint64(n), ctypes.c_int16(off), ctypes.c_int16(ec)]
        if algo == "custom_n_mult_xor_shift":
            args.append(ctypes.c_int16(2))
        args += [ctypes.c_uint64(d_in.value), ctypes.c_uint64(d_out.value)]
        drv.launch(fn, blocks, threads, args)
        got = np.zeros(n, dtype=want.dtype)
        drv.dtoh(got, d_out)
        drv.free(d_in)
        drv.free(d_out)
        total += n
        bad = got != want
        if "ub_" + key in kat.files:
            clamp_checked += int(kat["ub_" + key].sum())
        if bad.any():
            mismatched += int(bad.sum())
            idx = np.nonzero(bad)[0][:4]
            failures.append({"case": key, "elements": idx.tolist(), "reference": got[idx].tolist(), "golden": want[idx].tolist()})
    report = {
        "vectors": len(manifest),
        "elements": total,
        "elements_on_shift_clamp": clamp_checked,
        "mismatched_elements": mismatched,
        "failures": failures[:50],
    }
    print(json.dumps({k: v for k, v in report.items() if k != "failures"}))
    for f in failures[:10]:
        print("MISMATCH", f)
    if out_path:
        out_path.parent.mkdir(parents=True, exist_ok=True)
        out_path.write_text(json.dumps(report, indent=1))
    return 0 if mismatched == 0 else 1


if __name__ == "__main__":
    out = None
    if "--out" in sys.argv:
        out = Path(sys.argv[sys.argv.index("--out") + 1])
    sys.exit(run(out))
