"""Times the reference's own hash kernels against vj_hash on the same GPU and the same keys:
2^30 keys of 8, 16 and 32 uniform random bytes, FNV-1a 64 and custom_xor_hw, 64-bit
chunks (the hash microbench). Test infrastructure: the reference's kernels come from
oracle/_ref/ref_h64_c64.cubin -- src/hash/hash.cu compiled unchanged for sm_103a by
oracle/ref_build.sh -- and run with its own dispatcher's grid (hash.cu:507-509: 256
threads, max(n / elements_per_thread / 256, 1) blocks, elements_per_thread = 1). Both
outputs are compared element for element before timing.

    python oracle/ref_hash_bench.py [--keys-log2 30] [--out FILE.json]

Exit status 0 on success, 2 when the cubin is absent.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(HERE))

from ref_gpu_check import Driver, mangled  # noqa: E402


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--keys-log2", type=int, default=30)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    cubin = HERE / "_ref" / "ref_h64_c64.cubin"
    if not cubin.exists():
        print("reference cubin not present (oracle/_ref is built where the reference sources are)")
        return 2
    import torch

    spec = importlib.util.spec_from_file_location("vj", ROOT / "vectorized-join_gb300" / "vj.py")
    vj = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vj)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    torch.empty(1, device=dev)  # torch's context is the device's primary context
    drv = Driver()
    mod = drv.module(cubin)
    n = 1 << args.keys_log2
    gen = torch.Generator(device=dev)
    gen.manual_seed(42)
    stream = torch.cuda.current_stream()
    results = []
    for eb in (8, 16, 32):
        keys = torch.randint(-(2**62), 2**62, (n * eb // 8,), dtype=torch.int64, generator=gen, device=dev)
        ours = torch.empty(n, dtype=torch.int64, device=dev)
        theirs = torch.empty(n, dtype=torch.int64, device=dev)
        for algo in ("fnv", "custom_xor_hw"):
            fn = drv.function(mod, mangled(algo, 64, 64))
            blocks = max(n // 256, 1)
            argv = [ctypes.c_uint64(n), ctypes.c_int16(0), ctypes.c_int16(eb // 8), ctypes.c_uint64(keys.data_ptr()), ctypes.c_uint64(theirs.data_ptr())]
            ptrs = (ctypes.c_void_p * len(argv))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in argv])

            def ref_launch():
                rc = drv.cu.cuLaunchKernel(fn, blocks, 1, 1, 256, 1, 1, 0, ctypes.c_void_p(stream.cuda_stream), ptrs, None)
                if rc != 0:
                    raise RuntimeError(f"cuLaunchKernel: {rc}")

            def our_launch():
                vj.hash(keys, n, 0, eb // 8, 64, 64, algo, ours, stream=stream)

            ref_launch()
            our_launch()
            torch.cuda.synchronize()
            assert torch.equal(ours, theirs), (eb, algo)
            times = {}
            for name, fn_ in (("reference", ref_launch), ("ours", our_launch)):
                for _ in range(2):
                    fn_()
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.reps + 1)]
                ev[0].record(stream)
                for k in range(args.reps):
                    fn_()
                    ev[k + 1].record(stream)
                torch.cuda.synchronize()
                times[name] = min(ev[k].elapsed_time(ev[k + 1]) for k in range(args.reps))
            gb = n * (eb + 8) / 1e9
            results.append(
                {
                    "key_bytes": eb,
                    "algo": algo,
                    "reference_ms": times["reference"],
                    "reference_GBps": gb / (times["reference"] / 1000),
                    "ours_ms": times["ours"],
                    "ours_GBps": gb / (times["ours"] / 1000),
                    "speedup": times["reference"] / times["ours"],
                }
            )
            print(json.dumps(results[-1]), flush=True)
        del keys, ours, theirs
        torch.cuda.empty_cache()
    if args.out:
        Path(args.out).write_text(json.dumps(results, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
