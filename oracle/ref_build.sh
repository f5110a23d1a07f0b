#!/usr/bin/env bash
# Builds oracle/_ref/ from the reference sources where they lie (read-only). Test
# infrastructure only: the products are checkers, never part of the library.
#   ref_hash_host_h{HB}_c{CB}  reference hash kernels run as host code (x86/Arm CPU)
#   ref_join_cpu               reference JoinProvider::join_cpu on host tables
#   ref_h{HB}_c{CB}.cubin      reference hash kernels for sm_103a (loaded on a GPU machine)
# usage: oracle/ref_build.sh REFERENCE_ROOT   (the checkout of vgerber/vectorized-join)
set -euo pipefail
REF=${1:?usage: oracle/ref_build.sh REFERENCE_ROOT}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/hash/hash.cu" ]; then
    echo "reference sources not found at $REF; oracle/_ref not built" >&2
    exit 0
fi
mkdir -p "$OUT"
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
NVCC="$CUDA_HOME/bin/nvcc"
pids=()
for HB in 32 64; do
    for CB in 8 32 64 128; do
        # hash.cu up to, not including, the dispatcher (it uses <<<>>>), then our main().
        ( { sed '/^void hash_func/,$d' "$REF/src/hash/hash.cu"; cat "$HERE/ref_hash_host_main.cpp"; } |
            g++ -std=c++17 -O1 -w -fsigned-char -x c++ -DREF_HB=$HB -DREF_CB=$CB \
                -include "$HERE/ref_shim.h" -I"$REF/src" -I"$CUDA_HOME/include" - \
                -o "$OUT/ref_hash_host_h${HB}_c${CB}" -L"$CUDA_HOME/lib64" -lcudart ) &
        pids+=($!)
        "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w -DREF_HB=$HB -DREF_CB=$CB \
            -I"$REF/src" "$HERE/ref_gpu_kernels.cu" -o "$OUT/ref_h${HB}_c${CB}.cubin" &
        pids+=($!)
    done
done
"$NVCC" -std=c++17 -O1 -w -gencode arch=compute_103a,code=sm_103a -I"$REF/src" \
    "$HERE/ref_join_cpu_main.cu" -o "$OUT/ref_join_cpu" -lcurand &
pids+=($!)
rc=0
for p in "${pids[@]}"; do
    wait "$p" || rc=1
done
exit $rc
