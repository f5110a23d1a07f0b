/*
 * Device-only build of the reference's hash kernels (src/hash/hash.cu:84-505) for sm_103a,
 * one cubin per (HASH_BITS, HASH_CHUNK_BITS) pair (recipe: oracle/ref_build.sh). The
 * cubins are loaded by oracle/ref_gpu_check.py through the CUDA driver API to pin the
 * oracle's hash restatement against the reference kernels run on the GPU, including the
 * *_shift variants whose out-of-range shifts C leaves undefined. Test infrastructure only.
 *
 * src/base/config.h is `#pragma once`: including it first and redefining the two widths
 * makes the later include from src/base/types.hpp a no-op, so REF_HB/REF_CB take effect.
 */
#include <cstdint>
#include "base/config.h"
#undef HASH_BITS
#define HASH_BITS REF_HB
#undef HASH_CHUNK_BITS
#define HASH_CHUNK_BITS REF_CB
#include "hash/hash.cu"
