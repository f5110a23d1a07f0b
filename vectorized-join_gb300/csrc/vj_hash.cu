// vj_hash.cu -- vj_hash: the reference's 13 hash algorithms (src/hash/hash.cu:84-505) for
// sm_103a, bit-exact, as streaming kernels bound by HBM bandwidth.
//
// One thread hashes one element per iteration of a grid-stride loop. Elements of 8, 16 or
// 32 bytes are fetched with 8/16-byte vector loads (a warp reads 256-1024 contiguous
// bytes per load instruction); other sizes fall back to 4-byte (or byte) loads. The hash
// arithmetic is a handful of integer ops per 32-bit lane, far below the memory time.
#include "vj_internal.cuh"

namespace vj {

namespace {

// Feed the chunks [chunk_offset, nchunks) held in registers (w = little-endian words of
// the element) into the state.
template <typename H, int CB, int ALGO, int WORDS>
__device__ __forceinline__ H hash_words(const uint32_t (&w)[WORDS], int chunk_offset) {
    constexpr int CHUNK_BYTES = CB / 8;
    constexpr int NCHUNKS = WORDS * 4 / CHUNK_BYTES;
    constexpr int ROUNDS = ALGO == VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT ? 2 : 1;
    HashState<H, CB, ALGO> st;
    st.init();
#pragma unroll
    for (int round = 0; round < ROUNDS; round++) {
#pragma unroll
        for (int c = 0; c < NCHUNKS; c++) {
            if (c < chunk_offset) {
                continue;
            }
            if (CB == 8) {
                const uint32_t word = w[c / 4];
                st.lane((int64_t)(int8_t)(uint8_t)(word >> (8 * (c % 4))));
            } else {
#pragma unroll
                for (int l = 0; l < CB / 32; l++) {
                    st.lane((int64_t)(uint64_t)w[c * (CB / 32) + l]);
                }
            }
            st.end_chunk();
        }
    }
    return st.h;
}

// Generic element (any number of chunks): loads chunk lanes one by one.
template <typename H, int CB, int ALGO>
__device__ __forceinline__ H hash_generic(const uint8_t *elem, int chunk_offset, int element_chunks) {
    constexpr int ROUNDS = ALGO == VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT ? 2 : 1;
    HashState<H, CB, ALGO> st;
    st.init();
    for (int round = 0; round < ROUNDS; round++) {
        for (int c = chunk_offset; c < element_chunks; c++) {
            if (CB == 8) {
                st.lane((int64_t)(int8_t)__ldg(elem + c));
            } else {
                const uint32_t *p = (const uint32_t *)(elem + (size_t)c * (CB / 8));
#pragma unroll
                for (int l = 0; l < CB / 32; l++) {
                    st.lane((int64_t)(uint64_t)__ldg(p + l));
                }
            }
            st.end_chunk();
        }
    }
    return st.h;
}

template <int EB>
__device__ __forceinline__ void load_element(const uint8_t *base, uint64_t e, uint32_t (&w)[EB / 4]) {
    if (EB == 8) {
        uint2 v = __ldcs((const uint2 *)base + e);
        w[0] = v.x;
        w[1] = v.y;
    } else {
        const uint4 *p = (const uint4 *)base + e * (EB / 16);
#pragma unroll
        for (int i = 0; i < EB / 16; i++) {
            uint4 v = __ldcs(p + i);
            w[4 * i] = v.x;
            w[4 * i + 1] = v.y;
            w[4 * i + 2] = v.z;
            w[4 * i + 3] = v.w;
        }
    }
}

constexpr int HASH_THREADS = 256;
constexpr int HASH_UNROLL = 4;

// EB > 0: every element is EB bytes (8/16/32), aligned for vector loads.
// EB == 0: generic path.
template <typename H, int CB, int ALGO, int EB>
__global__ void __launch_bounds__(HASH_THREADS) hash_kernel(const uint8_t *__restrict__ in, uint64_t n, int chunk_offset, int element_chunks, H *__restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * HASH_THREADS;
    uint64_t e = (uint64_t)blockIdx.x * HASH_THREADS + threadIdx.x;
    if constexpr (EB > 0) {
        // UN independent elements per thread per step keep several loads in flight; 32-byte
        // elements run one per thread over a grid that covers them all (faster on GB300:
        // new blocks keep every SM full where grid-stride threads would serialise).
        constexpr int UN = EB == 32 ? 1 : HASH_UNROLL;
        for (; e + (UN - 1) * stride < n; e += UN * stride) {
            uint32_t w[UN][EB / 4];
#pragma unroll
            for (int u = 0; u < UN; u++) {
                load_element<EB>(in, e + u * stride, w[u]);
            }
#pragma unroll
            for (int u = 0; u < UN; u++) {
                __stcs(out + e + u * stride, hash_words<H, CB, ALGO, EB / 4>(w[u], chunk_offset));
            }
        }
        for (; e < n; e += stride) {
            uint32_t w[EB / 4];
            load_element<EB>(in, e, w);
            __stcs(out + e, hash_words<H, CB, ALGO, EB / 4>(w, chunk_offset));
        }
    } else {
        const size_t elem_bytes = (size_t)element_chunks * (CB / 8);
        for (; e < n; e += stride) {
            out[e] = hash_generic<H, CB, ALGO>(in + e * elem_bytes, chunk_offset, element_chunks);
        }
    }
}

template <typename H, int CB, int ALGO>
int launch_algo(const uint8_t *in, uint64_t n, int chunk_offset, int element_chunks, H *out, int grid, cudaStream_t stream) {
    const size_t eb = (size_t)element_chunks * (CB / 8);
    const bool aligned16 = ((uintptr_t)in % 16) == 0;
    const bool aligned8 = ((uintptr_t)in % 8) == 0;
    bool launched = false;
    if constexpr (CB <= 64) {
        if (eb == 8 && aligned8) {
            hash_kernel<H, CB, ALGO, 8><<<grid, HASH_THREADS, 0, stream>>>(in, n, chunk_offset, element_chunks, out);
            launched = true;
        }
    }
    if (!launched && eb == 16 && aligned16) {
        hash_kernel<H, CB, ALGO, 16><<<grid, HASH_THREADS, 0, stream>>>(in, n, chunk_offset, element_chunks, out);
        launched = true;
    }
    if (!launched && eb == 32 && aligned16) {
        hash_kernel<H, CB, ALGO, 32><<<grid, HASH_THREADS, 0, stream>>>(in, n, chunk_offset, element_chunks, out);
        launched = true;
    }
    if (!launched) {
        hash_kernel<H, CB, ALGO, 0><<<grid, HASH_THREADS, 0, stream>>>(in, n, chunk_offset, element_chunks, out);
    }
    return cuda_error(cudaGetLastError(), "hash kernel launch");
}

template <typename H, int CB>
int launch_cb(const uint8_t *in, uint64_t n, int chunk_offset, int element_chunks, int algo, H *out, int grid, cudaStream_t stream) {
    switch (algo) {
#define VJ_CASE(A) \
    case A:        \
        return launch_algo<H, CB, A>(in, n, chunk_offset, element_chunks, out, grid, stream);
        VJ_CASE(VJ_HASH_FNV)
        VJ_CASE(VJ_HASH_CUSTOM_XOR)
        VJ_CASE(VJ_HASH_CUSTOM_XOR_SHIFT)
        VJ_CASE(VJ_HASH_CUSTOM_XOR_HW)
        VJ_CASE(VJ_HASH_CUSTOM_MULT_XOR_SHIFT)
        VJ_CASE(VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT)
        VJ_CASE(VJ_HASH_CUSTOM_MULT_XOR_HW)
        VJ_CASE(VJ_HASH_CUSTOM_MULT)
        VJ_CASE(VJ_HASH_CUSTOM_MULT_SHIFT)
        VJ_CASE(VJ_HASH_CUSTOM_MULT_HW)
        VJ_CASE(VJ_HASH_CUSTOM_ADD)
        VJ_CASE(VJ_HASH_CUSTOM_ADD_SHIFT)
        VJ_CASE(VJ_HASH_CUSTOM_ADD_HW)
#undef VJ_CASE
    }
    return set_error(VJ_ERR_INVALID_ARGUMENT, "vj_hash: unknown algorithm id %d", algo);
}

template <typename H>
int launch_h(const uint8_t *in, uint64_t n, int chunk_offset, int element_chunks, int chunk_bits, int algo, H *out, int grid, cudaStream_t stream) {
    switch (chunk_bits) {
    case 8:
        return launch_cb<H, 8>(in, n, chunk_offset, element_chunks, algo, out, grid, stream);
    case 32:
        return launch_cb<H, 32>(in, n, chunk_offset, element_chunks, algo, out, grid, stream);
    case 64:
        return launch_cb<H, 64>(in, n, chunk_offset, element_chunks, algo, out, grid, stream);
    case 128:
        return launch_cb<H, 128>(in, n, chunk_offset, element_chunks, algo, out, grid, stream);
    }
    return set_error(VJ_ERR_INVALID_ARGUMENT, "vj_hash: chunk_bits must be 8, 32, 64 or 128 (got %d)", chunk_bits);
}

}  // namespace

}  // namespace vj

extern "C" int vj_hash(const void *d_elements, uint64_t n, int chunk_offset, int element_chunks, int chunk_bits, int hash_bits, int algo, void *d_hashes, vj_stream_t stream) {
    using namespace vj;
    VJ_CHECK(algo >= 0 && algo < VJ_HASH_COUNT, VJ_ERR_INVALID_ARGUMENT, "vj_hash: unknown algorithm id %d", algo);
    VJ_CHECK(hash_bits == 32 || hash_bits == 64, VJ_ERR_INVALID_ARGUMENT, "vj_hash: hash_bits must be 32 or 64 (got %d)", hash_bits);
    VJ_CHECK(chunk_bits == 8 || chunk_bits == 32 || chunk_bits == 64 || chunk_bits == 128, VJ_ERR_INVALID_ARGUMENT, "vj_hash: chunk_bits must be 8, 32, 64 or 128 (got %d)", chunk_bits);
    VJ_CHECK(element_chunks >= 0 && element_chunks <= 32767 && chunk_offset >= 0 && chunk_offset <= 32767, VJ_ERR_INVALID_ARGUMENT,
             "vj_hash: element_chunks and chunk_offset must be in [0, 32767] (the reference's short)");
    if (n == 0) {
        return VJ_OK;
    }
    VJ_CHECK(d_elements != nullptr && d_hashes != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_hash: null buffer");
    const uintptr_t align = (uintptr_t)(chunk_bits / 8);  // chunk_t is char, uint1, uint2 or uint4
    VJ_CHECK((uintptr_t)d_elements % align == 0, VJ_ERR_INVALID_ARGUMENT, "vj_hash: elements must be aligned to the chunk size");
    VJ_CHECK((uintptr_t)d_hashes % (hash_bits / 8) == 0, VJ_ERR_INVALID_ARGUMENT, "vj_hash: hashes must be aligned to the hash size");
    int device = 0;
    VJ_CUDA(cudaGetDevice(&device));
    DeviceInfo info;
    VJ_TRY(device_info(device, &info));
    // Grid: 8 resident blocks of 256 threads per SM, or fewer for small inputs; 32-byte
    // elements (one per thread) get a block per 256 elements.
    const bool wide = chunk_bits >= 32 && element_chunks * (chunk_bits / 8) == 32 && chunk_offset == 0;
    const uint64_t per_block = (uint64_t)HASH_THREADS * (wide ? 1 : HASH_UNROLL);
    uint64_t blocks = (n + per_block - 1) / per_block;
    const uint64_t max_blocks = wide ? (1ull << 31) - 1 : (uint64_t)info.sms * 8;
    int grid = (int)(blocks < max_blocks ? (blocks ? blocks : 1) : max_blocks);
    const uint8_t *in = (const uint8_t *)d_elements;
    cudaStream_t s = (cudaStream_t)stream;
    if (hash_bits == 64) {
        return launch_h<uint64_t>(in, n, chunk_offset, element_chunks, chunk_bits, algo, (uint64_t *)d_hashes, grid, s);
    }
    return launch_h<uint32_t>(in, n, chunk_offset, element_chunks, chunk_bits, algo, (uint32_t *)d_hashes, grid, s);
}
