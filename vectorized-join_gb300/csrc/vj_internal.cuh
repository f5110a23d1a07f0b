// vj_internal.cuh -- shared device helpers and host plumbing of the sm_103a join library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <vector>

#include "vj.h"

namespace vj {

// ------------------------------------------------------------------ host errors

int set_error(int status, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);

#define VJ_CUDA(expr)                                                \
    do {                                                             \
        cudaError_t vj_e_ = (expr);                                  \
        if (vj_e_ != cudaSuccess) return ::vj::cuda_error(vj_e_, #expr); \
    } while (0)

#define VJ_CHECK(cond, status, ...)                                  \
    do {                                                             \
        if (!(cond)) return ::vj::set_error((status), __VA_ARGS__);  \
    } while (0)

#define VJ_TRY(expr)                                                 \
    do {                                                             \
        int vj_s_ = (expr);                                          \
        if (vj_s_ != VJ_OK) return vj_s_;                            \
    } while (0)

// ------------------------------------------------------------------ hashing

__host__ __device__ __forceinline__ uint64_t fmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t pair_digest(uint64_t r, uint64_t s) {
    return fmix64(r ^ fmix64(s + 0x9e3779b97f4a7c15ull));
}

template <typename H>
struct HashTraits;
template <>
struct HashTraits<uint64_t> {
    static constexpr int bits = 64;
    static constexpr uint64_t prime = 1099511628211ull;          // 2^40 + 2^8 + 0xb3
    static constexpr uint64_t basis = 14695981039346656037ull;
};
template <>
struct HashTraits<uint32_t> {
    static constexpr int bits = 32;
    static constexpr uint32_t prime = 16777619u;                 // 2^24 + 2^8 + 0x93
    static constexpr uint32_t basis = 2166136261u;
};

__device__ __forceinline__ uint32_t reverse_bits(uint32_t x) { return __brev(x); }
__device__ __forceinline__ uint64_t reverse_bits(uint64_t x) { return __brevll(x); }
__device__ __forceinline__ uint32_t rotl32(uint32_t v, uint32_t s) { return __funnelshift_l(v, v, s); }

// The reference's get_max_shift() (hash.cu:60-62) with its integer types.
__host__ __device__ constexpr int32_t max_shift_of(int hash_bits, int chunk_bits) {
    return (int32_t)(uint16_t)((int32_t)(uint16_t)((uint64_t)(hash_bits / 8) - (uint64_t)(chunk_bits / 8) * 8u) + 1);
}

// State of one element's hash for algorithm ALGO with hash type H and chunk width CB.
// lane() takes each chunk lane widened as C widens it: a sign-extended char for CB == 8,
// a zero-extended 32-bit word otherwise. Mirrors hash.cu:84-505 operation by operation.
template <typename H, int CB, int ALGO>
struct HashState {
    static constexpr int HB = HashTraits<H>::bits;
    static constexpr int32_t MS = max_shift_of(HB, CB);
    H h;
    int32_t shift_i;
    uint32_t shift_u;
    int16_t off;
    int16_t op;

    __device__ __forceinline__ void init() {
        shift_i = 0;
        shift_u = 0;
        off = 0;
        op = 0;
        if (ALGO == VJ_HASH_FNV) {
            h = HashTraits<H>::basis;
        } else if (ALGO == VJ_HASH_CUSTOM_MULT || ALGO == VJ_HASH_CUSTOM_MULT_SHIFT || ALGO == VJ_HASH_CUSTOM_MULT_HW) {
            h = 1;
        } else {
            h = 0;
        }
    }
    // value << amount, where amounts outside [0, HB) give 0 (the PTX shl clamp).
    __device__ __forceinline__ static H shl(H v, int32_t amount) {
        return (uint32_t)amount >= (uint32_t)HB ? H(0) : H(v << amount);
    }
    __device__ __forceinline__ void offset_from_lane(int64_t lane) {
        if (CB == 8) {
            int32_t sum = (int32_t)off + (int32_t)lane;
            off = (int16_t)(sum % MS);
        } else {
            uint32_t sum = (uint32_t)(int32_t)off + (uint32_t)lane;
            off = (int16_t)(uint16_t)(sum % (uint32_t)MS);
        }
    }
    __device__ __forceinline__ void offset_from_hash(H ch) {
        H sum = (H)(int64_t)off + ch;
        off = (int16_t)(uint16_t)(sum % (H)MS);
    }
    __device__ __forceinline__ void lane(int64_t lv) {
        const H ch = (H)lv;
        const uint32_t u = (uint32_t)lv;
        switch (ALGO) {
        case VJ_HASH_FNV:
            h = (H)((h ^ ch) * HashTraits<H>::prime);
            break;
        case VJ_HASH_CUSTOM_ADD:
            h = (H)(h + ch);
            break;
        case VJ_HASH_CUSTOM_ADD_SHIFT:
            offset_from_lane(lv);
            h = (H)(h + shl(ch, off));
            break;
        case VJ_HASH_CUSTOM_ADD_HW:
            h = (H)(h + (H)rotl32(u, (uint32_t)shift_i));
            shift_i++;
            break;
        case VJ_HASH_CUSTOM_XOR:
            h ^= ch;
            break;
        case VJ_HASH_CUSTOM_XOR_SHIFT:
            offset_from_lane(lv);
            h ^= shl(ch, off);
            break;
        case VJ_HASH_CUSTOM_XOR_HW:
            shift_u += u;
            h ^= (H)rotl32(u, shift_u);
            h = reverse_bits(h);
            break;
        case VJ_HASH_CUSTOM_MULT:
            h = (H)(1u + h * (H)(ch + 1u));
            break;
        case VJ_HASH_CUSTOM_MULT_SHIFT:
            offset_from_lane(lv);
            h = (H)(1u + shl((H)(h * (H)(ch + 1u)), off));
            break;
        case VJ_HASH_CUSTOM_MULT_HW:
            shift_i = (int32_t)((uint32_t)shift_i + u);
            h = (H)(1u + h * (H)((H)rotl32(u, (uint32_t)shift_i) + 1u));
            h = reverse_bits(h);
            break;
        case VJ_HASH_CUSTOM_MULT_XOR_SHIFT:
        case VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT:
            offset_from_hash(ch);
            if (op & 1) {
                h = (H)(1u + h * shl((H)(ch + 1u), off));
            } else {
                h = (H)(h ^ shl(ch, off));
            }
            op = (int16_t)(op + 1);
            break;
        case VJ_HASH_CUSTOM_MULT_XOR_HW:
            if (op & 1) {
                h = (H)(1u + h * (H)rotl32((uint32_t)(H)(ch + 1u), (uint32_t)(int32_t)off));
            } else {
                h = (H)(h ^ (H)rotl32((uint32_t)ch, (uint32_t)(int32_t)off));
            }
            op = (int16_t)(op + 1);
            off = (int16_t)(uint16_t)((uint64_t)(int64_t)off + (uint64_t)ch);
            h = reverse_bits(h);
            break;
        }
    }
    __device__ __forceinline__ void end_chunk() {
        if (ALGO == VJ_HASH_CUSTOM_ADD_HW) {
            h = reverse_bits(h);
        }
    }
};

// FNV-1a over the 32-bit words of a key row: the reference's hash of a join key row
// (JoinProvider::hash_table feeds the key columns to hash_fnv, join_provider.cuh:926-931).
template <typename H, int KW>
__device__ __forceinline__ H fnv_words(const uint32_t (&w)[KW]) {
    H h = HashTraits<H>::basis;
#pragma unroll
    for (int i = 0; i < KW; i++) {
        h = (H)((h ^ (H)w[i]) * HashTraits<H>::prime);
    }
    return h;
}

// ------------------------------------------------------------------ key rows

template <int KW>
struct Key {
    uint32_t w[KW];
};

template <int KW>
__device__ __forceinline__ Key<KW> load_key(const void *base, uint64_t row) {
    Key<KW> k;
    if (KW == 1) {
        k.w[0] = __ldg((const uint32_t *)base + row);
    } else {
        const uint2 *p = (const uint2 *)base + row * (KW / 2);
#pragma unroll
        for (int i = 0; i < KW / 2; i++) {
            uint2 v = __ldg(p + i);
            k.w[2 * i] = v.x;
            k.w[2 * i + 1] = v.y;
        }
    }
    return k;
}

// Streaming load: the row is read once, keep it out of L1.
template <int KW>
__device__ __forceinline__ Key<KW> load_key_stream(const void *base, uint64_t row) {
    Key<KW> k;
    if (KW == 1) {
        k.w[0] = __ldcs((const uint32_t *)base + row);
    } else {
        const uint2 *p = (const uint2 *)base + row * (KW / 2);
#pragma unroll
        for (int i = 0; i < KW / 2; i++) {
            uint2 v = __ldcs(p + i);
            k.w[2 * i] = v.x;
            k.w[2 * i + 1] = v.y;
        }
    }
    return k;
}

template <int KW>
__device__ __forceinline__ void store_key(void *base, uint64_t row, const Key<KW> &k) {
    if (KW == 1) {
        ((uint32_t *)base)[row] = k.w[0];
    } else {
        uint2 *p = (uint2 *)base + row * (KW / 2);
#pragma unroll
        for (int i = 0; i < KW / 2; i++) {
            p[i] = make_uint2(k.w[2 * i], k.w[2 * i + 1]);
        }
    }
}

template <int KW>
__device__ __forceinline__ bool key_equal(const Key<KW> &a, const Key<KW> &b) {
    bool eq = true;
#pragma unroll
    for (int i = 0; i < KW; i++) {
        eq &= a.w[i] == b.w[i];
    }
    return eq;
}

template <int PB>
struct PayloadType;
template <>
struct PayloadType<4> {
    using T = uint32_t;
};
template <>
struct PayloadType<8> {
    using T = unsigned long long;
};

// ------------------------------------------------------------------ bulk copies (TMA engine)
//
// 1-D global->shared copies by the Blackwell bulk-copy (TMA) engine, completing on an
// mbarrier with a transaction count, and shared->global bulk stores. Every wait is bounded:
// after WAIT_NS nanoseconds of polling the caller gets `false` and is expected to flag the
// error and leave (a legitimate wait lasts microseconds).

constexpr uint64_t WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation and earlier generic-proxy accesses of shared memory
// visible to the async proxy (issue before handing a buffer to a bulk copy).
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase of `bar` with the given parity to complete; false once WAIT_NS have
// passed without it.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 16; i++) {
            if (mbar_try_wait(bar, parity)) return true;
        }
        if (global_ns() - t0 > WAIT_NS) return false;
    }
}

// Plain arrival (release at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}

// Named barrier `id` over `count` threads (a multiple of 32) that also ORs a predicate:
// every participating thread gets true if any passed true.
__device__ __forceinline__ bool bar_or(uint32_t id, uint32_t count, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, %2, %3, q;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id), "r"(count)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void bar_sync(uint32_t id, uint32_t count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Shared->global bulk store (dst, src 16-byte aligned; bytes a multiple of 16), tracked by
// the issuing thread's bulk groups.
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// The issuing thread's bulk stores have read their shared-memory sources.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// The issuing thread's bulk stores are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Stores under an L2 evict-last policy. A partition pass writes each bucket's rows as
// runs that start at any 16-byte offset, so a run's first and last 32-byte sectors are
// only partly written until the next tile's run of the same bucket completes them; kept in
// L2 until then, they go to HBM once and whole instead of being read back and merged (for
// the 2^27 x 2^29 join the two scatter passes went from 6.05 + 5.22 to 5.84 + 5.02 ms).
__device__ __forceinline__ uint64_t l2_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void st_evict_last(void *p, const uint4 &v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_evict_last(void *p, const uint2 &v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(p), "r"(v.x), "r"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_evict_last(uint16_t *p, uint16_t v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.u16 [%0], %1, %2;" ::"l"(p), "h"(v), "l"(pol) : "memory");
}

// Prefetch [src, src + bytes) into L2 through the bulk-copy engine (no completion to wait
// for; src 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// The 16-byte aligned window of global memory that covers rows [a, b) of a column with
// `cb`-byte rows starting at `base`. Bytes outside the column inside that window share a
// 16-byte chunk with column bytes, so reading them cannot cross a page boundary.
struct ColWindow {
    const unsigned char *src;  // window start (16-byte aligned)
    uint32_t bytes;            // window size (multiple of 16)
    uint32_t delta;            // offset of row a inside the window
};

__device__ __forceinline__ ColWindow col_window(const void *base, uint32_t cb, uint32_t a, uint32_t b) {
    const uintptr_t lo = (uintptr_t)base + (uintptr_t)a * cb;
    const uintptr_t hi = (uintptr_t)base + (uintptr_t)b * cb;
    const uintptr_t wlo = lo & ~(uintptr_t)15;
    const uintptr_t whi = (hi + 15) & ~(uintptr_t)15;
    ColWindow w;
    w.src = (const unsigned char *)wlo;
    w.bytes = (uint32_t)(whi - wlo);
    w.delta = (uint32_t)(lo - wlo);
    return w;
}

// Key of KW words at byte address p in shared memory (p aligned to 8 for KW >= 2, 4 for KW 1).
template <int KW>
__device__ __forceinline__ Key<KW> key_from_smem(const unsigned char *p) {
    Key<KW> k;
    if (KW == 1) {
        k.w[0] = *(const uint32_t *)p;
    } else {
#pragma unroll
        for (int i = 0; i < KW / 2; i++) {
            uint2 v = ((const uint2 *)p)[i];
            k.w[2 * i] = v.x;
            k.w[2 * i + 1] = v.y;
        }
    }
    return k;
}

template <int KW>
__device__ __forceinline__ void key_to_smem(unsigned char *p, const Key<KW> &k) {
    if (KW == 1) {
        *(uint32_t *)p = k.w[0];
    } else {
#pragma unroll
        for (int i = 0; i < KW / 2; i++) ((uint2 *)p)[i] = make_uint2(k.w[2 * i], k.w[2 * i + 1]);
    }
}

// ------------------------------------------------------------------ host side

struct DeviceInfo {
    int device = 0;
    int sms = 0;
    size_t smem_optin = 0;
    size_t l2_bytes = 0;
};

int device_info(int device, DeviceInfo *out);

// Tuning cache: the fastest plan found for a class of join shapes.
struct TuneKey {
    int32_t kw, pb, lg_r, lg_s, algo, hash_bits;
    bool operator==(const TuneKey &o) const { return kw == o.kw && pb == o.pb && lg_r == o.lg_r && lg_s == o.lg_s && algo == o.algo && hash_bits == o.hash_bits; }
};
struct TuneEntry {
    TuneKey key;
    vj_join_options opt;
    float ms;
};

}  // namespace vj

// Context (defined in vj_runtime.cu).
struct vj_ctx {
    int device;
    vj::DeviceInfo info;
    uint64_t budget;        // 0 = unbounded
    void *workspace;
    size_t workspace_bytes;
    uint64_t owned_bytes;   // library-owned results
    void *stage;            // device staging for vj_join_host
    size_t stage_bytes;
    // vj_join_host's pipeline: a stream for copies in, one for copies out, and its events
    // (created on first use: call start, copies in done, copies out done, build side copied
    // in, then one per probe-side chunk copied in and one per chunk joined, up to 16 chunks)
    cudaStream_t host_in, host_out;
    cudaEvent_t host_ev[4 + 2 * 16];
    bool host_ready;
    bool profiling;
    cudaEvent_t events[16];  // created on first use
    bool events_ready;
    vj_profile last;         // filled after each join when profiling
    int launches;            // library kernels launched by the current join
    int sm_reserve;          // SMs the join's kernels leave free (vj_join_host's copy kernels run there)
    std::vector<vj::TuneEntry> tuned;  // vj_tune results, consulted by automatic joins
};

namespace vj {
// Stage event marks of a profiled join (no-ops when profiling is off).
enum ProfileMark {
    PM_PASS0 = 0,  // + 4 * pass: before plan_units
    PM_HIST_END = 1,
    PM_SCAN_END = 2,
    PM_SCATTER_END = 3,
    PM_PROBE_BEGIN = 8,
    PM_PROBE_END = 9,
    PM_COUNT = 10
};
void profile_mark(vj_ctx *ctx, int mark, cudaStream_t stream);
// Grows the context workspace to at least `bytes` (stream-ordered; contents not kept).
int workspace_reserve(vj_ctx *ctx, size_t bytes, cudaStream_t stream, void **out);
int owned_alloc(vj_ctx *ctx, size_t bytes, cudaStream_t stream, void **out);
// Counts one device or page-locked host allocation made by the library (vj_allocation_count).
void note_allocation();
void owned_release(vj_ctx *ctx, size_t bytes);
// Shape class of a join (vj_tune's cache key) and the tuned options for an automatic join.
TuneKey tune_key(const vj_table *r, const vj_table *s, const vj_join_options *opt);
const vj_join_options *tuned_options(const vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *opt);
// Upper estimate of the device bytes a vj_join of r and s takes from a context.
int join_footprint(const vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *opt, uint64_t *bytes);
}  // namespace vj
