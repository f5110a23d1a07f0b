// vj_runtime.cu -- errors, context and workspace, pair digest, seeded workload generator.
#include "vj_internal.cuh"

#include <atomic>

#include <cstring>
#include <mutex>
#include <string>

namespace vj {

namespace {
thread_local char g_last_error[512] = "";
std::mutex g_info_mutex;
DeviceInfo g_info[64];
bool g_info_valid[64] = {};
}  // namespace

int set_error(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_error(cudaError_t e, const char *what) {
    if (e == cudaSuccess) {
        return VJ_OK;
    }
    return set_error(e == cudaErrorMemoryAllocation ? VJ_ERR_OUT_OF_MEMORY : VJ_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int device_info(int device, DeviceInfo *out) {
    VJ_CHECK(device >= 0 && device < 64, VJ_ERR_INVALID_ARGUMENT, "device index %d out of range", device);
    std::lock_guard<std::mutex> lock(g_info_mutex);
    if (!g_info_valid[device]) {
        DeviceInfo d;
        d.device = device;
        VJ_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, device));
        int v = 0;
        VJ_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        d.smem_optin = (size_t)v;
        VJ_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, device));
        d.l2_bytes = (size_t)v;
        g_info[device] = d;
        g_info_valid[device] = true;
    }
    *out = g_info[device];
    return VJ_OK;
}

int workspace_reserve(vj_ctx *ctx, size_t bytes, cudaStream_t stream, void **out) {
    if (bytes <= ctx->workspace_bytes && ctx->workspace) {
        *out = ctx->workspace;
        return VJ_OK;
    }
    // Grow by 1/8 beyond the request so that slightly larger calls do not reallocate.
    size_t want = bytes + bytes / 8;
    uint64_t after = ctx->owned_bytes + ctx->stage_bytes + want;
    if (ctx->budget && after > ctx->budget) {
        want = bytes;
        after = ctx->owned_bytes + ctx->stage_bytes + want;
    }
    VJ_CHECK(!ctx->budget || after <= ctx->budget, VJ_ERR_BUDGET, "workspace of %zu bytes exceeds the context budget (%llu bytes, %llu in use)", bytes, (unsigned long long)ctx->budget,
             (unsigned long long)(ctx->owned_bytes + ctx->stage_bytes));
    if (ctx->workspace) {
        VJ_CUDA(cudaFreeAsync(ctx->workspace, stream));
        ctx->workspace = nullptr;
        ctx->workspace_bytes = 0;
    }
    void *p = nullptr;
    VJ_CUDA(cudaMallocAsync(&p, want, stream));
    note_allocation();
    ctx->workspace = p;
    ctx->workspace_bytes = want;
    *out = p;
    return VJ_OK;
}

namespace {
std::atomic<uint64_t> g_allocations{0};
}

void note_allocation() { g_allocations.fetch_add(1, std::memory_order_relaxed); }

int owned_alloc(vj_ctx *ctx, size_t bytes, cudaStream_t stream, void **out) {
    uint64_t after = ctx->owned_bytes + ctx->workspace_bytes + ctx->stage_bytes + bytes;
    VJ_CHECK(!ctx->budget || after <= ctx->budget, VJ_ERR_BUDGET, "result of %zu bytes exceeds the context budget (%llu bytes)", bytes, (unsigned long long)ctx->budget);
    void *p = nullptr;
    VJ_CUDA(cudaMallocAsync(&p, bytes ? bytes : 16, stream));
    note_allocation();
    ctx->owned_bytes += bytes;
    *out = p;
    return VJ_OK;
}

void profile_mark(vj_ctx *ctx, int mark, cudaStream_t stream) {
    if (!ctx || !ctx->profiling) {
        return;
    }
    if (!ctx->events_ready) {
        for (int i = 0; i < 16; i++) {
            cudaEventCreate(&ctx->events[i]);
        }
        ctx->events_ready = true;
    }
    cudaEventRecord(ctx->events[mark], stream);
}

void owned_release(vj_ctx *ctx, size_t bytes) {
    ctx->owned_bytes = ctx->owned_bytes >= bytes ? ctx->owned_bytes - bytes : 0;
}

namespace {

// ------------------------------------------------------------------ pair digest

template <typename P>
__global__ void __launch_bounds__(256) digest_kernel(const P *__restrict__ pairs, uint64_t count, unsigned long long *sum_xor) {
    uint64_t s = 0, x = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t d = pair_digest((uint64_t)pairs[2 * i], (uint64_t)pairs[2 * i + 1]);
        s += d;
        x ^= d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        x ^= __shfl_xor_sync(0xffffffffu, x, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sum_xor[0], (unsigned long long)s);
        atomicXor(&sum_xor[1], (unsigned long long)x);
    }
}

// ------------------------------------------------------------------ generator
// Same formulas as the CPU oracle's generator (oracle/vj_oracle.c).

__host__ __device__ __forceinline__ uint64_t gen_stream(uint64_t seed, uint64_t tag) {
    return fmix64(seed * 0xd1b54a32d192ed03ull + tag * 0xaef17502108ef2d9ull + 0x243f6a8885a308d3ull);
}

__device__ __forceinline__ uint64_t rng_at(uint64_t stream_base, uint64_t i) {
    return fmix64(stream_base + (i + 1) * 0x9e3779b97f4a7c15ull);
}

__device__ __forceinline__ uint32_t ukey31(uint64_t base101, uint64_t i) {
    const uint32_t m = 0x7fffffffu;
    uint32_t x = (uint32_t)((i + base101) & m);
    x = (x * 0x6b43a9b5u + 0x1234567u) & m;
    x ^= x >> 16;
    x = (x * 0x2c1b3c6du + 0x7654321u) & m;
    x ^= x >> 13;
    x = (x * 0x297a2d39u) & m;
    x ^= x >> 16;
    return x;
}

struct GenArgs {
    uint64_t nr, ns, thr;
    uint64_t base_key64, base_key31, base_coin, base_row;
    int key_bytes, payload_bytes;
    void *rk, *rp, *sk, *sp;
};

constexpr uint64_t MISS_BASE64 = 1ull << 62;

__global__ void __launch_bounds__(256) gen_kernel(GenArgs a) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.nr; i += stride) {
        if (a.key_bytes == 8) {
            ((uint64_t *)a.rk)[i] = fmix64(i + a.base_key64);
        } else {
            ((uint32_t *)a.rk)[i] = ukey31(a.base_key31, i);
        }
        if (a.payload_bytes == 8) {
            ((uint64_t *)a.rp)[i] = i;
        } else {
            ((uint32_t *)a.rp)[i] = (uint32_t)i;
        }
    }
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < a.ns; j += stride) {
        const bool hit = a.nr > 0 && (rng_at(a.base_coin, j) >> 32) < a.thr;
        const uint64_t row = hit ? rng_at(a.base_row, j) % a.nr : 0;
        if (a.key_bytes == 8) {
            ((uint64_t *)a.sk)[j] = fmix64((hit ? row : MISS_BASE64 + j) + a.base_key64);
        } else {
            ((uint32_t *)a.sk)[j] = ukey31(a.base_key31, hit ? row : a.nr + j);
        }
        if (a.payload_bytes == 8) {
            ((uint64_t *)a.sp)[j] = j;
        } else {
            ((uint32_t *)a.sp)[j] = (uint32_t)j;
        }
    }
}

__global__ void __launch_bounds__(256) gen_expect_kernel(GenArgs a, unsigned long long *acc) {
    uint64_t c = 0, s = 0, x = 0;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < a.ns; j += (uint64_t)gridDim.x * blockDim.x) {
        if (a.nr > 0 && (rng_at(a.base_coin, j) >> 32) < a.thr) {
            uint64_t row = rng_at(a.base_row, j) % a.nr;
            uint64_t d = pair_digest(row, j);
            c++;
            s += d;
            x ^= d;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        s += __shfl_xor_sync(0xffffffffu, s, o);
        x ^= __shfl_xor_sync(0xffffffffu, x, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], (unsigned long long)c);
        atomicAdd(&acc[1], (unsigned long long)s);
        atomicXor(&acc[2], (unsigned long long)x);
    }
}

GenArgs make_gen_args(uint64_t seed, int key_bytes, int payload_bytes, uint64_t nr, uint64_t ns, uint64_t thr) {
    GenArgs a;
    a.nr = nr;
    a.ns = ns;
    a.thr = thr;
    a.base_key64 = gen_stream(seed, 100);
    a.base_key31 = gen_stream(seed, 101);
    a.base_coin = gen_stream(seed, 1);
    a.base_row = gen_stream(seed, 2);
    a.key_bytes = key_bytes;
    a.payload_bytes = payload_bytes;
    a.rk = a.rp = a.sk = a.sp = nullptr;
    return a;
}

int grid_for(uint64_t n, int per_sm) {
    int device = 0;
    cudaGetDevice(&device);
    DeviceInfo info;
    if (device_info(device, &info) != VJ_OK) {
        info.sms = 148;
    }
    uint64_t blocks = (n + 255) / 256;
    uint64_t cap = (uint64_t)info.sms * per_sm;
    return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

// Small device scratch for results read back by the host (one per device, reused).
int host_result_scratch(unsigned long long **d, unsigned long long **h) {
    static thread_local unsigned long long *dev[64] = {};
    static thread_local unsigned long long *pinned = nullptr;
    int device = 0;
    VJ_CUDA(cudaGetDevice(&device));
    VJ_CHECK(device >= 0 && device < 64, VJ_ERR_UNSUPPORTED, "device %d is beyond the 64 devices the library keeps result words for", device);
    if (!dev[device]) {
        VJ_CUDA(cudaMalloc(&dev[device], 4 * sizeof(unsigned long long)));
        note_allocation();
    }
    if (!pinned) {
        VJ_CUDA(cudaMallocHost(&pinned, 4 * sizeof(unsigned long long)));
        note_allocation();
    }
    *d = dev[device];
    *h = pinned;
    return VJ_OK;
}

}  // namespace

}  // namespace vj

// ====================================================================== C ABI

static const char *const kAlgoNames[VJ_HASH_COUNT] = {
    "fnv", "custom_xor", "custom_xor_shift", "custom_xor_hw", "custom_mult_xor_shift", "custom_n_mult_xor_shift", "custom_mult_xor_hw", "custom_mult", "custom_mult_shift", "custom_mult_hw", "custom_add", "custom_add_shift", "custom_add_hw",
};

extern "C" int vj_version(void) {
    return 10000;  // 1.0.0
}

extern "C" const char *vj_status_string(int status) {
    switch (status) {
    case VJ_OK: return "ok";
    case VJ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VJ_ERR_UNSUPPORTED: return "unsupported";
    case VJ_ERR_CUDA: return "CUDA error";
    case VJ_ERR_OUT_OF_MEMORY: return "out of device memory";
    case VJ_ERR_CAPACITY: return "output capacity too small";
    case VJ_ERR_DEVICE: return "device-side limit reached";
    case VJ_ERR_BUDGET: return "memory budget exceeded";
    }
    return "unknown status";
}

extern "C" size_t vj_last_error(char *buf, size_t len) {
    size_t n = strlen(vj::g_last_error);
    if (buf && len) {
        size_t c = n < len - 1 ? n : len - 1;
        memcpy(buf, vj::g_last_error, c);
        buf[c] = 0;
    }
    return n;
}

extern "C" int vj_hash_algo_id(const char *name) {
    if (!name) {
        return -1;
    }
    for (int i = 0; i < VJ_HASH_COUNT; i++) {
        if (strcmp(name, kAlgoNames[i]) == 0) {
            return i;
        }
    }
    return -1;
}

extern "C" const char *vj_hash_algo_name(int algo) {
    return algo >= 0 && algo < VJ_HASH_COUNT ? kAlgoNames[algo] : nullptr;
}

extern "C" int vj_ctx_create(int device, uint64_t memory_budget_bytes, vj_ctx **out) {
    using namespace vj;
    VJ_CHECK(out != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_ctx_create: out is null");
    *out = nullptr;
    int count = 0;
    VJ_CUDA(cudaGetDeviceCount(&count));
    VJ_CHECK(device >= 0 && device < count, VJ_ERR_INVALID_ARGUMENT, "vj_ctx_create: device %d of %d", device, count);
    VJ_CUDA(cudaSetDevice(device));
    // Keep freed stream-ordered memory in the device's default pool instead of unmapping it
    // at every synchronisation, so repeated joins do not remap their workspace. This is a
    // property of this process's pool, not of the GPU.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    vj_ctx *c = new vj_ctx();
    c->device = device;
    c->budget = memory_budget_bytes;
    c->workspace = nullptr;
    c->workspace_bytes = 0;
    c->owned_bytes = 0;
    c->stage = nullptr;
    c->stage_bytes = 0;
    c->host_in = c->host_out = nullptr;
    c->host_ready = false;
    c->profiling = false;
    c->events_ready = false;
    memset(&c->last, 0, sizeof(c->last));
    c->launches = 0;
    int st = device_info(device, &c->info);
    if (st != VJ_OK) {
        delete c;
        return st;
    }
    *out = c;
    return VJ_OK;
}

extern "C" int vj_ctx_trim(vj_ctx *ctx) {
    using namespace vj;
    VJ_CHECK(ctx != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_ctx_trim: null context");
    VJ_CUDA(cudaSetDevice(ctx->device));
    VJ_CUDA(cudaDeviceSynchronize());
    if (ctx->workspace) {
        VJ_CUDA(cudaFree(ctx->workspace));
    }
    if (ctx->stage) {
        VJ_CUDA(cudaFree(ctx->stage));
    }
    ctx->workspace = nullptr;
    ctx->workspace_bytes = 0;
    ctx->stage = nullptr;
    ctx->stage_bytes = 0;
    return VJ_OK;
}

extern "C" int vj_ctx_set_profiling(vj_ctx *ctx, int enabled) {
    using namespace vj;
    VJ_CHECK(ctx != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_ctx_set_profiling: null context");
    ctx->profiling = enabled != 0;
    return VJ_OK;
}

extern "C" int vj_ctx_last_profile(const vj_ctx *ctx, vj_profile *out) {
    using namespace vj;
    VJ_CHECK(ctx != nullptr && out != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_ctx_last_profile: null argument");
    *out = ctx->last;
    return VJ_OK;
}

extern "C" int vj_ctx_destroy(vj_ctx *ctx) {
    if (!ctx) {
        return VJ_OK;
    }
    if (ctx->events_ready) {
        for (int i = 0; i < 16; i++) {
            cudaEventDestroy(ctx->events[i]);
        }
    }
    int st = vj_ctx_trim(ctx);
    if (ctx->host_ready) {
        cudaSetDevice(ctx->device);
        for (cudaEvent_t e : ctx->host_ev) cudaEventDestroy(e);
        cudaStreamDestroy(ctx->host_in);
        cudaStreamDestroy(ctx->host_out);
    }
    delete ctx;
    return st;
}

extern "C" uint64_t vj_ctx_memory_in_use(const vj_ctx *ctx) {
    return ctx ? ctx->owned_bytes + ctx->workspace_bytes + ctx->stage_bytes : 0;
}

extern "C" int vj_result_free(vj_ctx *ctx, vj_result *result) {
    using namespace vj;
    VJ_CHECK(ctx && result, VJ_ERR_INVALID_ARGUMENT, "vj_result_free: null argument");
    if (result->owned && result->pairs) {
        VJ_CUDA(cudaFree(result->pairs));
        owned_release(ctx, (size_t)result->capacity * 2 * (size_t)(result->payload_bytes ? result->payload_bytes : 8));
    }
    result->pairs = nullptr;
    result->count = 0;
    result->capacity = 0;
    result->owned = 0;
    return VJ_OK;
}

extern "C" int vj_pairs_digest(const void *d_pairs, uint64_t count, int payload_bytes, uint64_t *h_sum, uint64_t *h_xor, vj_stream_t stream) {
    using namespace vj;
    VJ_CHECK(payload_bytes == 4 || payload_bytes == 8, VJ_ERR_INVALID_ARGUMENT, "vj_pairs_digest: payload_bytes must be 4 or 8");
    VJ_CHECK(count == 0 || d_pairs, VJ_ERR_INVALID_ARGUMENT, "vj_pairs_digest: null pairs");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *d, *h;
    VJ_TRY(host_result_scratch(&d, &h));
    VJ_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s));
    if (count) {
        int grid = grid_for(count, 8);
        if (payload_bytes == 8) {
            digest_kernel<unsigned long long><<<grid, 256, 0, s>>>((const unsigned long long *)d_pairs, count, d);
        } else {
            digest_kernel<uint32_t><<<grid, 256, 0, s>>>((const uint32_t *)d_pairs, count, d);
        }
        VJ_CUDA(cudaGetLastError());
    }
    VJ_CUDA(cudaMemcpyAsync(h, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    VJ_CUDA(cudaStreamSynchronize(s));
    if (h_sum) *h_sum = h[0];
    if (h_xor) *h_xor = h[1];
    return VJ_OK;
}

extern "C" int vj_generate_join(uint64_t seed, int key_bytes, int payload_bytes, uint64_t nr, uint64_t ns, uint64_t match_threshold, void *d_r_keys, void *d_r_payloads, void *d_s_keys, void *d_s_payloads,
                                vj_stream_t stream) {
    using namespace vj;
    VJ_CHECK(key_bytes == 4 || key_bytes == 8, VJ_ERR_INVALID_ARGUMENT, "vj_generate_join: key_bytes must be 4 or 8");
    VJ_CHECK(payload_bytes == 4 || payload_bytes == 8, VJ_ERR_INVALID_ARGUMENT, "vj_generate_join: payload_bytes must be 4 or 8");
    VJ_CHECK(key_bytes == 8 || nr + ns <= (1ull << 31), VJ_ERR_INVALID_ARGUMENT, "vj_generate_join: 4-byte keys need |R| + |S| <= 2^31");
    VJ_CHECK((nr == 0 || (d_r_keys && d_r_payloads)) && (ns == 0 || (d_s_keys && d_s_payloads)), VJ_ERR_INVALID_ARGUMENT, "vj_generate_join: null buffer");
    GenArgs a = make_gen_args(seed, key_bytes, payload_bytes, nr, ns, match_threshold);
    a.rk = d_r_keys;
    a.rp = d_r_payloads;
    a.sk = d_s_keys;
    a.sp = d_s_payloads;
    gen_kernel<<<grid_for(nr > ns ? nr : ns, 16), 256, 0, (cudaStream_t)stream>>>(a);
    return cuda_error(cudaGetLastError(), "gen_kernel launch");
}

extern "C" int vj_generate_join_expect(uint64_t seed, uint64_t nr, uint64_t ns, uint64_t match_threshold, uint64_t *count, uint64_t *h_sum, uint64_t *h_xor, vj_stream_t stream) {
    using namespace vj;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *d, *h;
    VJ_TRY(host_result_scratch(&d, &h));
    VJ_CUDA(cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), s));
    GenArgs a = make_gen_args(seed, 8, 8, nr, ns, match_threshold);
    gen_expect_kernel<<<grid_for(ns, 8), 256, 0, s>>>(a, d);
    VJ_CUDA(cudaGetLastError());
    VJ_CUDA(cudaMemcpyAsync(h, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    VJ_CUDA(cudaStreamSynchronize(s));
    if (count) *count = h[0];
    if (h_sum) *h_sum = h[1];
    if (h_xor) *h_xor = h[2];
    return VJ_OK;
}

extern "C" uint64_t vj_allocation_count(void) { return vj::g_allocations.load(std::memory_order_relaxed); }
