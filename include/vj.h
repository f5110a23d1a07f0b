/*
 * vj.h -- C ABI of the GB300 (sm_103a) hash-join library.
 *
 * Drop-in boundary for the hash and join path of vgerber/vectorized-join:
 *   vj_hash          replaces hash_func                (src/hash/hash.cu:507-557)
 *   vj_partition     replaces partition_gpu            (src/join/join_provider.cu:610-661)
 *   vj_build_probe   replaces build_and_probe_gpu      (src/join/join_provider.cu:669-847)
 *   vj_join          replaces JoinProvider::join       (src/join/join_provider.cuh:230-421)
 *   vj_result_free   replaces db_table::free of the rs table the join allocates
 *                                                      (src/base/types.hpp:235-261)
 * The reference exposes these as C++ functions over db_table/db_hash_table structs and
 * compile-time hash/chunk widths (src/base/config.h:27-31); here the widths are runtime
 * arguments and every call returns a status instead of exiting the process
 * (src/base/debug.cuh:64-82). include/vj_compat.hpp rebuilds the reference's C++ names on
 * top of this header.
 *
 * Conventions
 *   - Every function returns an int status (VJ_OK = 0). vj_last_error() gives the message
 *     of the last failure on the calling thread.
 *   - Pointers named d_* are device pointers, h_* host pointers. Tables are views: the
 *     library never frees or mutates caller memory (the reference's join partitions its
 *     inputs in place, src/join/join_provider.cuh:659-663; this one does not).
 *   - vj_stream_t is ABI-identical to cudaStream_t. Calls are stream-ordered on it; calls
 *     that return a host value (a count, a host histogram) synchronise that stream.
 *   - Rows per table are limited to 2^32 - 1.
 */
#ifndef VJ_H
#define VJ_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VJ_API __attribute__((visibility("default")))
#else
#define VJ_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *vj_stream_t;

enum vj_status {
    VJ_OK = 0,
    VJ_ERR_INVALID_ARGUMENT = 1,
    VJ_ERR_UNSUPPORTED = 2,
    VJ_ERR_CUDA = 3,
    VJ_ERR_OUT_OF_MEMORY = 4,
    VJ_ERR_CAPACITY = 5,  /* caller-provided output too small; the needed count is returned */
    VJ_ERR_DEVICE = 6,    /* a kernel reported an internal limit (bounded loop ran out) */
    VJ_ERR_BUDGET = 7     /* request exceeds the context's HBM budget */
};

/* Hash algorithm ids, in the order of the reference dispatcher (src/hash/hash.cu:515-541). */
enum vj_hash_algo {
    VJ_HASH_FNV = 0,
    VJ_HASH_CUSTOM_XOR = 1,
    VJ_HASH_CUSTOM_XOR_SHIFT = 2,
    VJ_HASH_CUSTOM_XOR_HW = 3,
    VJ_HASH_CUSTOM_MULT_XOR_SHIFT = 4,
    VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT = 5,
    VJ_HASH_CUSTOM_MULT_XOR_HW = 6,
    VJ_HASH_CUSTOM_MULT = 7,
    VJ_HASH_CUSTOM_MULT_SHIFT = 8,
    VJ_HASH_CUSTOM_MULT_HW = 9,
    VJ_HASH_CUSTOM_ADD = 10,
    VJ_HASH_CUSTOM_ADD_SHIFT = 11,
    VJ_HASH_CUSTOM_ADD_HW = 12,
    VJ_HASH_COUNT = 13
};

VJ_API int vj_version(void);
/* Device and page-locked host allocations the library has made in this process (workspaces,
 * library-owned results, staging buffers, result words). A diagnostic: a call that claims
 * to allocate nothing, such as vj_partition_noalloc, leaves it unchanged. */
VJ_API uint64_t vj_allocation_count(void);
VJ_API const char *vj_status_string(int status);
/* Copies the calling thread's last error message into buf (NUL-terminated); returns its length. */
VJ_API size_t vj_last_error(char *buf, size_t len);

/* Algorithm id for a reference algorithm name ("fnv", "custom_xor_hw", ...), or -1. The
 * reference silently launches nothing for an unknown name (src/hash/hash.cu:515-541). */
VJ_API int vj_hash_algo_id(const char *name);
VJ_API const char *vj_hash_algo_name(int algo);

/*
 * vj_hash -- hash_func (src/hash/hash.cu:507-557).
 * Element e occupies element_chunks chunks of chunk_bits/8 bytes starting at
 * d_elements + e * element_chunks * chunk_bits/8; chunks [chunk_offset, element_chunks) are
 * hashed. chunk_bits: 8, 32, 64 or 128 (HASH_CHUNK_BITS); hash_bits: 32 or 64 (HASH_BITS).
 * d_hashes receives n u32 or u64 values. Bit-exact with the reference kernels, including
 * the sign-extended char chunks of chunk_bits 8 and the *_shift variants' shift amounts
 * outside [0, hash_bits), which give 0 as the reference's compiled shifts do.
 * d_elements must be aligned to the chunk size. Asynchronous on stream.
 */
VJ_API int vj_hash(const void *d_elements, uint64_t n, int chunk_offset, int element_chunks, int chunk_bits, int hash_bits, int algo, void *d_hashes, vj_stream_t stream);

/* Library context: device, stream-ordered workspace, tuning cache and HBM budget. The
 * reference keeps the equivalent per-device state in DeviceConfig
 * (src/join/join_provider.cuh:124-220). A context may be used from one thread at a time. */
typedef struct vj_ctx vj_ctx;

/* memory_budget_bytes: upper bound on device memory the context allocates (workspace and
 * library-owned results); 0 = no bound beyond the device. */
VJ_API int vj_ctx_create(int device, uint64_t memory_budget_bytes, vj_ctx **out);
VJ_API int vj_ctx_destroy(vj_ctx *ctx);
/* Device memory currently held by the context (workspace + owned results), in bytes. */
VJ_API uint64_t vj_ctx_memory_in_use(const vj_ctx *ctx);
/* Frees the cached workspace (owned results stay valid). */
VJ_API int vj_ctx_trim(vj_ctx *ctx);

/*
 * Per-stage GPU times of the last vj_join / vj_build_probe / vj_join_host on a context with
 * profiling enabled -- the reference's JoinSummary / PartitionSummary / ProbeSummary
 * (src/join/join_provider.cuh:54-106, src/join/join_provider.cu:37-93). Events are
 * recorded on the join's stream between launches; unlike the reference's profiling
 * (join_provider.cu:148-157) nothing synchronises between kernels.
 */
typedef struct vj_profile {
    int32_t passes;             /* radix passes of the last join (0..2) */
    int32_t kernel_launches;    /* library kernels launched by the last join */
    int32_t radix_bits[2];
    uint32_t build_rows;        /* rows per shared-memory table */
    uint32_t probe_rows;        /* probe rows per work item */
    float ms_histogram[2];      /* histogram kernel of each pass */
    float ms_scatter[2];        /* scatter kernel of each pass */
    float ms_plan[2];           /* unit planning and the two scans of each pass */
    float ms_probe;             /* work-item planning + build/probe kernel */
    float ms_total;             /* first partition launch to the end of the probe */
    uint64_t rows[2];           /* |R|, |S| */
    uint64_t matches;
    int32_t tables;             /* VJ_TABLES_SHARED: where build tables lived */
    int32_t fallbacks;          /* always 0 (kept for layout compatibility) */
} vj_profile;

enum { VJ_TABLES_SHARED = 0, VJ_TABLES_L2 = 1 };

VJ_API int vj_ctx_set_profiling(vj_ctx *ctx, int enabled);
VJ_API int vj_ctx_last_profile(const vj_ctx *ctx, vj_profile *out);

/*
 * A columnar table view (db_table, src/base/types.hpp:128-266). keys: row-major rows of
 * key_words 32-bit words -- 1 for an int32 key, 2 for one u64 column, 2*c for c u64 key
 * columns (c <= 4). payloads: one payload_bytes (4 or 8) value per row -- the reference's
 * primary_keys column. A join output pair is (build payload, probe payload).
 */
typedef struct vj_table {
    const void *keys;
    const void *payloads;
    uint64_t rows;
    int32_t key_words;
    int32_t payload_bytes;
} vj_table;

/*
 * vj_partition -- one radix pass, partition_gpu (src/join/join_provider.cu:610-661).
 * Bucket of row i = (hash_i >> radix_shift) & (2^radix_bits - 1), where hash_i is
 * d_hashes_in[i] (u32/u64 by hash_bits) when given, else the hash_algo hash of the row's
 * key words (as hash_func with 32-bit chunks computes it). Rows are scattered to
 * d_keys_out / d_payloads_out (and their hashes to d_hashes_out when both hash arrays are
 * given) grouped by bucket in ascending bucket order; the order inside a bucket is
 * unspecified, as in the reference. radix_bits: 1..12.
 * Histogram and exclusive offsets (2^radix_bits u64 each) go to the device arrays and/or
 * the host arrays that are not NULL; host arrays make the call synchronous, as the
 * reference's copies back to the host do (join_provider.cu:645-646), and turn a kernel's
 * error flag into VJ_ERR_DEVICE. Without host arrays the call is asynchronous: a kernel
 * error then shows as UINT64_MAX in every histogram entry (the output is incomplete).
 */
VJ_API int vj_partition(vj_ctx *ctx, const vj_table *in, const void *d_hashes_in, int hash_bits, int hash_algo, void *d_keys_out, void *d_payloads_out, void *d_hashes_out, int radix_shift, int radix_bits,
                 uint64_t *d_histogram, uint64_t *d_offsets, uint64_t *h_histogram, uint64_t *h_offsets, vj_stream_t stream);

/*
 * vj_partition_noalloc -- vj_partition without a context, and without allocating anything.
 * It has no counterpart in the reference (whose partition_gpu allocates its buffers on every
 * call). It is meant for callers that cannot allocate device memory: an engine that has
 * handed all of HBM to its own buffer pool, so that cudaMalloc fails or would compete with
 * it, or one that keeps other streams busy and cannot let a cudaFree synchronise the device.
 *
 * Arguments, bucket rule, outputs and errors are those of vj_partition. The caller passes
 * every input and output; the working memory of the pass (per-unit bucket counts and
 * offsets, bucket bounds, an error flag) is one static device array of
 * VJ_NOALLOC_SCRATCH_BYTES that each GPU which loads the library holds until the process
 * exits. The call runs no cudaMalloc, cudaFree or other allocating routine.
 *   - radix_bits: 1..VJ_NOALLOC_MAX_RADIX_BITS; larger values return VJ_ERR_UNSUPPORTED
 *     before anything is launched.
 *   - It runs on the calling thread's current device. The first call on each device looks
 *     up the device address of the static array (cudaGetSymbolAddress) and keeps it; make
 *     that first call before any stream capture. CUDA loads modules lazily: the static array
 *     and the module's code take their device memory at that first call, so make it before
 *     the caller's pool reserves the device's memory (a call with rows = 0 is enough).
 *   - Errors of its kernels are reported as vj_partition reports them: VJ_ERR_DEVICE with
 *     host arrays, UINT64_MAX in every histogram entry without.
 *   - Every call on a device shares the one array, which keeps what the last call left in
 *     it; each call clears what must start at zero itself. Calls that overlap on the GPU
 *     (streams with no order between them, or threads without a lock) race on the array and
 *     give wrong results: put them on one stream or serialise them.
 */
#define VJ_NOALLOC_SCRATCH_BYTES (4u << 20)
#define VJ_NOALLOC_MAX_RADIX_BITS 10
VJ_API int vj_partition_noalloc(const vj_table *in, const void *d_hashes_in, int hash_bits, int hash_algo, void *d_keys_out, void *d_payloads_out, void *d_hashes_out, int radix_shift, int radix_bits,
                         uint64_t *d_histogram, uint64_t *d_offsets, uint64_t *h_histogram, uint64_t *h_offsets, vj_stream_t stream);

/*
 * vj_build_probe -- build_and_probe_gpu (src/join/join_provider.cu:669-847).
 * Builds a hash table over r and probes it with s; a match is a pair of rows with equal
 * hashes (when hash arrays are given) and equal key words. Writes up to `capacity` pairs
 * (r payload, s payload), each payload_bytes wide, to d_pairs in unspecified order and
 * the match count to *count. key_offset is accepted for signature parity (the reference
 * takes its slot from hash >> key_offset); the result does not depend on it.
 * Returns VJ_ERR_CAPACITY (with *count = needed) when capacity is too small.
 * Synchronises stream.
 */
VJ_API int vj_build_probe(vj_ctx *ctx, const vj_table *r, const void *d_r_hashes, const vj_table *s, const void *d_s_hashes, int hash_bits, int key_offset, void *d_pairs, uint64_t capacity, uint64_t *count,
                   vj_stream_t stream);

/* Join options (JoinConfig, src/join/join_provider.cuh:108-122). A zero-initialised struct
 * means "automatic": FNV-1a, 64-bit hash, passes, radix bits and table size from the tuner. */
/* flags: VJ_JOIN_FIXED_PASSES takes passes and radix_bits as given. Build tables are
 * shared-memory tables per build chunk of <= 2048 rows after up to two radix passes;
 * VJ_JOIN_SHARED_TABLES names that explicitly. VJ_JOIN_L2_TABLES (L2-resident tables per
 * partition after one pass) is no longer offered: it was slower than shared-memory tables
 * on every measured shape, and a join that asks for it returns VJ_ERR_UNSUPPORTED. */
/* VJ_JOIN_TEST_DEVICE_FLAG is for tests of error reporting: after the probe a kernel sets a
 * flag in the join's device error word, as a kernel whose bounded wait ran out does, and the
 * call returns VJ_ERR_DEVICE. VJ_JOIN_BATCH_LAUNCHES (vj_join_batch only) runs the batch as
 * its phases' separate kernel launches instead of the one fused, persistent launch (same
 * results; kept for comparison). */
enum { VJ_JOIN_FIXED_PASSES = 1, VJ_JOIN_SHARED_TABLES = 2, VJ_JOIN_L2_TABLES = 4, VJ_JOIN_TEST_DEVICE_FLAG = 1 << 16, VJ_JOIN_BATCH_LAUNCHES = 1 << 17 };
typedef struct vj_join_options {
    int32_t hash_algo;      /* VJ_HASH_*: the hash the partitions are cut from */
    int32_t hash_bits;      /* 32 or 64; 0 = 64 */
    int32_t flags;          /* VJ_JOIN_FIXED_PASSES: take passes and radix_bits as given */
    int32_t passes;         /* 0..2 radix passes (with VJ_JOIN_FIXED_PASSES) */
    int32_t radix_bits[2];  /* bits of pass 1 and pass 2 (with VJ_JOIN_FIXED_PASSES) */
    int32_t build_rows;     /* build rows per shared-memory table, rounded up to a power of
                               two and capped by shared memory; 0 = largest that fits */
    int32_t probe_rows;     /* probe rows per work item; 0 = automatic */
    int32_t probe_threads;  /* threads per probe block (64..1024, multiple of 32; one warp
                               fetches work and flushes pairs, the others build and probe);
                               0 = automatic (1024) */
    int32_t probe_sub_rows; /* unused (kept for layout compatibility) */
    int32_t table_load_pct; /* largest load of a build table in percent (50, 25 or 12: table
                               slots per build row 2, 4 or 8); 0 = automatic (12) */
    int32_t reserved[3];
} vj_join_options;

/* Join output. If pairs != NULL and capacity > 0 on entry, the caller owns the buffer (device
 * memory, capacity pairs); otherwise the library allocates it from the context (owned = 1)
 * and vj_result_free releases it. */
typedef struct vj_result {
    void *pairs;        /* count x (build payload, probe payload), payload_bytes each */
    uint64_t count;
    uint64_t capacity;
    int32_t owned;
    int32_t payload_bytes;
} vj_result;

/*
 * vj_join -- JoinProvider::join for device tables (src/join/join_provider.cuh:286-421):
 * hash -> radix partition (0-2 passes) -> per-partition shared-memory build/probe -> pairs.
 * The pairs are the multiset of (r payload, s payload) over rows with equal key words, in
 * unspecified order. r and s must have the same key_words and payload_bytes.
 * Synchronises stream (the count is returned on the host).
 */
VJ_API int vj_join(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, vj_result *result, vj_stream_t stream);

/*
 * vj_join_host -- the same join with HOST tables and a HOST output buffer: copies r and s
 * to the device, joins, and copies the pairs back (up to capacity pairs). Host memory that
 * is page-locked transfers at full link speed. A probe side of at least twice the build
 * side and 2^23 rows is pipelined: it is copied in chunks of about |R| rows (2 to 16), each
 * chunk is joined with the whole build side as soon as it has landed, and its pairs are
 * copied back while the next chunk is joined (copies in, joins and copies out overlap; the
 * pairs are the same, grouped by chunk). Returns when the pairs are in h_pairs. Returns
 * VJ_ERR_CAPACITY with *count = needed when capacity is too small; h_pairs then holds an
 * unspecified part of the pairs. With profiling on, the profile is that of the last chunk.
 */
VJ_API int vj_join_host(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, void *h_pairs, uint64_t capacity, uint64_t *count, vj_stream_t stream);

VJ_API int vj_result_free(vj_ctx *ctx, vj_result *result);

/*
 * Autotuner. The reference sweeps its tunables (bucket counts, vector sizes, kernel shapes)
 * from TOML grids in separate benchmark runs (src/benchmark/configuration.hpp:200-305).
 * vj_tune runs candidate plans of a join of r and s on this context -- the planner's
 * choice, the same with fuller tables (load <= 1/4, 1/2) and with 512-thread probe blocks,
 * two passes with the bits split both ways around the total that fills the shared-memory
 * tables (and one bit more or less), one pass; at most max_candidates (0 = 16) -- each a
 * full join into d_pairs (capacity
 * pairs), and keeps the fastest for the join's shape class (key words, payload bytes,
 * ceil(log2 |R|), ceil(log2 |S|), hash algorithm and width of `base`). Later vj_join calls
 * on this context with automatic options (NULL or all fields zero but the hash) of that
 * class use it, and so do vj_join_host, vj_join_batch (for the class of its largest join:
 * max_build_rows build rows, probe rows in the batch's ratio) and the slots of a server
 * the cache is shared with (vj_server_share_tuning). *best / *best_ms (optional) receive
 * the winner and its time.
 * vj_tune_save / vj_tune_load write / merge the context's cache as a text file.
 */
VJ_API int vj_tune(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *base, void *d_pairs, uint64_t capacity, int max_candidates, vj_join_options *best, float *best_ms,
                   vj_stream_t stream);
VJ_API int vj_tune_save(const vj_ctx *ctx, const char *path);
VJ_API int vj_tune_load(vj_ctx *ctx, const char *path);

/*
 * vj_join_batch -- many independent joins in one launch sequence. The reference runs one
 * JoinProvider::join per call; its nearest counterpart is the bucket-pair work list of a
 * single join (src/join/join_provider.cuh:717-795).
 * joins: 1..16384. Join j joins build rows [d_r_offsets[j], d_r_offsets[j+1]) of r with probe rows
 * [d_s_offsets[j], d_s_offsets[j+1]) of s (device arrays of joins + 1 uint64_t, starting
 * at 0, ending at the table's rows, non-decreasing). Its pairs (r payload, s payload) go to
 * d_pairs[d_pair_offsets[j] .. d_pair_offsets[j+1]) (pair_capacity pairs in all) and their
 * number to d_counts[j]; a count above the join's range means the pairs past the range
 * were dropped. max_build_rows: the largest join's build rows (plans the radix pass; 0 =
 * all of r). *d_status (device, optional) receives the kernels' flags: 0 = ok, 16 = an
 * offset was out of range or decreasing and was clamped (that join's results are then
 * unspecified), 64 = a grid-barrier wait of the fused launch ran out (a block could not
 * run: the results are unspecified). Asynchronous: no host synchronisation, and once the
 * context's workspace has grown to a batch of this shape, no allocation -- repeated calls
 * can be captured in a CUDA graph after one call outside the capture. The batch runs as
 * one persistent, cooperative kernel launch (plus memsets of its counters): the radix pass,
 * the build tables and the probes of all joins, phase after phase over the whole GPU
 * (probe_threads is ignored: its blocks are 1024 threads). Each join's pairs equal
 * vj_join's on the same rows.
 */
VJ_API int vj_join_batch(vj_ctx *ctx, const vj_table *r, const vj_table *s, uint32_t joins, const uint64_t *d_r_offsets, const uint64_t *d_s_offsets, uint64_t max_build_rows,
                         const vj_join_options *options, void *d_pairs, const uint64_t *d_pair_offsets, uint64_t pair_capacity, uint64_t *d_counts, uint32_t *d_status, vj_stream_t stream);

/*
 * Join server -- the serving form of the join: requests of different sizes arrive over
 * time, are admitted while the memory held by running joins stays within a budget, and
 * run concurrently (one context and stream per slot, whose partition buffers stay
 * resident between requests). The reference bounds memory and concurrency inside a single
 * join (DeviceConfig::reserve_memory, src/join/join_provider.cuh:138-150; its probe-thread
 * semaphore and stream pool, :453-480, :534-560); here the unit is a whole request.
 *   vj_server_create: `slots` concurrent joins (1..64) under memory_budget_bytes (0 = the
 *     device's free memory at creation).
 *   vj_server_submit: queue a join of DEVICE tables r and s; its pairs go to the caller's
 *     d_pairs (capacity pairs). Tables and output must stay valid until the request is
 *     waited for. A join whose estimated footprint exceeds the whole budget is refused
 *     with VJ_ERR_BUDGET. Admission is in arrival order, except that a request that fits
 *     may pass a head that does not (at most 8 times per head).
 *   vj_server_wait: block until the request is done (one waiter per request: a second
 *     thread waiting for the same id gets VJ_ERR_INVALID_ARGUMENT); its status is vj_join's (VJ_OK, or
 *     VJ_ERR_CAPACITY with count = pairs needed), times are seconds since the server
 *     started. Each request's result equals vj_join's on the same tables.
 *   vj_server_destroy: finishes every queued request, then frees the slots.
 */
typedef struct vj_server vj_server;
typedef struct vj_request_result {
    int32_t status;
    int32_t slot;       /* slot that ran it */
    uint64_t count;     /* pairs of the join */
    double submit_s;    /* submitted, started, finished: seconds since the server started */
    double start_s;
    double finish_s;
    int32_t passes;     /* the plan the join ran: radix passes, their bits, build rows per table */
    int32_t radix_bits[2];
    uint32_t build_rows;
} vj_request_result;
typedef struct vj_server_stats {
    uint64_t submitted;
    uint64_t completed;
    uint64_t peak_bytes;  /* largest sum of the bytes the slots held or had reserved */
    uint64_t budget;
    int32_t peak_running; /* most requests running at once */
    int32_t slots;
} vj_server_stats;
VJ_API int vj_server_create(int device, uint64_t memory_budget_bytes, int slots, vj_server **out);
VJ_API int vj_server_submit(vj_server *srv, const vj_table *r, const vj_table *s, const vj_join_options *options, void *d_pairs, uint64_t capacity, uint64_t *request_id);
VJ_API int vj_server_wait(vj_server *srv, uint64_t request_id, vj_request_result *out);
VJ_API int vj_server_stats_get(vj_server *srv, vj_server_stats *out);
/* Copies the tuning cache of ctx (vj_tune results, vj_tune_load entries) into every slot:
 * requests with automatic options then run the tuned plan of their shape class. Call it
 * while no request is queued or running (VJ_ERR_INVALID_ARGUMENT otherwise). */
VJ_API int vj_server_share_tuning(vj_server *srv, const vj_ctx *ctx);
VJ_API int vj_server_destroy(vj_server *srv);

/* Order-independent digest of a pair list: sum and xor of a 64-bit mix of each pair, the
 * same function the CPU oracle computes. For comparing full-size joins without sorting.
 * Synchronises stream. */
VJ_API int vj_pairs_digest(const void *d_pairs, uint64_t count, int payload_bytes, uint64_t *h_sum, uint64_t *h_xor, vj_stream_t stream);

/*
 * Seeded workload generator (replaces the reference's time-seeded curand generator,
 * src/benchmark/data_generator.cu:148-229). Build rows get unique keys (a bijection of the
 * row index; in [0, 2^31) for 4-byte keys) and payload = row id. Probe row j takes the key
 * of build row rng(j) % nr when (rng'(j) >> 32) < match_threshold, else a key no build row
 * has; payload = j. Same values as the CPU oracle's generator. Asynchronous on stream.
 */
VJ_API int vj_generate_join(uint64_t seed, int key_bytes, int payload_bytes, uint64_t nr, uint64_t ns, uint64_t match_threshold, void *d_r_keys, void *d_r_payloads, void *d_s_keys, void *d_s_payloads,
                     vj_stream_t stream);

/* Expected (count, digest sum, digest xor) of the join of vj_generate_join's tables, computed
 * on the device from the generator alone. Synchronises stream. */
VJ_API int vj_generate_join_expect(uint64_t seed, uint64_t nr, uint64_t ns, uint64_t match_threshold, uint64_t *count, uint64_t *h_sum, uint64_t *h_xor, vj_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* VJ_H */
