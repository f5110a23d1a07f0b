/*
 * vj_oracle.c -- CPU oracle for the hash -> radix partition -> build/probe join path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: tests, the smoke check and the
 * bench's CPU-baseline leg load it. No product code path calls it, and the GPU library
 * never falls back to it.
 *
 * It restates, in plain C, the algorithms of the reference (vgerber/vectorized-join):
 *   - the 13 hash kernels of src/hash/hash.cu:84-505 (FNV-1a and the "custom" family),
 *     evaluated with the same integer types the reference's CUDA code uses, including the
 *     sign-extended `char` chunks of HASH_CHUNK_BITS == 8 (src/base/types.hpp:15-16);
 *   - the radix partition of src/join/join_provider.cu:315-380 (histogram of
 *     (hash >> shift) & (bins-1), exclusive prefix, scatter);
 *   - the chained hash table build/probe of src/join/join_provider.cu:382-442 and
 *     :536-591 (slot = (hash >> key_offset) % slots, 1-based links, match = equal hash
 *     and every key word equal), emitting (build payload, probe payload) pairs like
 *     copy_probe_results_kernel (src/join/join_provider.cu:593-608);
 *   - the join-result contract of JoinProvider::join_cpu (src/join/join_provider.cuh:241-284):
 *     the multiset of pairs of rows whose key columns are all equal.
 *
 * The shift amounts of the *_shift variants can leave [0, hash bits) (get_max_shift(),
 * src/hash/hash.cu:60-62, is not the intended bound). C leaves such shifts undefined; the
 * reference's device code compiles them to PTX shl, whose amount is unsigned and clamps
 * at the register width, so the result is 0. The oracle computes exactly that and raises
 * a flag per element so tests can tell which outputs rest on it.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define VJO_API __attribute__((visibility("default")))

/* Algorithm ids follow the order of the reference dispatcher, src/hash/hash.cu:515-541. */
enum {
    ALG_FNV = 0,
    ALG_XOR = 1,
    ALG_XOR_SHIFT = 2,
    ALG_XOR_HW = 3,
    ALG_MULT_XOR_SHIFT = 4,
    ALG_N_MULT_XOR_SHIFT = 5,
    ALG_MULT_XOR_HW = 6,
    ALG_MULT = 7,
    ALG_MULT_SHIFT = 8,
    ALG_MULT_HW = 9,
    ALG_ADD = 10,
    ALG_ADD_SHIFT = 11,
    ALG_ADD_HW = 12,
    ALG_COUNT = 13
};

/* ---------------------------------------------------------------- bit helpers */

static uint32_t rev32(uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; i < 32; i++) {
        r = (r << 1) | (v & 1u);
        v >>= 1;
    }
    return r;
}

static uint64_t rev64(uint64_t v) {
    return ((uint64_t)rev32((uint32_t)v) << 32) | rev32((uint32_t)(v >> 32));
}

/* __funnelshift_l(v, v, s): rotate left by (s & 31)  (hash.cu:72-74). */
static uint32_t rotl32(uint32_t v, uint32_t s) {
    s &= 31u;
    return s ? (v << s) | (v >> (32u - s)) : v;
}

/* get_max_shift() of hash.cu:60-62 evaluated with the reference's integer types:
 * (unsigned short)(sizeof(hash_t) - sizeof(chunk_t) * 8) + 1. */
static int32_t max_shift(int hash_bits, int chunk_bits) {
    uint64_t hb = (uint64_t)(hash_bits / 8);
    uint64_t cb = (uint64_t)(chunk_bits / 8);
    uint16_t t = (uint16_t)(hb - cb * 8u); /* size_t arithmetic wraps, then truncates */
    return (int32_t)(uint16_t)((int32_t)t + 1);
}

typedef struct {
    int hb;          /* hash bits: 32 or 64 */
    uint64_t hm;     /* hash mask */
    int byte_mode;   /* chunk_bits == 8: chunk_t is (signed) char */
    int32_t ms;      /* get_max_shift() */
    int ub;          /* set when a shift amount left [0, hb) */
} hctx;

/* value << amount as the reference's device code computes it (PTX shl clamps). */
static uint64_t shl_dev(hctx *c, uint64_t v, int32_t amount) {
    if ((uint32_t)amount >= (uint32_t)c->hb) {
        c->ub = 1;
        return 0;
    }
    return (v << amount) & c->hm;
}

/* `hash_offset = (hash_offset + chunk) % get_max_shift();` for the add/xor/mult *_shift
 * kernels (hash.cu:155, :159, :242, :246, :339, :343). In byte mode both operands are
 * int (signed remainder); for 32-bit lanes the sum is unsigned int. */
static int16_t shift_offset_lane(hctx *c, int16_t off, int64_t lane) {
    if (c->byte_mode) {
        int32_t sum = (int32_t)off + (int32_t)lane;
        return (int16_t)(sum % c->ms);
    }
    uint32_t sum = (uint32_t)(int32_t)off + (uint32_t)lane;
    return (int16_t)(uint16_t)(sum % (uint32_t)c->ms);
}

/* The same statement inside mult_xor_shift() (hash.cu:398-406), where chunk is hash_t. */
static int16_t shift_offset_hash(hctx *c, int16_t off, uint64_t ch) {
    if (c->hb == 64) {
        uint64_t sum = (uint64_t)(int64_t)off + ch;
        return (int16_t)(uint16_t)(sum % (uint64_t)c->ms);
    }
    uint32_t sum = (uint32_t)(int32_t)off + (uint32_t)ch;
    return (int16_t)(uint16_t)(sum % (uint32_t)c->ms);
}

static uint64_t reverse_h(hctx *c, uint64_t h) {
    return c->hb == 64 ? rev64(h) : (uint64_t)rev32((uint32_t)h);
}

typedef struct {
    uint64_t h;
    int32_t shift_i;    /* int shift (add_hw, mult_hw) */
    uint32_t shift_u;   /* uint32_t shift (xor_hw) */
    int16_t off;        /* short hash_offset */
    int16_t op;         /* short operation */
} hstate;

static void init_state(int algo, hctx *c, hstate *s) {
    memset(s, 0, sizeof(*s));
    switch (algo) {
    case ALG_FNV:
        s->h = c->hb == 64 ? 14695981039346656037ull : 2166136261ull; /* hash.cu:52-58 */
        break;
    case ALG_MULT:
    case ALG_MULT_SHIFT:
    case ALG_MULT_HW:
        s->h = 1; /* hash.cu:305, :332, :365 */
        break;
    default:
        s->h = 0;
    }
}

/* One lane of one chunk. `lane` is the chunk value widened the way C converts it:
 * a sign-extended char in byte mode, a zero-extended 32-bit word otherwise. */
static void feed_lane(int algo, hctx *c, hstate *s, int64_t lane) {
    const uint64_t hm = c->hm;
    const uint64_t ch = (uint64_t)lane & hm;   /* (hash_t)chunk */
    const uint32_t u32 = (uint32_t)lane;       /* (unsigned int)chunk */
    const uint64_t prime = c->hb == 64 ? 1099511628211ull : 16777619ull; /* hash.cu:44-50 */
    switch (algo) {
    case ALG_FNV: /* hash.cu:96-111 */
        s->h = ((s->h ^ ch) * prime) & hm;
        break;
    case ALG_ADD: /* hash.cu:128-138 */
        s->h = (s->h + ch) & hm;
        break;
    case ALG_ADD_SHIFT: /* hash.cu:155-170 */
        s->off = shift_offset_lane(c, s->off, lane);
        s->h = (s->h + shl_dev(c, ch, s->off)) & hm;
        break;
    case ALG_ADD_HW: /* hash.cu:187-197 (reverse happens per chunk, see end_chunk) */
        s->h = (s->h + (uint64_t)rotl32(u32, (uint32_t)s->shift_i)) & hm;
        s->shift_i++;
        break;
    case ALG_XOR: /* hash.cu:215-225 */
        s->h ^= ch;
        break;
    case ALG_XOR_SHIFT: /* hash.cu:242-257 */
        s->off = shift_offset_lane(c, s->off, lane);
        s->h ^= shl_dev(c, ch, s->off);
        break;
    case ALG_XOR_HW: /* hash.cu:274-294 */
        s->shift_u += u32;
        s->h ^= (uint64_t)rotl32(u32, s->shift_u);
        s->h = reverse_h(c, s->h);
        break;
    case ALG_MULT: /* hash.cu:311-321 */
        s->h = (1u + s->h * ((ch + 1u) & hm)) & hm;
        break;
    case ALG_MULT_SHIFT: /* hash.cu:339-354: 1 + ((hash * (chunk + 1)) << offset) */
        s->off = shift_offset_lane(c, s->off, lane);
        s->h = (1u + shl_dev(c, (s->h * ((ch + 1u) & hm)) & hm, s->off)) & hm;
        break;
    case ALG_MULT_HW: /* hash.cu:371-391 */
        s->shift_i = (int32_t)((uint32_t)s->shift_i + u32);
        s->h = (1u + s->h * (((uint64_t)rotl32(u32, (uint32_t)s->shift_i) + 1u) & hm)) & hm;
        s->h = reverse_h(c, s->h);
        break;
    case ALG_MULT_XOR_SHIFT:
    case ALG_N_MULT_XOR_SHIFT: /* mult_xor_shift(), hash.cu:398-406 */
        s->off = shift_offset_hash(c, s->off, ch);
        if (s->op & 1) {
            s->h = (1u + s->h * shl_dev(c, (ch + 1u) & hm, s->off)) & hm;
        } else {
            s->h = s->h ^ shl_dev(c, ch, s->off);
        }
        s->op = (int16_t)(s->op + 1);
        break;
    case ALG_MULT_XOR_HW: /* mult_xor_hw(), hash.cu:408-417 */
        if (s->op & 1) {
            s->h = (1u + s->h * (uint64_t)rotl32((uint32_t)((ch + 1u) & hm), (uint32_t)(int32_t)s->off)) & hm;
        } else {
            s->h = s->h ^ (uint64_t)rotl32((uint32_t)ch, (uint32_t)(int32_t)s->off);
        }
        s->op = (int16_t)(s->op + 1);
        s->off = (int16_t)(uint16_t)((uint64_t)(int64_t)s->off + ch);
        s->h = reverse_h(c, s->h);
        break;
    }
}

static void end_chunk(int algo, hctx *c, hstate *s) {
    if (algo == ALG_ADD_HW) {
        s->h = reverse_h(c, s->h); /* hash.cu:199, once per chunk */
    }
}

/* Hash one element: chunks [chunk_offset, element_chunks) of the element that starts at
 * `elem` (hash.cu:90-115). Returns the hash; *ub is set if a shift left [0, hash bits). */
VJO_API uint64_t vjo_hash_element(const uint8_t *elem, int chunk_offset, int element_chunks, int chunk_bits, int hash_bits, int algo, int *ub) {
    hctx c;
    c.hb = hash_bits;
    c.hm = hash_bits == 64 ? ~0ull : 0xffffffffull;
    c.byte_mode = chunk_bits == 8;
    c.ms = max_shift(hash_bits, chunk_bits);
    c.ub = 0;
    hstate s;
    init_state(algo, &c, &s);
    const int chunk_bytes = chunk_bits / 8;
    const int rounds = algo == ALG_N_MULT_XOR_SHIFT ? 2 : 1; /* hash.cu:526 passes rounds = 2 */
    for (int round = 0; round < rounds; round++) {
        for (int ci = chunk_offset; ci < element_chunks; ci++) {
            const uint8_t *chunk = elem + (size_t)ci * chunk_bytes;
            if (c.byte_mode) {
                feed_lane(algo, &c, &s, (int64_t)(int8_t)chunk[0]);
            } else {
                for (int l = 0; l < chunk_bits / 32; l++) {
                    uint32_t w;
                    memcpy(&w, chunk + 4 * l, 4);
                    feed_lane(algo, &c, &s, (int64_t)(uint64_t)w);
                }
            }
            end_chunk(algo, &c, &s);
        }
    }
    if (ub) {
        *ub = c.ub;
    }
    return s.h & c.hm;
}

/* hash_func() over a whole buffer (hash.cu:507-557): element e starts at byte
 * e * element_chunks * chunk_bytes. Output is u32 or u64 per element by hash_bits.
 * ub_flags (optional) receives one byte per element. */
VJO_API void vjo_hash(const void *elements, uint64_t n, int chunk_offset, int element_chunks, int chunk_bits, int hash_bits, int algo, void *out, uint8_t *ub_flags) {
    const uint8_t *base = (const uint8_t *)elements;
    const size_t stride = (size_t)element_chunks * (size_t)(chunk_bits / 8);
    for (uint64_t e = 0; e < n; e++) {
        int ub = 0;
        uint64_t h = vjo_hash_element(base + e * stride, chunk_offset, element_chunks, chunk_bits, hash_bits, algo, &ub);
        if (hash_bits == 64) {
            ((uint64_t *)out)[e] = h;
        } else {
            ((uint32_t *)out)[e] = (uint32_t)h;
        }
        if (ub_flags) {
            ub_flags[e] = (uint8_t)ub;
        }
    }
}

/* ---------------------------------------------------------------- partition */

/* One radix pass like partition_gpu (join_provider.cu:610-661): histogram of
 * (hash >> shift) & (bins - 1), exclusive prefix into offsets, and a scatter of row
 * indices. The reference's scatter order inside a bucket depends on atomics; this one is
 * stable (row order), which is one of the orders the reference can produce. */
VJO_API void vjo_partition(const void *hashes, int hash_bits, uint64_t n, int radix_shift, int radix_bits, uint64_t *histogram, uint64_t *offsets, uint64_t *perm) {
    const uint64_t bins = 1ull << radix_bits;
    memset(histogram, 0, bins * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) {
        uint64_t h = hash_bits == 64 ? ((const uint64_t *)hashes)[i] : ((const uint32_t *)hashes)[i];
        histogram[(h >> radix_shift) & (bins - 1)]++;
    }
    uint64_t run = 0;
    for (uint64_t b = 0; b < bins; b++) {
        offsets[b] = run;
        run += histogram[b];
    }
    if (!perm) {
        return;
    }
    uint64_t *cursor = (uint64_t *)malloc(bins * sizeof(uint64_t));
    memcpy(cursor, offsets, bins * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) {
        uint64_t h = hash_bits == 64 ? ((const uint64_t *)hashes)[i] : ((const uint32_t *)hashes)[i];
        perm[cursor[(h >> radix_shift) & (bins - 1)]++] = i;
    }
    free(cursor);
}

/* ---------------------------------------------------------------- join */

/* Order-independent digest of one output pair. The GPU library computes the same
 * function over its output so full-size joins can be compared without sorting. */
static inline uint64_t fmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

VJO_API uint64_t vjo_pair_digest(uint64_t r_payload, uint64_t s_payload) {
    return fmix64(r_payload ^ fmix64(s_payload + 0x9e3779b97f4a7c15ull));
}

typedef struct {
    /* inputs */
    const uint32_t *r_keys, *s_keys; /* rows of kw 32-bit words */
    const uint64_t *r_pay, *s_pay;
    uint64_t nr, ns;
    int kw;
    int hash_bits, algo, radix_bits;
    const uint64_t *r_hash, *s_hash; /* per-row hash */
    const uint64_t *r_perm, *s_perm; /* rows grouped by bucket */
    const uint64_t *r_off, *s_off;   /* bucket offsets, bins + 1 entries */
    uint64_t bins;
    /* per-thread work */
    uint64_t bucket_begin, bucket_end;
    uint64_t *pairs;   /* 2 per match, may be NULL */
    uint64_t cap;
    uint64_t count;
    uint64_t digest_sum, digest_xor;
} join_task;

static int keys_equal(const uint32_t *a, const uint32_t *b, int kw) {
    for (int i = 0; i < kw; i++) {
        if (a[i] != b[i]) {
            return 0;
        }
    }
    return 1;
}

/* Chained table over one bucket of R, probed by the same bucket of S
 * (join_provider.cu:382-399 build, :401-442 probe; load factor 0.25 as in the shipped
 * TOML profiles, slots = max(1, load * n) as ProbeConfig::get_table_slots, cu:238-240). */
static void *join_worker(void *arg) {
    join_task *t = (join_task *)arg;
    const int kw = t->kw;
    uint32_t *slots = NULL;
    uint32_t *links = NULL;
    uint64_t slots_cap = 0, links_cap = 0;
    for (uint64_t b = t->bucket_begin; b < t->bucket_end; b++) {
        const uint64_t r0 = t->r_off[b], r1 = t->r_off[b + 1];
        const uint64_t s0 = t->s_off[b], s1 = t->s_off[b + 1];
        const uint64_t nrb = r1 - r0;
        if (nrb == 0 || s1 == s0) {
            continue;
        }
        uint64_t nslots = (uint64_t)(0.25f * (float)nrb);
        if (nslots < 1) {
            nslots = 1;
        }
        if (nslots > slots_cap) {
            free(slots);
            slots = (uint32_t *)malloc(nslots * sizeof(uint32_t));
            slots_cap = nslots;
        }
        if (nrb > links_cap) {
            free(links);
            links = (uint32_t *)malloc(nrb * sizeof(uint32_t));
            links_cap = nrb;
        }
        memset(slots, 0, nslots * sizeof(uint32_t));
        const int key_offset = t->radix_bits;
        for (uint64_t i = 0; i < nrb; i++) {
            uint64_t row = t->r_perm[r0 + i];
            uint64_t slot = (t->r_hash[row] >> key_offset) % nslots;
            links[i] = slots[slot]; /* atomicExch(&slot, i + 1) in serial order */
            slots[slot] = (uint32_t)(i + 1);
        }
        for (uint64_t j = s0; j < s1; j++) {
            uint64_t srow = t->s_perm[j];
            uint64_t sh = t->s_hash[srow];
            uint32_t e = slots[(sh >> key_offset) % nslots];
            const uint32_t *sk = t->s_keys + srow * (uint64_t)kw;
            while (e) {
                e--;
                uint64_t rrow = t->r_perm[r0 + e];
                if (t->r_hash[rrow] == sh && keys_equal(t->r_keys + rrow * (uint64_t)kw, sk, kw)) {
                    uint64_t rp = t->r_pay[rrow], sp = t->s_pay[srow];
                    if (t->pairs && t->count < t->cap) {
                        t->pairs[2 * t->count] = rp;
                        t->pairs[2 * t->count + 1] = sp;
                    }
                    uint64_t d = vjo_pair_digest(rp, sp);
                    t->digest_sum += d;
                    t->digest_xor ^= d;
                    t->count++;
                }
                e = links[e];
            }
        }
    }
    free(slots);
    free(links);
    return NULL;
}

static int cmp_pair(const void *a, const void *b) {
    const uint64_t *x = (const uint64_t *)a, *y = (const uint64_t *)b;
    if (x[0] != y[0]) {
        return x[0] < y[0] ? -1 : 1;
    }
    if (x[1] != y[1]) {
        return x[1] < y[1] ? -1 : 1;
    }
    return 0;
}

typedef struct {
    const uint32_t *keys;
    uint64_t begin, end;
    int kw, hash_bits, algo;
    uint64_t *hash;
} hash_task;

static void *hash_worker(void *arg) {
    hash_task *t = (hash_task *)arg;
    for (uint64_t i = t->begin; i < t->end; i++) {
        /* the key row is hashed as 32-bit lanes (chunk_bits 32), as JoinProvider::hash_table
         * feeds column_values to hash_func (join_provider.cuh:926-931) */
        t->hash[i] = vjo_hash_element((const uint8_t *)(t->keys + i * (uint64_t)t->kw), 0, t->kw, 32, t->hash_bits, t->algo, NULL);
    }
    return NULL;
}

/* Multiset equi-join of R and S (the result contract of join_cpu, join_provider.cuh:241-284)
 * computed with the reference's hash -> radix partition -> chained-table probe. Keys are
 * rows of kw 32-bit words, payloads are u64. If pairs != NULL and cap >= count, the pairs
 * (r_payload, s_payload) are written sorted. Returns the match count; digests receive the
 * sum and xor of vjo_pair_digest over all pairs. threads <= 0 means 1. */
VJO_API uint64_t vjo_join(const uint32_t *r_keys, const uint64_t *r_pay, uint64_t nr, const uint32_t *s_keys, const uint64_t *s_pay, uint64_t ns, int kw, int hash_bits, int algo, int radix_bits,
                          int threads, uint64_t *pairs, uint64_t cap, uint64_t *digest_sum, uint64_t *digest_xor) {
    if (threads <= 0) {
        threads = 1;
    }
    if (threads > 256) {
        threads = 256;
    }
    const uint64_t bins = 1ull << radix_bits;
    uint64_t *r_hash = (uint64_t *)malloc((nr ? nr : 1) * sizeof(uint64_t));
    uint64_t *s_hash = (uint64_t *)malloc((ns ? ns : 1) * sizeof(uint64_t));
    pthread_t tid[256];
    hash_task ht[256];
    for (int side = 0; side < 2; side++) {
        const uint32_t *keys = side ? s_keys : r_keys;
        uint64_t n = side ? ns : nr;
        uint64_t *hv = side ? s_hash : r_hash;
        for (int t = 0; t < threads; t++) {
            ht[t].keys = keys;
            ht[t].begin = n * (uint64_t)t / (uint64_t)threads;
            ht[t].end = n * (uint64_t)(t + 1) / (uint64_t)threads;
            ht[t].kw = kw;
            ht[t].hash_bits = hash_bits;
            ht[t].algo = algo;
            ht[t].hash = hv;
            pthread_create(&tid[t], NULL, hash_worker, &ht[t]);
        }
        for (int t = 0; t < threads; t++) {
            pthread_join(tid[t], NULL);
        }
    }
    uint64_t *r_perm = (uint64_t *)malloc((nr ? nr : 1) * sizeof(uint64_t));
    uint64_t *s_perm = (uint64_t *)malloc((ns ? ns : 1) * sizeof(uint64_t));
    uint64_t *r_off = (uint64_t *)malloc((bins + 1) * sizeof(uint64_t));
    uint64_t *s_off = (uint64_t *)malloc((bins + 1) * sizeof(uint64_t));
    uint64_t *hist = (uint64_t *)malloc(bins * sizeof(uint64_t));
    vjo_partition(r_hash, 64, nr, 0, radix_bits, hist, r_off, r_perm);
    r_off[bins] = nr;
    vjo_partition(s_hash, 64, ns, 0, radix_bits, hist, s_off, s_perm);
    s_off[bins] = ns;
    free(hist);

    join_task jt[256];
    uint64_t total = 0, dsum = 0, dxor = 0;
    for (int t = 0; t < threads; t++) {
        memset(&jt[t], 0, sizeof(jt[t]));
        jt[t].r_keys = r_keys;
        jt[t].s_keys = s_keys;
        jt[t].r_pay = r_pay;
        jt[t].s_pay = s_pay;
        jt[t].nr = nr;
        jt[t].ns = ns;
        jt[t].kw = kw;
        jt[t].hash_bits = hash_bits;
        jt[t].algo = algo;
        jt[t].radix_bits = radix_bits;
        jt[t].r_hash = r_hash;
        jt[t].s_hash = s_hash;
        jt[t].r_perm = r_perm;
        jt[t].s_perm = s_perm;
        jt[t].r_off = r_off;
        jt[t].s_off = s_off;
        jt[t].bins = bins;
        jt[t].bucket_begin = bins * (uint64_t)t / (uint64_t)threads;
        jt[t].bucket_end = bins * (uint64_t)(t + 1) / (uint64_t)threads;
        jt[t].pairs = NULL;
        pthread_create(&tid[t], NULL, join_worker, &jt[t]);
    }
    for (int t = 0; t < threads; t++) {
        pthread_join(tid[t], NULL);
        total += jt[t].count;
        dsum += jt[t].digest_sum;
        dxor ^= jt[t].digest_xor;
    }
    if (pairs && cap >= total && total > 0) {
        /* second sweep writes the pairs into per-thread slices, then sorts */
        uint64_t base = 0;
        for (int t = 0; t < threads; t++) {
            uint64_t c = jt[t].count;
            jt[t].pairs = pairs + 2 * base;
            jt[t].cap = c;
            jt[t].count = 0;
            jt[t].digest_sum = 0;
            jt[t].digest_xor = 0;
            base += c;
            pthread_create(&tid[t], NULL, join_worker, &jt[t]);
        }
        for (int t = 0; t < threads; t++) {
            pthread_join(tid[t], NULL);
        }
        qsort(pairs, total, 2 * sizeof(uint64_t), cmp_pair);
    }
    free(r_hash);
    free(s_hash);
    free(r_perm);
    free(s_perm);
    free(r_off);
    free(s_off);
    if (digest_sum) {
        *digest_sum = dsum;
    }
    if (digest_xor) {
        *digest_xor = dxor;
    }
    return total;
}

/* Nested-loop join over the same inputs: the literal join_cpu algorithm
 * (join_provider.cuh:249-282), for small cases. Pairs come out in (s, r) loop order. */
VJO_API uint64_t vjo_join_nested(const uint32_t *r_keys, const uint64_t *r_pay, uint64_t nr, const uint32_t *s_keys, const uint64_t *s_pay, uint64_t ns, int kw, uint64_t *pairs, uint64_t cap) {
    uint64_t m = 0;
    for (uint64_t s = 0; s < ns; s++) {
        for (uint64_t r = 0; r < nr; r++) {
            if (keys_equal(r_keys + r * (uint64_t)kw, s_keys + s * (uint64_t)kw, kw)) {
                if (pairs && m < cap) {
                    pairs[2 * m] = r_pay[r];
                    pairs[2 * m + 1] = s_pay[s];
                }
                m++;
            }
        }
    }
    return m;
}

VJO_API void vjo_sort_pairs(uint64_t *pairs, uint64_t count) {
    qsort(pairs, count, 2 * sizeof(uint64_t), cmp_pair);
}

/* ---------------------------------------------------------------- workload generator */
/*
 * Seeded counter-based inputs, identical to the GPU generator of the library
 * (csrc/vj_gen.cu): every value is a pure function of (seed, row), so the CPU and the GPU
 * produce the same tables without copying them. The reference seeds curand with
 * time(NULL) (src/benchmark/data_generator.cu:134, :169); these generators replace it with
 * reproducible draws of the shapes the benchmark configurations name.
 */

static inline uint64_t gen_stream(uint64_t seed, uint64_t tag) {
    return fmix64(seed * 0xd1b54a32d192ed03ull + tag * 0xaef17502108ef2d9ull + 0x243f6a8885a308d3ull);
}

VJO_API uint64_t vjo_rng(uint64_t seed, uint64_t tag, uint64_t i) {
    return fmix64(gen_stream(seed, tag) + (i + 1) * 0x9e3779b97f4a7c15ull);
}

/* unique 64-bit key of logical row i: a bijection of i */
VJO_API uint64_t vjo_ukey64(uint64_t seed, uint64_t i) {
    return fmix64(i + gen_stream(seed, 100));
}

/* unique key in [0, 2^31) of logical row i (i < 2^31): a bijection on 31 bits */
VJO_API uint32_t vjo_ukey31(uint64_t seed, uint64_t i) {
    const uint32_t m = 0x7fffffffu;
    uint32_t x = (uint32_t)((i + gen_stream(seed, 101)) & m);
    x = (x * 0x6b43a9b5u + 0x1234567u) & m;
    x ^= x >> 16;
    x = (x * 0x2c1b3c6du + 0x7654321u) & m;
    x ^= x >> 13;
    x = (x * 0x297a2d39u) & m;
    x ^= x >> 16;
    return x;
}

/* Miss keys are unique keys of logical rows at or above this index, so they never equal a
 * build key (build rows use logical rows [0, |R|)). */
#define VJO_MISS_BASE64 (1ull << 62)

/*
 * Generate a build table R (unique keys, payload = row id) and a probe table S whose row j
 * takes, with probability match_thr / 2^32, the key of build row rng % |R| and otherwise a
 * unique miss key. key_bytes is 4 (keys in [0, 2^31)) or 8. Payloads are u64 here; the
 * tests narrow them where the workload is int32. r_of_s (optional) receives the matched
 * build row of each probe row or UINT64_MAX. Returns the number of matching probe rows.
 */
VJO_API uint64_t vjo_gen_join(uint64_t seed, int key_bytes, uint64_t nr, uint64_t ns, uint64_t match_thr, void *r_keys, uint64_t *r_pay, void *s_keys, uint64_t *s_pay, uint64_t *r_of_s) {
    for (uint64_t i = 0; i < nr; i++) {
        if (key_bytes == 8) {
            ((uint64_t *)r_keys)[i] = vjo_ukey64(seed, i);
        } else {
            ((uint32_t *)r_keys)[i] = vjo_ukey31(seed, i);
        }
        if (r_pay) {
            r_pay[i] = i;
        }
    }
    uint64_t matches = 0;
    for (uint64_t j = 0; j < ns; j++) {
        uint64_t coin = vjo_rng(seed, 1, j) >> 32;
        uint64_t row;
        int hit = nr > 0 && coin < match_thr;
        if (hit) {
            row = vjo_rng(seed, 2, j) % nr;
        } else {
            row = VJO_MISS_BASE64 + j;
        }
        if (key_bytes == 8) {
            ((uint64_t *)s_keys)[j] = vjo_ukey64(seed, row);
        } else {
            ((uint32_t *)s_keys)[j] = vjo_ukey31(seed, hit ? row : (uint64_t)nr + j);
        }
        if (s_pay) {
            s_pay[j] = j;
        }
        if (r_of_s) {
            r_of_s[j] = hit ? row : UINT64_MAX;
        }
        matches += (uint64_t)hit;
    }
    return matches;
}

/* Expected (count, digest sum, digest xor) of the join of the tables vjo_gen_join makes,
 * from the generator alone (build keys are unique, so each hit pairs with one build row). */
VJO_API uint64_t vjo_gen_join_expect(uint64_t seed, uint64_t nr, uint64_t ns, uint64_t match_thr, uint64_t *digest_sum, uint64_t *digest_xor) {
    uint64_t m = 0, ds = 0, dx = 0;
    for (uint64_t j = 0; j < ns; j++) {
        uint64_t coin = vjo_rng(seed, 1, j) >> 32;
        if (nr > 0 && coin < match_thr) {
            uint64_t row = vjo_rng(seed, 2, j) % nr;
            uint64_t d = vjo_pair_digest(row, j);
            ds += d;
            dx ^= d;
            m++;
        }
    }
    if (digest_sum) {
        *digest_sum = ds;
    }
    if (digest_xor) {
        *digest_xor = dx;
    }
    return m;
}
