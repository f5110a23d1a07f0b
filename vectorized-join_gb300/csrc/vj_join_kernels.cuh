// vj_join_kernels.cuh -- radix partition and build/probe kernels of the join path.
//
// Data layout (HBM). Caller tables are columnar: a key array of rows of KW 32-bit words, a
// payload array of PB-byte values and, for the reference-compatible entry points, a hash
// array. The partition passes of a join write row-contiguous buffers (one "row" = key,
// payload[, hash], Layout::STRIDE bytes), so that each bucket run of a tile is one
// contiguous burst and one bulk copy fetches a chunk of rows. Nothing else is
// materialised per row: the partitioning hash is recomputed from the key in every kernel
// (a few integer ops per row).
//
// A pass over a set of "segments" (contiguous row ranges, e.g. the partitions of the
// previous pass) runs two kernels (see "partition kernels" below): a histogram that counts
// units of rows per bucket and writes the partition bounds, and a persistent scatter that
// finds each unit's write cursors by decoupled look-back over the units' counts, sorts
// tiles by bucket in shared memory and writes bucket runs as contiguous bursts.
// The probe stage plans (partition, build chunk, probe chunk) work items and runs a
// persistent kernel in which one warp fetches items, copies their build rows in and
// flushes their pairs out, while the other warps build shared-memory tables and probe
// (see "probe kernel").
#pragma once

#include "vj_internal.cuh"

namespace vj {

constexpr int MAX_RADIX_BITS = 12;
constexpr int PART_THREADS = 512;
constexpr int PLAN_THREADS = 1024;

struct HashSpec {
    int algo;       // VJ_HASH_* when the hash is recomputed from the key
    int hash_bits;  // 32 or 64
    int mix;        // 1: extract bits from mix_hash(hash), 0: from the raw hash
};

constexpr int round_up(int x, int a) { return (x + a - 1) / a * a; }

// Row-contiguous layout of a partition buffer row.
template <int KW, int PB, int HS>
struct Layout {
    static constexpr int KB = KW * 4;
    static constexpr int PAY_OFF = round_up(KB, PB);
    static constexpr int HASH_OFF = HS ? round_up(PAY_OFF + PB, HS) : PAY_OFF + PB;
    static constexpr int STRIDE = round_up(HASH_OFF + HS, 8);
};

struct Side {
    // columnar input (a caller's table)
    const void *keys_in;
    const void *pay_in;
    const void *hash_in;   // HS != 0 only
    // row-contiguous input (the previous pass's output)
    const void *rows_in;
    // row-contiguous output (a join's partition buffer) ...
    void *rows_out;
    // ... or columnar output (vj_partition writes the caller's swap columns)
    void *keys_out;
    void *pay_out;
    void *hash_out;        // HS != 0 only (may be null: hashes not moved)
    uint32_t rows;
    // the next pass's bucket of every output row (u16 at the row's output position), written
    // by a first pass whose second pass then counts these instead of re-reading the rows
    uint16_t *bid_out;
    const uint16_t *bid_in;
};

struct PassParams {
    Side side[2];
    int nsides;
    int Q;                       // segments per side (G = nsides * Q)
    const uint32_t *seg_begin;   // [G], null: one segment = the whole side
    const uint32_t *seg_end;
    int shift;                   // bucket = (hash >> shift) & (2^bits - 1)
    int bits;
    HashSpec hs;
    int next_shift, next_bits;   // bucket of the next pass (bid_out)
    // Units: segment g's rows are cut into units of `target` rows (its last one shorter, at
    // least one unit per segment); units [first[g], first[g + 1]) belong to segment g. The
    // last units of the pass are cut in four (split_plan): units from `split_from` on are
    // quarters of the units they replace. The plan (target, first[0..G], split_from) is
    // `plan` on the device or, when plan is null, hplan (G <= 2, planned on the host).
    const uint32_t *plan;
    uint32_t hplan[5];
    int max_units;
    uint32_t min_unit_rows;
    uint32_t split;              // units to cut in four at the end of the pass (0: none)
    uint32_t *ctl;               // [4], zero before the pass: units counted, scatter ticket
    uint32_t *seg_done;          // [G], zero before the pass: units counted per segment
    uint32_t *seg_tot;           // [G*bins], zero before the pass: the segments' bucket totals
    unsigned long long *look;    // [max_units][bins]: look-back words (flag | value)
    uint32_t *part_begin;        // [G*bins]
    uint32_t *part_end;          // [G*bins]
    uint32_t *error;             // bit 4: a bulk-copy wait ran out
    // the next pass's plan over this pass's partitions (written by the unit counted last)
    uint32_t *next_plan;         // [G*bins + 3] or null
    int next_max_units;
    uint32_t next_split;
};

struct ProbeParams {
    // columnar (unpartitioned) or row-contiguous (partitioned) sources of both tables
    const void *r_keys, *r_pay, *r_hash, *r_rows_in;
    const void *s_keys, *s_pay, *s_hash, *s_rows_in;
    const uint32_t *r_begin, *r_end;  // [np]; null: one partition = whole table
    const uint32_t *s_begin, *s_end;
    uint32_t r_rows, s_rows;
    int np;
    uint32_t rcap;         // build rows per item (a power of two)
    uint32_t schunk;       // probe rows per item
    uint32_t tcap;         // table slots per table buffer (a power of two, >= rcap * tmul)
    uint32_t tmul;         // table slots per build row of an item (2, 4 or 8: load <= 1/tmul)
    uint32_t scap;         // staged output pairs per item
    uint32_t *item_begin;  // [np+2]: prefix, total, and whether item_desc is filled
    uint4 *item_desc;      // [item_cap]: build rows [x, y), probe rows [z, w) of each item
    uint32_t *item_join;   // [item_cap]: join of each item (batches of joins)
    uint32_t item_cap;
    int slot_shift;        // rows with a hash: table slot = (mix_hash(hash) >> slot_shift) & (capacity - 1)
    uint32_t *ticket;
    unsigned long long *out_count;
    void *out;
    uint64_t capacity;
    HashSpec hs;
    uint32_t *error;
    // batches of joins (out_begin set): join j's pairs go to out[out_begin[j],
    // out_begin[j+1]), counted in out_counts[j]; item_join gives each item's join
    uint32_t joins;
    const unsigned long long *out_begin;
    unsigned long long *out_counts;
};

// ------------------------------------------------------------------ small helpers

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024, multiple of 32).
// `warp_sums` needs 32 entries. Returns the exclusive prefix; *total gets the block sum.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *warp_sums, T *total) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nwarps ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nwarps) warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    T before = warp > 0 ? warp_sums[warp - 1] : T(0);
    T result = before + x - v;
    if (total) *total = warp_sums[nwarps - 1];
    __syncthreads();
    return result;
}

// Generic (non-FNV) row hash, out of line.
template <typename H, int ALGO>
__device__ H row_hash_algo(const uint32_t *w, int kw) {
    constexpr int ROUNDS = ALGO == VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT ? 2 : 1;
    HashState<H, 32, ALGO> st;
    st.init();
    for (int round = 0; round < ROUNDS; round++) {
        for (int i = 0; i < kw; i++) {
            st.lane((int64_t)(uint64_t)w[i]);
            st.end_chunk();
        }
    }
    return st.h;
}

template <typename H>
__device__ H row_hash_h(const uint32_t *w, int kw, int algo) {
    switch (algo) {
    case VJ_HASH_CUSTOM_XOR: return row_hash_algo<H, VJ_HASH_CUSTOM_XOR>(w, kw);
    case VJ_HASH_CUSTOM_XOR_SHIFT: return row_hash_algo<H, VJ_HASH_CUSTOM_XOR_SHIFT>(w, kw);
    case VJ_HASH_CUSTOM_XOR_HW: return row_hash_algo<H, VJ_HASH_CUSTOM_XOR_HW>(w, kw);
    case VJ_HASH_CUSTOM_MULT_XOR_SHIFT: return row_hash_algo<H, VJ_HASH_CUSTOM_MULT_XOR_SHIFT>(w, kw);
    case VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT: return row_hash_algo<H, VJ_HASH_CUSTOM_N_MULT_XOR_SHIFT>(w, kw);
    case VJ_HASH_CUSTOM_MULT_XOR_HW: return row_hash_algo<H, VJ_HASH_CUSTOM_MULT_XOR_HW>(w, kw);
    case VJ_HASH_CUSTOM_MULT: return row_hash_algo<H, VJ_HASH_CUSTOM_MULT>(w, kw);
    case VJ_HASH_CUSTOM_MULT_SHIFT: return row_hash_algo<H, VJ_HASH_CUSTOM_MULT_SHIFT>(w, kw);
    case VJ_HASH_CUSTOM_MULT_HW: return row_hash_algo<H, VJ_HASH_CUSTOM_MULT_HW>(w, kw);
    case VJ_HASH_CUSTOM_ADD: return row_hash_algo<H, VJ_HASH_CUSTOM_ADD>(w, kw);
    case VJ_HASH_CUSTOM_ADD_SHIFT: return row_hash_algo<H, VJ_HASH_CUSTOM_ADD_SHIFT>(w, kw);
    case VJ_HASH_CUSTOM_ADD_HW: return row_hash_algo<H, VJ_HASH_CUSTOM_ADD_HW>(w, kw);
    default: return row_hash_algo<H, VJ_HASH_FNV>(w, kw);
    }
}

// One copy per key width: a single copy shared by every layout's kernels is compiled to
// the widest caller's frame, and every caller then pays in registers (the 2^27 x 2^29 join's
// pass-1 scatter spilled 20 bytes and ran 0.3 ms slower).
template <int KW>
static __device__ __noinline__ uint64_t row_hash_generic(const uint32_t *w, int kw, int algo, int hash_bits) {
    if (hash_bits == 64) {
        return row_hash_h<uint64_t>(w, kw, algo);
    }
    return (uint64_t)row_hash_h<uint32_t>(w, kw, algo);
}

// Hash of a key row as hash_func would compute it over 32-bit chunks.
template <int KW>
__device__ __forceinline__ uint64_t row_hash(const Key<KW> &k, const HashSpec &hs) {
    if (hs.algo == VJ_HASH_FNV) {
        return hs.hash_bits == 64 ? fnv_words<uint64_t, KW>(k.w) : (uint64_t)fnv_words<uint32_t, KW>(k.w);
    }
    uint32_t w[KW];
#pragma unroll
    for (int i = 0; i < KW; i++) w[i] = k.w[i];
    return row_hash_generic<KW>(w, KW, hs.algo, hs.hash_bits);
}

// Multiplicative (Fibonacci) mix: its top bits depend on every bit of the hash. The join
// cuts its partitions from the top bits, most significant first; rows that carry their hash
// take the table slot from the bits right below them (table_slot), so rows of one partition
// still spread over the table.
__device__ __forceinline__ uint64_t mix_hash(uint64_t h) {
    return h * 0x9e3779b97f4a7c15ull;
}

// Table slot bits of a build or probe row (masked by the table size; tables hold at most
// 2^SLOT_BITS slots). With hashes carried in the rows: mix_hash(hash) right below the
// partition bits. Otherwise the top bits of a multiplicative mix of the key itself: the
// tables are private to the probe and build and probe rows agree on the function, so the
// probe computes no row hash -- a fold and one multiply where FNV-1a 64 of an 8-byte key is
// eight dependent multiplies. The fold (x -> x ^ x >> 32, a bijection) lets every key bit
// reach the top bits. (With the match ballots below: 4.04 -> 3.77 ms for the 2^27 x 2^29
// join's probe.)
constexpr int SLOT_BITS = 14;
template <int KW, int HS>
__device__ __forceinline__ uint32_t table_slot(const Key<KW> &k, uint64_t h, int slot_shift) {
    if (HS) return (uint32_t)(mix_hash(h) >> slot_shift);
    uint64_t x = k.w[0] | (KW > 1 ? (uint64_t)k.w[1] << 32 : 0ull);
#pragma unroll
    for (int i = 2; i < KW; i += 2) x = (x ^ (x >> 32)) * 0x9e3779b97f4a7c15ull ^ (k.w[i] | (i + 1 < KW ? (uint64_t)k.w[i + 1] << 32 : 0ull));
    x ^= x >> 32;
    return (uint32_t)((x * 0x9e3779b97f4a7c15ull) >> (64 - SLOT_BITS));
}

__device__ __forceinline__ uint64_t bucket_hash(uint64_t h, const HashSpec &hs) {
    return hs.mix ? mix_hash(h) : h;
}

template <int HS>
__device__ __forceinline__ uint64_t read_hash(const unsigned char *p) {
    if (HS == 8) return *(const unsigned long long *)p;
    return *(const uint32_t *)p;
}

// ------------------------------------------------------------------ rows in shared memory
//
// A chunk of rows [a, b) of a table is copied into shared memory by bulk copies of the
// 16-byte aligned windows that cover it: one window for a row-contiguous source, one per
// column for a columnar source. The view gives key / payload / hash of row a + i.

template <int KW, int PB, int HS, bool AOS>
struct Chunk {
    using L = Layout<KW, PB, HS>;
    using P = typename PayloadType<PB>::T;
    __host__ __device__ static constexpr size_t col(size_t bytes) { return (bytes + 32 + 15) / 16 * 16; }
    __host__ __device__ static constexpr size_t bytes(uint32_t rows) {
        return AOS ? col((size_t)rows * L::STRIDE) : col((size_t)rows * L::KB) + col((size_t)rows * PB) + (HS ? col((size_t)rows * HS) : 0);
    }
    // shared-memory views
    const unsigned char *k;
    const unsigned char *p;
    const unsigned char *h;
    __device__ __forceinline__ Key<KW> key(uint32_t i) const { return key_from_smem<KW>(k + (size_t)i * (AOS ? L::STRIDE : L::KB)); }
    __device__ __forceinline__ P pay(uint32_t i) const { return *(const P *)(p + (size_t)i * (AOS ? L::STRIDE : PB)); }
    __device__ __forceinline__ uint64_t hash(uint32_t i) const { return read_hash<HS>(h + (size_t)i * (AOS ? L::STRIDE : HS)); }
    __device__ __forceinline__ uint64_t h_of(uint32_t i, const HashSpec &hs) const { return HS ? hash(i) : row_hash<KW>(key(i), hs); }
    // copy of row i as raw bytes into `dst` (row-contiguous layout), one shared-memory
    // store per row where the row is 8 or 16 bytes: the rows land at random positions, and
    // a warp's store costs as many passes as lanes hitting one bank group, so two stores of
    // half rows cost twice the bank conflicts of one. Row-contiguous inputs are the join's
    // own buffers (256-byte aligned), so their rows are 16-byte aligned when STRIDE is.
    __device__ __forceinline__ void copy_row(uint32_t i, unsigned char *dst) const {
        if (AOS) {
            const unsigned char *src = k + (size_t)i * L::STRIDE;
            if (L::STRIDE % 16 == 0) {
#pragma unroll
                for (int o = 0; o < L::STRIDE; o += 16) *(uint4 *)(dst + o) = *(const uint4 *)(src + o);
            } else {
#pragma unroll
                for (int o = 0; o < L::STRIDE; o += 8) *(uint2 *)(dst + o) = *(const uint2 *)(src + o);
            }
        } else if (KW == 2 && PB == 8 && HS == 0) {
            const uint2 kk = *(const uint2 *)(k + (size_t)i * 8);
            const uint2 pp = *(const uint2 *)(p + (size_t)i * 8);
            *(uint4 *)dst = make_uint4(kk.x, kk.y, pp.x, pp.y);
        } else if (KW == 1 && PB == 4 && HS == 0) {
            *(uint2 *)dst = make_uint2(*(const uint32_t *)(k + (size_t)i * 4), *(const uint32_t *)(p + (size_t)i * 4));
        } else {
            key_to_smem<KW>(dst, key(i));
            *(P *)(dst + L::PAY_OFF) = pay(i);
            if (HS == 8) *(unsigned long long *)(dst + L::HASH_OFF) = hash(i);
            if (HS == 4) *(uint32_t *)(dst + L::HASH_OFF) = (uint32_t)hash(i);
        }
    }

    // Issue the copies of rows [a, b) into `buf` (capacity `cap` rows); deltas[0..2] receive
    // the offsets of row a inside the windows. Called by one thread.
    __device__ __forceinline__ static void issue(const void *keys, const void *pay, const void *hash, const void *rows, uint32_t a, uint32_t b, uint32_t cap, unsigned char *buf, uint64_t *bar,
                                                 uint32_t *deltas) {
        if (AOS) {
            const ColWindow w = col_window(rows, L::STRIDE, a, b);
            deltas[0] = w.delta;
            mbar_arrive_expect_tx(bar, w.bytes);
            bulk_g2s(buf, w.src, w.bytes, bar);
        } else {
            const ColWindow wk = col_window(keys, L::KB, a, b);
            const ColWindow wp = col_window(pay, PB, a, b);
            uint32_t total = wk.bytes + wp.bytes;
            ColWindow wh{nullptr, 0, 0};
            if (HS) {
                wh = col_window(hash, HS, a, b);
                total += wh.bytes;
            }
            deltas[0] = wk.delta;
            deltas[1] = wp.delta;
            deltas[2] = wh.delta;
            const size_t kcol = col((size_t)cap * L::KB), pcol = col((size_t)cap * PB);
            mbar_arrive_expect_tx(bar, total);
            bulk_g2s(buf, wk.src, wk.bytes, bar);
            bulk_g2s(buf + kcol, wp.src, wp.bytes, bar);
            if (HS) bulk_g2s(buf + kcol + pcol, wh.src, wh.bytes, bar);
        }
    }

    // Ask L2 for rows [a, b) ahead of their bulk copy. Called by one thread.
    __device__ __forceinline__ static void prefetch(const void *keys, const void *pay, const void *hash, const void *rows, uint32_t a, uint32_t b) {
        if (a >= b) return;
        if (AOS) {
            const ColWindow w = col_window(rows, L::STRIDE, a, b);
            bulk_prefetch_l2(w.src, w.bytes);
        } else {
            const ColWindow wk = col_window(keys, L::KB, a, b);
            const ColWindow wp = col_window(pay, PB, a, b);
            bulk_prefetch_l2(wk.src, wk.bytes);
            bulk_prefetch_l2(wp.src, wp.bytes);
            if (HS) {
                const ColWindow wh = col_window(hash, HS, a, b);
                bulk_prefetch_l2(wh.src, wh.bytes);
            }
        }
    }

    __device__ __forceinline__ static Chunk view(const unsigned char *buf, uint32_t cap, const uint32_t *deltas) {
        Chunk c;
        if (AOS) {
            c.k = buf + deltas[0];
            c.p = c.k + L::PAY_OFF;
            c.h = c.k + L::HASH_OFF;
        } else {
            const size_t kcol = col((size_t)cap * L::KB), pcol = col((size_t)cap * PB);
            c.k = buf + deltas[0];
            c.p = buf + kcol + deltas[1];
            c.h = buf + kcol + pcol + deltas[2];
        }
        return c;
    }
};

// ------------------------------------------------------------------ partition kernels
//
// A pass over G segments runs two kernels:
//   histogram  each block counts one unit (a row range of one segment) per bucket in shared
//              memory and publishes the counts as the unit's look-back words; the segment's
//              bucket totals add up in global memory. The block that counts a segment's last
//              unit turns its totals into partition bounds, and the block that counts the
//              last unit of all plans the next pass's units over those partitions.
//   scatter    persistent; blocks take units by ticket, in order. A unit's write cursor per
//              bucket is its partition's begin plus the rows of the segment's earlier units
//              in that bucket, found by decoupled look-back: a predecessor's word holds
//              either its own count or, once that unit has looked back itself, its inclusive
//              prefix, so a walk stops at the nearest inclusive prefix. The block then
//              streams the unit's rows through shared memory in tiles (bulk copies, double
//              buffered across units), ranks each tile by bucket, sorts it in shared memory
//              and writes each bucket run as one contiguous burst.

// Look-back words: flag (2 bits) | value (62 bits).
constexpr unsigned long long LB_AGG = 1, LB_INC = 2;
constexpr unsigned long long LB_VALUE = (1ull << 62) - 1;
__device__ __forceinline__ unsigned long long lb_pack(unsigned long long flag, unsigned long long v) { return (flag << 62) | v; }
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) { asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory"); }
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Unit u of a pass: segment g (of side `side`), rows [a, b); its index in the segment and
// whether it is the segment's first / last unit.
struct UnitRange {
    uint32_t g, side, a, b, rank;
    bool first, last;
};

__device__ __forceinline__ const uint32_t *plan_first(const PassParams &P) { return P.plan ? P.plan + 1 : P.hplan + 1; }

__device__ __forceinline__ uint32_t plan_total(const PassParams &P) { return plan_first(P)[P.nsides * P.Q]; }

// Units of segment g.
__device__ __forceinline__ uint32_t seg_units(const PassParams &P, uint32_t g) {
    const uint32_t *first = plan_first(P);
    return first[g + 1] - first[g];
}

__device__ __forceinline__ UnitRange unit_range(const PassParams &P, uint32_t u) {
    const uint32_t G = (uint32_t)(P.nsides * P.Q);
    const uint32_t *first = plan_first(P);
    const uint32_t target = P.plan ? P.plan[0] : P.hplan[0];
    const uint32_t from = first[G + 1];  // the first quarter unit
    uint32_t lo = 0, hi = G - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (first[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t g = lo, f0 = first[g], f1 = first[g + 1];
    UnitRange r;
    r.g = g;
    r.side = g / (uint32_t)P.Q;
    const uint32_t sb = P.seg_begin ? P.seg_begin[g] : 0;
    const uint32_t se = P.seg_end ? P.seg_end[g] : P.side[r.side].rows;
    // the whole unit it is (or a quarter of): index in the plan before the split
    const uint32_t whole = u < from ? u : from + (u - from) / 4;
    const uint32_t seg0 = f0 <= from ? f0 : from + (f0 - from) / 4;
    const unsigned long long a = (unsigned long long)sb + (unsigned long long)(whole - seg0) * target;
    unsigned long long ra = a < se ? a : se;
    unsigned long long rb = a + target < se ? a + target : se;
    if (u >= from) {
        const unsigned long long len = rb - ra, q = (u - from) & 3u;
        rb = ra + len * (q + 1) / 4;
        ra = ra + len * q / 4;
    }
    r.a = (uint32_t)ra;
    r.b = (uint32_t)rb;
    r.rank = u - f0;
    r.first = u == f0;
    r.last = u + 1 == f1;
    return r;
}

// Units from `from` on (the last `split` whole units of the plan, in unit order) become four
// quarter units each: unit index x of the whole-unit plan maps to split_index(x).
__host__ __device__ __forceinline__ uint32_t split_index(uint32_t x, uint32_t from) { return x <= from ? x : from + 4 * (x - from); }

// One block: units of `target` rows for the G segments [begin[g], end[g]) -- at least one per
// segment, so that every segment's bounds are written by its last unit. plan[0] = target,
// plan[1 + g] = the first unit of g, plan[1 + G] = all units, plan[2 + G] = the first quarter
// unit: the last min(split, units / 4) whole units are cut in four, so that blocks finishing
// a pass take short units (its tail shrinks by as much). target is the larger of min_rows
// and the rows that spread the segments over max_units - G - 3 split units.
static __device__ void plan_block(const uint32_t *begin, const uint32_t *end, uint32_t G, uint32_t max_units, uint32_t min_rows, uint32_t split, uint32_t *plan) {
    __shared__ unsigned long long s_w64[32];
    __shared__ uint32_t s_w32[32];
    __shared__ uint32_t s_target;
    const uint32_t per = (G + blockDim.x - 1) / blockDim.x;
    const uint32_t g0 = threadIdx.x * per;
    unsigned long long rows = 0;
    for (uint32_t g = g0; g < g0 + per && g < G; g++) rows += end[g] - begin[g];
    unsigned long long total = 0;
    block_exclusive_scan<unsigned long long>(rows, s_w64, &total);
    if (threadIdx.x == 0) {
        const unsigned long long room = max_units > G + 3 * split ? (unsigned long long)(max_units - G - 3 * split) : 1ull;
        unsigned long long t = (total + room - 1) / room;
        if (t < min_rows) t = min_rows;
        if (t < 1) t = 1;
        if (t > 0x7fffffffull) t = 0x7fffffffull;
        s_target = (uint32_t)t;
    }
    __syncthreads();
    const uint32_t target = s_target;
    uint32_t mine = 0;
    for (uint32_t g = g0; g < g0 + per && g < G; g++) {
        const uint32_t n = end[g] - begin[g];
        mine += n ? (n + target - 1) / target : 1u;
    }
    uint32_t units = 0;
    uint32_t run = block_exclusive_scan<uint32_t>(mine, s_w32, &units);
    const uint32_t from = units - min(split, units / 4);
    for (uint32_t g = g0; g < g0 + per && g < G; g++) {
        plan[1 + g] = split_index(run, from);
        const uint32_t n = end[g] - begin[g];
        run += n ? (n + target - 1) / target : 1u;
    }
    if (threadIdx.x == 0) {
        plan[0] = target;
        plan[1 + G] = split_index(units, from);
        plan[2 + G] = from;
    }
}

// One block: the unit plan of a pass over device segments (batches of joins).
static __global__ void __launch_bounds__(PLAN_THREADS) plan_kernel(PassParams P, uint32_t *plan) {
    plan_block(P.seg_begin, P.seg_end, (uint32_t)(P.nsides * P.Q), (uint32_t)P.max_units, P.min_unit_rows, P.split, plan);
}

// L2 prefetch of what the histogram reads of rows [a, b): the hash or key column, or the rows.
template <int KW, int PB, int HS, bool AOS>
__device__ __forceinline__ void histogram_prefetch(const Side &S, uint32_t a, uint32_t b) {
    using L = Layout<KW, PB, HS>;
    if (a >= b) return;
    const ColWindow w = AOS ? col_window(S.rows_in, L::STRIDE, a, b) : (HS ? col_window(S.hash_in, HS, a, b) : col_window(S.keys_in, L::KB, a, b));
    bulk_prefetch_l2(w.src, w.bytes);
}

// Hash of row i read straight from global memory (histogram pass).
template <int KW, int PB, int HS, bool AOS>
__device__ __forceinline__ uint64_t global_row_hash(const Side &S, uint32_t i, const HashSpec &hs) {
    using L = Layout<KW, PB, HS>;
    if (AOS) {
        const unsigned char *row = (const unsigned char *)S.rows_in + (size_t)i * L::STRIDE;
        if (HS == 8) return __ldcs((const unsigned long long *)(row + L::HASH_OFF));
        if (HS == 4) return __ldcs((const uint32_t *)(row + L::HASH_OFF));
        Key<KW> k;
        if (KW == 1) {
            k.w[0] = __ldcs((const uint32_t *)row);
        } else {
#pragma unroll
            for (int j = 0; j < KW / 2; j++) {
                uint2 v = __ldcs((const uint2 *)row + j);
                k.w[2 * j] = v.x;
                k.w[2 * j + 1] = v.y;
            }
        }
        return row_hash<KW>(k, hs);
    }
    if (HS == 8) return __ldcs((const unsigned long long *)S.hash_in + i);
    if (HS == 4) return __ldcs((const uint32_t *)S.hash_in + i);
    return row_hash<KW>(load_key_stream<KW>(S.keys_in, i), hs);
}

// Rows [a, b) of a 16-byte aligned column whose 16-byte groups hold G rows, by the whole
// block (NT threads): whole groups by 16-byte loads, two in flight per thread; the rows
// before the first whole group and after the last one at a time. one(i) counts row i,
// group(v) the G rows of a loaded group. Fewer, wider loads keep more bytes in flight per
// thread: for the 2^27 x 2^29 int64 join, pass 1's key counts took 0.85 ms instead of 1.20
// (two 8-byte keys a load) and pass 2's bucket-id counts 0.32 instead of 0.41 (eight ids).
template <int NT, int G, typename One, typename Group>
__device__ __forceinline__ void count_groups(const void *column, uint32_t a, uint32_t b, One one, Group group) {
    const uint4 *col = (const uint4 *)column;
    const uint32_t ga = (a + G - 1) / G, gb = b / G;
    const bool whole = ga < gb;
    const uint32_t head = whole ? ga * G - a : b - a, tail = whole ? b - gb * G : 0;
    for (uint32_t t = threadIdx.x; t < head + tail; t += NT) one(t < head ? a + t : gb * G + (t - head));
    if (!whole) return;
    uint32_t q = ga + threadIdx.x;
    for (; q + NT < gb; q += 2 * NT) {
        const uint4 v0 = __ldcs(col + q), v1 = __ldcs(col + q + NT);
        group(v0);
        group(v1);
    }
    for (; q < gb; q += NT) group(__ldcs(col + q));
}

// Block scratch of the histogram: the unit (kept in shared memory, so no registers are held
// across the count), the block-scan words and the last-unit flag.
struct HistShared {
    UnitRange unit;
    uint32_t u;
    uint32_t warp[32];
    uint32_t last;
};

// Counts of unit u by the whole block (NT threads); s_hist holds 2^bits words.
template <int KW, int PB, int HS, bool AOS, int NT>
__device__ __forceinline__ void histogram_unit(const PassParams &P, uint32_t u, uint32_t *s_hist, HistShared &sh) {
    const uint32_t bins = 1u << P.bits;
    const uint64_t mask = bins - 1;
    if (threadIdx.x == 0) {
        sh.unit = unit_range(P, u);
        sh.u = u;
    }
    for (uint32_t b = threadIdx.x; b < bins; b += NT) s_hist[b] = 0;
    __syncthreads();
    const UnitRange &U = sh.unit;
    const Side &S = P.side[U.side];

    // ---- count
    const auto count_row = [&](uint32_t i) { atomicAdd(&s_hist[(bucket_hash(global_row_hash<KW, PB, HS, AOS>(S, i, P.hs), P.hs) >> P.shift) & mask], 1u); };
    if (AOS && S.bid_in && ((uintptr_t)S.bid_in & 15) == 0) {
        // buckets written by the previous pass: 2 bytes a row instead of the row
        count_groups<NT, 8>(
            S.bid_in, U.a, U.b, [&](uint32_t i) { atomicAdd(&s_hist[__ldcs(S.bid_in + i) & mask], 1u); },
            [&](const uint4 &v) {
                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    atomicAdd(&s_hist[w[k] & 0xffffu & mask], 1u);
                    atomicAdd(&s_hist[(w[k] >> 16) & mask], 1u);
                }
            });
    } else if (!AOS && HS == 0 && KW <= 2 && ((uintptr_t)S.keys_in & 15) == 0) {
        // 4- or 8-byte keys, 4 or 2 a load (the group size of wider keys is never used)
        count_groups<NT, (KW <= 2 ? 4 / KW : 1)>(S.keys_in, U.a, U.b, count_row, [&](const uint4 &v) {
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int k = 0; k < 4; k += KW) {
                Key<KW> key;
#pragma unroll
                for (int x = 0; x < KW; x++) key.w[x] = w[k + x];
                atomicAdd(&s_hist[(bucket_hash(row_hash<KW>(key, P.hs), P.hs) >> P.shift) & mask], 1u);
            }
        });
    } else if (S.bid_in) {
        constexpr int UB = 8;
        uint32_t i = U.a + threadIdx.x;
        for (; i + (UB - 1) * NT < U.b; i += UB * NT) {
            uint32_t v[UB];
#pragma unroll
            for (int k = 0; k < UB; k++) v[k] = __ldcs(S.bid_in + i + k * NT);
#pragma unroll
            for (int k = 0; k < UB; k++) atomicAdd(&s_hist[v[k] & mask], 1u);
        }
        for (; i < U.b; i += NT) atomicAdd(&s_hist[__ldcs(S.bid_in + i) & mask], 1u);
    } else {
        constexpr int UNROLL = 4;
        constexpr uint32_t STEP = UNROLL * NT;
        // keep the next AHEAD steps of this unit on their way to L2
        constexpr uint32_t AHEAD = 4;
        if (threadIdx.x == 0) histogram_prefetch<KW, PB, HS, AOS>(S, U.a, min(U.b, U.a + AHEAD * STEP));
        uint32_t i = U.a + threadIdx.x;
        for (; i + (UNROLL - 1) * NT < U.b; i += UNROLL * NT) {
            if (threadIdx.x == 0) {
                const uint32_t pa = i + AHEAD * STEP;
                if (pa < U.b) histogram_prefetch<KW, PB, HS, AOS>(S, pa, min(U.b, pa + STEP));
            }
            uint64_t h[UNROLL];
#pragma unroll
            for (int k = 0; k < UNROLL; k++) h[k] = global_row_hash<KW, PB, HS, AOS>(S, i + k * NT, P.hs);
#pragma unroll
            for (int k = 0; k < UNROLL; k++) atomicAdd(&s_hist[(bucket_hash(h[k], P.hs) >> P.shift) & mask], 1u);
        }
        for (; i < U.b; i += NT) count_row(i);
    }
    __syncthreads();

    // ---- publish: the unit's counts (its look-back words; the segment's first unit's are
    // already its inclusive prefix) and the segment's totals
    unsigned long long *L = P.look + (size_t)sh.u * bins;
    for (uint32_t b = threadIdx.x; b < bins; b += NT) {
        const uint32_t c = s_hist[b];
        L[b] = lb_pack(U.first ? LB_INC : LB_AGG, c);
        if (c) atomicAdd(&P.seg_tot[(size_t)U.g * bins + b], c);
    }
    // the block's totals are ordered before its count of the segment's units: the barrier
    // orders them before thread 0, whose fence makes them visible device-wide
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        sh.last = atomicAdd(&P.seg_done[U.g], 1u) + 1 == seg_units(P, U.g);
    }
    __syncthreads();
    // ---- the segment's last unit counted: partition bounds of the segment
    if (sh.last) {
        __threadfence();
        const uint32_t *tot = P.seg_tot + (size_t)U.g * bins;
        const uint32_t per = (bins + NT - 1) / NT;
        const uint32_t b0 = threadIdx.x * per;
        uint32_t mine = 0;
        for (uint32_t b = b0; b < b0 + per && b < bins; b++) mine += __ldcg(tot + b);
        uint32_t run = block_exclusive_scan<uint32_t>(mine, sh.warp, nullptr);
        run += P.seg_begin ? P.seg_begin[U.g] : 0;
        for (uint32_t b = b0; b < b0 + per && b < bins; b++) {
            P.part_begin[(size_t)U.g * bins + b] = run;
            run += __ldcg(tot + b);
            P.part_end[(size_t)U.g * bins + b] = run;
        }
    }

    // ---- the last unit of all: the next pass's plan over this pass's partitions
    if (P.next_plan) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            sh.last = atomicAdd(&P.ctl[0], 1u) + 1 == plan_total(P);
        }
        __syncthreads();
        if (sh.last) {
            __threadfence();
            plan_block(P.part_begin, P.part_end, (uint32_t)(P.nsides * P.Q) * bins, (uint32_t)P.next_max_units, P.min_unit_rows, P.next_split, P.next_plan);
        }
    }
}

// Grid: one block per unit of the plan (blocks past the plan's units leave at once). Four
// blocks per SM (32 registers a thread) keep enough loads in flight.
// LOOP: a grid smaller than the plan (SMs left to other work) takes units blockIdx.x,
// blockIdx.x + gridDim.x, ... (a separate instance: the loop costs the one-unit kernel
// registers at its 32-register bound).
template <int KW, int PB, int HS, bool AOS, bool LOOP = false>
__global__ void __launch_bounds__(PART_THREADS, 4) histogram_kernel(PassParams P) {
    extern __shared__ uint32_t s_hist[];
    __shared__ HistShared sh;
    if constexpr (LOOP) {
        uint32_t u = blockIdx.x;
        while (u < plan_total(P)) {
            histogram_unit<KW, PB, HS, AOS, PART_THREADS>(P, u, s_hist, sh);
            const uint32_t next = sh.u + gridDim.x;
            __syncthreads();  // every thread has read sh.u before the next unit rewrites it
            u = next;
        }
    } else {
        if (blockIdx.x >= plan_total(P)) return;
        histogram_unit<KW, PB, HS, AOS, PART_THREADS>(P, blockIdx.x, s_hist, sh);
    }
}

// Shared memory of the scatter kernel: two input tiles filled by bulk copies, the
// bucket-sorted output tile (row-contiguous), each sorted row's bucket, and per bucket the
// tile's counts (two tiles), its start in the sorted tile and the unit's write cursor.
template <int KW, int PB, int HS, bool IN_AOS, int ITEMS, int NT = PART_THREADS>
struct ScatterSmem {
    using L = Layout<KW, PB, HS>;
    static constexpr int T = NT * ITEMS;
    static constexpr size_t IN_BUF = Chunk<KW, PB, HS, IN_AOS>::bytes(T);
    static constexpr size_t OUT = (size_t)T * (L::STRIDE + 4);  // rows + bucket word per row
    // + per bucket: counts of two tiles, start, cursor; chunk totals past 1024 buckets
    static constexpr size_t bytes(uint32_t bins) { return 16 + 2 * IN_BUF + OUT + (size_t)bins * 4 * 4 + (bins > 1024 ? bins / 32 * 4 : 0); }
};

// Rows per thread of a scatter tile: the largest of 4, 2, 1 whose block (with 2^9 bins)
// fits twice in an SM's 228 KB with the per-block 1 KB reservation and ~0.1 KB of static
// shared memory (wider passes, up to 2^12 bins, run one block per SM).
constexpr size_t SCATTER_HALF_SM = 228 * 1024 / 2 - 1024 - 128;
template <int KW, int PB, int HS, bool IN_AOS>
constexpr int scatter_items() {
    return ScatterSmem<KW, PB, HS, IN_AOS, 4>::IN_BUF * 2 + ScatterSmem<KW, PB, HS, IN_AOS, 4>::OUT + 16 + 512 * 16 <= SCATTER_HALF_SM   ? 4
           : ScatterSmem<KW, PB, HS, IN_AOS, 2>::IN_BUF * 2 + ScatterSmem<KW, PB, HS, IN_AOS, 2>::OUT + 16 + 512 * 16 <= SCATTER_HALF_SM ? 2
                                                                                                                                     : 1;
}

// Tile descriptor passed from the issuing thread to the block: unit, rows [a, b),
// segment | side << 30 | (first tile of its unit) << 31, and the unit's index in its
// segment. unit ~0: no tile (end).
struct TileDesc {
    uint32_t unit, a, b, gs, rank;
};

// State of the scatter's issuing thread: the unit it is cutting into tiles.
struct TileIssuer {
    uint32_t u = 0, a = 0, e = 0, g = 0, side = 0, rank = 0;
    bool fresh = false;
};

// Rows of bucket b in the units of u's segment before u (u is the rank-th unit of its
// segment), by decoupled look-back over the units' words, LB at a time; then u's own word
// becomes its inclusive prefix for the units after it. The histogram wrote every unit's
// count before the scatter started, so no word is ever missing: a walk never waits.
__device__ __forceinline__ unsigned long long look_back(const PassParams &P, uint32_t u, uint32_t rank, uint32_t b, uint32_t bins) {
    constexpr uint32_t LB = 4;
    unsigned long long *mine = P.look + (size_t)u * bins + b;
    unsigned long long prefix = 0;
    if (rank > 0) {
        const unsigned long long own = ld_relaxed(mine);
        uint32_t left = rank;  // predecessors in the segment not yet added
        uint32_t v = u - 1;
        bool done = false;
        while (!done && left) {
            const uint32_t n = left < LB ? left : LB;
            unsigned long long w[LB];
#pragma unroll
            for (uint32_t i = 0; i < LB; i++) w[i] = i < n ? ld_relaxed(P.look + (size_t)(v - i) * bins + b) : 0ull;
#pragma unroll
            for (uint32_t i = 0; i < LB; i++) {
                if (done || i >= n) continue;
                prefix += w[i] & LB_VALUE;
                done = (w[i] >> 62) == LB_INC;
            }
            v -= n;
            left -= n;
        }
        st_relaxed(mine, lb_pack(LB_INC, prefix + (own & LB_VALUE)));
    }
    return prefix;
}

// The same, out of line: for buckets past the block's threads (passes of more than 2^9
// buckets), whose look-back happens while a tile's ranks are held in registers.
static __device__ __noinline__ unsigned long long look_back_far(const PassParams &P, uint32_t u, uint32_t rank, uint32_t b, uint32_t bins) { return look_back(P, u, rank, b, bins); }

// Issuing thread of the scatter: the next tile of its current unit, or the first tile of
// the next unit taken by ticket. Units without rows are skipped; their look-back words stay
// counts of zero, which later walks add and pass.
template <int KW, int PB, int HS, bool IN_AOS, int T>
__device__ __forceinline__ void scatter_issue(const PassParams &P, TileIssuer &is, uint32_t total, unsigned char *buf, uint64_t *bar, TileDesc *desc, uint32_t *deltas) {
    using C = Chunk<KW, PB, HS, IN_AOS>;
    const uint32_t bins = 1u << P.bits;
    while (is.a >= is.e) {
        const uint32_t u = atomicAdd(&P.ctl[1], 1u);
        if (u >= total) {
            *desc = TileDesc{~0u, 0, 0, 0, 0};
            mbar_arrive(bar);
            return;
        }
        const UnitRange U = unit_range(P, u);
        is.u = u;
        is.a = U.a;
        is.e = U.b;
        is.g = U.g;
        is.side = U.side;
        is.rank = U.rank;
        is.fresh = true;
        if (U.a < U.b && bins >= 4) {  // bulk prefetches take multiples of 16 bytes
            bulk_prefetch_l2(P.look + (size_t)u * bins, bins * 8);
            bulk_prefetch_l2(P.part_begin + (size_t)U.g * bins, bins * 4);
        }
    }
    const uint32_t b = min(is.e, is.a + (uint32_t)T);
    *desc = TileDesc{is.u, is.a, b, is.g | (is.side << 30) | (is.fresh ? 1u << 31 : 0u), is.rank};
    const Side &S = P.side[is.side];
    fence_proxy_async();
    C::issue(S.keys_in, S.pay_in, S.hash_in, S.rows_in, is.a, b, T, buf, bar, deltas);
    is.a = b;
    is.fresh = false;
}

// Block scratch of the scatter: the two tiles' descriptors and window offsets.
struct ScatterShared {
    TileDesc tile[2];
    uint32_t delta[2][3];
};

// The scatter of a pass by the whole block (NT threads) until the units run out; s_raw is
// the block's ScatterSmem<..., NT>::bytes(bins) of dynamic shared memory (128-byte aligned).
template <int KW, int PB, int HS, bool IN_AOS, bool OUT_AOS, int ITEMS, int NT>
__device__ __forceinline__ void scatter_run(const PassParams &P, unsigned char *s_raw, ScatterShared &sh) {
    using L = Layout<KW, PB, HS>;
    using C = Chunk<KW, PB, HS, IN_AOS>;
    using Pt = typename PayloadType<PB>::T;
    using SM = ScatterSmem<KW, PB, HS, IN_AOS, ITEMS, NT>;
    constexpr int T = SM::T;
    uint64_t *bar = (uint64_t *)s_raw;
    unsigned char *inb0 = s_raw + 16;
    unsigned char *out_rows = inb0 + 2 * SM::IN_BUF;
    // bucket of each sorted row, and in the high half the next pass's bucket (bid_out)
    uint32_t *st_b = (uint32_t *)(out_rows + (size_t)T * L::STRIDE);
    const uint32_t bins = 1u << P.bits;
    uint32_t *s_cnt = st_b + T;            // [2][bins]: counts of the tile (by parity)
    uint32_t *s_start = s_cnt + 2 * bins;  // [bins]: bucket start in the sorted tile
    uint32_t *s_run = s_start + bins;      // [bins]: output row of the tile's first row of the bucket
    uint32_t *s_chunk = s_run + bins;      // [bins / 32]: chunk totals (more than 1024 buckets)
    TileDesc *s_tile = sh.tile;
    uint32_t (*s_delta)[3] = sh.delta;
    const uint32_t total = plan_total(P);
    const uint64_t mask = bins - 1;
    const uint64_t nmask = (1ull << P.next_bits) - 1;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr uint32_t NW = NT / 32;

    TileIssuer is;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_proxy_async();
    }
    for (uint32_t b = threadIdx.x; b < 2 * bins; b += NT) s_cnt[b] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        scatter_issue<KW, PB, HS, IN_AOS, T>(P, is, total, inb0, &bar[0], &s_tile[0], s_delta[0]);
        scatter_issue<KW, PB, HS, IN_AOS, T>(P, is, total, inb0 + SM::IN_BUF, &bar[1], &s_tile[1], s_delta[1]);
    }

    for (uint32_t k = 0;; k++) {
        const uint32_t buf = k & 1;
        uint32_t *cnt = s_cnt + buf * bins;
        uint32_t *cnt_prev = s_cnt + (buf ^ 1) * bins;
        const bool ok = mbar_wait(&bar[buf], (k >> 1) & 1);
        const TileDesc D = s_tile[buf];
        const bool end = D.unit == ~0u;
        const Side &S = P.side[(D.gs >> 30) & 1];
        const uint32_t nt = D.b - D.a;
        const bool fresh = (D.gs >> 31) != 0;
        // a unit's first tile: this thread's first bucket's cursor by look-back, before the
        // ranks below are live (the other buckets', past the block's threads, in the scan)
        uint32_t lb0 = 0;
        if (ok && !end && fresh && threadIdx.x < bins) lb0 = (uint32_t)look_back(P, D.unit, D.rank, threadIdx.x, bins);
        uint32_t bk[ITEMS], rk[ITEMS];  // bucket | next pass's bucket << 16, rank in the tile
        const C in = C::view(inb0 + buf * SM::IN_BUF, T, s_delta[buf]);
        if (ok && !end) {
#pragma unroll
            for (int j = 0; j < ITEMS; j++) {
                const uint32_t i = j * NT + threadIdx.x;
                if (i < nt) {
                    const uint64_t mh = bucket_hash(in.h_of(i, P.hs), P.hs);
                    const uint32_t b = (uint32_t)((mh >> P.shift) & mask);
                    bk[j] = b | (OUT_AOS ? (uint32_t)((mh >> P.next_shift) & nmask) << 16 : 0u);
                    rk[j] = atomicAdd(&cnt[b], 1u);
                }
            }
        }
        if (__syncthreads_or(!ok)) {
            // a bulk copy never landed: flag it, let the other buffer's copy land, leave
            if (threadIdx.x == 0) {
                atomicOr(P.error, 4u);
                mbar_wait(&bar[buf ^ 1], ((k + 1) >> 1) & 1);
            }
            return;
        }
        if (end) break;

        // ---- per bucket: the unit's cursor (look-back for a unit's first tile, else the
        // previous tile's counts added), the previous tile's counts cleared, the start of the
        // bucket's rows in the sorted tile
        const uint32_t g = D.gs & 0x3fffffffu;
        for (uint32_t b = threadIdx.x; b < bins; b += NT) {
            if (fresh) s_run[b] = P.part_begin[(size_t)g * bins + b] + (b == threadIdx.x ? lb0 : (uint32_t)look_back_far(P, D.unit, D.rank, b, bins));
            else s_run[b] += cnt_prev[b];
            cnt_prev[b] = 0;
        }
        if (bins <= 1024) {
            // each warp adds up the buckets before its chunk itself: no barrier
            for (uint32_t c = warp; c * 32 < bins; c += NW) {
                const uint32_t b = c * 32 + lane;
                const uint32_t v = b < bins ? cnt[b] : 0u;
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if ((int)lane >= o) x += y;
                }
                uint32_t s = 0;
                for (uint32_t i = lane; i < c * 32; i += 32) s += cnt[i];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (b < bins) s_start[b] = s + x - v;
            }
        } else {
            // chunk totals first (one more barrier)
            const uint32_t nchunks = bins / 32;
            for (uint32_t c = warp; c < nchunks; c += NW) {
                uint32_t v = cnt[c * 32 + lane];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) s_chunk[c] = v;
            }
            __syncthreads();
            for (uint32_t c = warp; c < nchunks; c += NW) {
                const uint32_t b = c * 32 + lane;
                const uint32_t v = cnt[b];
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if ((int)lane >= o) x += y;
                }
                uint32_t s = 0;
                for (uint32_t i = lane; i < c; i += 32) s += s_chunk[i];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                s_start[b] = s + x - v;
            }
        }
        __syncthreads();
        // ---- rows into bucket order
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            const uint32_t i = j * NT + threadIdx.x;
            if (i < nt) {
                const uint32_t pos = s_start[bk[j] & 0xffffu] + rk[j];
                in.copy_row(i, out_rows + (size_t)pos * L::STRIDE);
                st_b[pos] = bk[j];
            }
        }
        __syncthreads();  // input buffer `buf` is free: refill it
        if (threadIdx.x == 0) scatter_issue<KW, PB, HS, IN_AOS, T>(P, is, total, inb0 + buf * SM::IN_BUF, &bar[buf], &s_tile[buf], s_delta[buf]);
        // ---- bucket runs out: row i of the sorted tile goes to cursor + (i - bucket start)
        for (uint32_t i = threadIdx.x; i < nt; i += NT) {
            const uint32_t sbk = st_b[i];
            const uint32_t b = sbk & 0xffffu;
            const uint32_t dst = s_run[b] + i - s_start[b];
            const unsigned char *row = out_rows + (size_t)i * L::STRIDE;
            if (OUT_AOS) {
                if (S.bid_out) st_evict_last(S.bid_out + dst, (uint16_t)(sbk >> 16), l2_evict_last());
                unsigned char *gp = (unsigned char *)S.rows_out + (size_t)dst * L::STRIDE;
                if (L::STRIDE % 16 == 0) {
                    const uint64_t pol = l2_evict_last();
#pragma unroll
                    for (int o = 0; o < L::STRIDE; o += 16) {
                        const uint4 v = *(const uint4 *)(row + o);
                        st_evict_last(gp + o, v, pol);
                    }
                } else {
                    const uint64_t pol = l2_evict_last();
#pragma unroll
                    for (int o = 0; o < L::STRIDE; o += 8) {
                        const uint2 v = *(const uint2 *)(row + o);
                        st_evict_last(gp + o, v, pol);
                    }
                }
            } else {
                store_key<KW>(S.keys_out, dst, key_from_smem<KW>(row));
                ((Pt *)S.pay_out)[dst] = *(const Pt *)(row + L::PAY_OFF);
                if (HS && S.hash_out) {
                    if (HS == 8) ((unsigned long long *)S.hash_out)[dst] = *(const unsigned long long *)(row + L::HASH_OFF);
                    else ((uint32_t *)S.hash_out)[dst] = *(const uint32_t *)(row + L::HASH_OFF);
                }
            }
        }
    }
}

template <int KW, int PB, int HS, bool IN_AOS, bool OUT_AOS, int ITEMS>
__global__ void __launch_bounds__(PART_THREADS) scatter_kernel(PassParams P) {
    extern __shared__ __align__(128) unsigned char s_raw[];
    __shared__ ScatterShared sh;
    scatter_run<KW, PB, HS, IN_AOS, OUT_AOS, ITEMS, PART_THREADS>(P, s_raw, sh);
}

// ------------------------------------------------------------------ probe kernels

// Work items of partition p: (build chunks) x (probe chunks), 0 if either side is empty.
__device__ __forceinline__ unsigned long long items_of(const ProbeParams &Q, int p) {
    const uint32_t nr = Q.r_begin ? Q.r_end[p] - Q.r_begin[p] : Q.r_rows;
    const uint32_t ns = Q.s_begin ? Q.s_end[p] - Q.s_begin[p] : Q.s_rows;
    if (!nr || !ns) return 0;
    return (unsigned long long)((nr + Q.rcap - 1) / Q.rcap) * ((ns + Q.schunk - 1) / Q.schunk);
}

// Work items, in three launches over blocks of PLAN_BLOCK partitions: items per partition
// and their prefix inside the block; the blocks' offsets and the total (the ticket and the
// counter reset); the global prefix and the item descriptors. A plan of 2^31 or more items
// (only reachable when almost every row shares one hash) is refused with error flag 2 and
// no items.
constexpr int PLAN_BLOCK = 256;

static __global__ void __launch_bounds__(PLAN_BLOCK) items_count_kernel(ProbeParams Q, unsigned long long *block_tot) {
    __shared__ unsigned long long s_warp[32];
    const int p = blockIdx.x * PLAN_BLOCK + threadIdx.x;
    const unsigned long long n = p < Q.np ? items_of(Q, p) : 0ull;
    unsigned long long tot = 0;
    const unsigned long long ex = block_exclusive_scan<unsigned long long>(n, s_warp, &tot);
    if (p < Q.np) Q.item_begin[p] = (uint32_t)(ex < 0xffffffffull ? ex : 0xffffffffull);
    if (threadIdx.x == 0) block_tot[blockIdx.x] = tot;
}

static __global__ void __launch_bounds__(PLAN_THREADS) items_scan_kernel(ProbeParams Q, unsigned long long *block_tot, int nblocks) {
    __shared__ unsigned long long s_warp[32];
    const int per = (nblocks + PLAN_THREADS - 1) / PLAN_THREADS;
    const int b0 = threadIdx.x * per;
    unsigned long long mine = 0;
    for (int b = b0; b < b0 + per && b < nblocks; b++) mine += block_tot[b];
    unsigned long long total = 0;
    unsigned long long run = block_exclusive_scan<unsigned long long>(mine, s_warp, &total);
    for (int b = b0; b < b0 + per && b < nblocks; b++) {
        const unsigned long long t = block_tot[b];
        block_tot[b] = run;
        run += t;
    }
    if (threadIdx.x == 0) {
        const bool too_many = total >= (1ull << 31);
        const bool fill = !too_many && total <= Q.item_cap;
        Q.item_begin[Q.np] = too_many ? 0u : (uint32_t)total;
        Q.item_begin[Q.np + 1] = fill ? 1u : 0u;
        if (too_many) atomicOr(Q.error, 2u);
        *Q.ticket = 0;
        *Q.out_count = 0;
    }
}

static __global__ void __launch_bounds__(PLAN_BLOCK) items_write_kernel(ProbeParams Q, const unsigned long long *block_base) {
    const int p = blockIdx.x * PLAN_BLOCK + threadIdx.x;
    if (p >= Q.np) return;
    unsigned long long run = block_base[blockIdx.x] + Q.item_begin[p];
    Q.item_begin[p] = (uint32_t)(run < 0xffffffffull ? run : 0xffffffffull);
    if (Q.item_begin[Q.np + 1] == 0u || !items_of(Q, p)) return;  // descriptors only when they all fit
    const uint32_t rb = Q.r_begin ? Q.r_begin[p] : 0, re = Q.r_begin ? Q.r_end[p] : Q.r_rows;
    const uint32_t sb = Q.s_begin ? Q.s_begin[p] : 0, se = Q.s_begin ? Q.s_end[p] : Q.s_rows;
    for (uint32_t r0 = rb; r0 < re; r0 += Q.rcap) {
        for (uint32_t s0 = sb; s0 < se; s0 += Q.schunk) {
            Q.item_desc[run++] = make_uint4(r0, min(re, r0 + Q.rcap), s0, min(se, s0 + Q.schunk));
        }
    }
}

// Output counter and range (first pair, capacity) of join j: its own for a batch of joins,
// the whole output otherwise.
template <bool BATCH, typename QP>
__device__ __forceinline__ unsigned long long *out_counter(const QP &Q, uint32_t j) {
    if constexpr (BATCH) return Q.out_counts + j;
    else return Q.out_count;
}
template <bool BATCH, typename QP>
__device__ __forceinline__ void out_range(const QP &Q, uint32_t j, unsigned long long *first, unsigned long long *cap) {
    if constexpr (BATCH) {
        *first = Q.out_begin[j];
        *cap = Q.out_begin[j + 1] - Q.out_begin[j];
    } else {
        *first = 0;
        *cap = Q.capacity;
    }
}

// ---- work items of a batch of joins
//
// Join j's build and probe rows after the pass are `parts` adjacent partitions on each side
// (a single one without a pass). Small joins need fewer: adjacent partitions are grouped,
// 2^k at a time, so a group holds about half a table of build rows -- rows of different
// partitions never match, so one table may hold several. Each group gives
// ceil(build rows / rcap) x ceil(probe rows / schunk) items.
struct BatchGroups {
    uint32_t groups, merge;
};
__device__ __forceinline__ BatchGroups batch_groups(const ProbeParams &Q, uint32_t parts, uint32_t j) {
    const uint32_t nr = Q.r_end[(size_t)j * parts + parts - 1] - Q.r_begin[(size_t)j * parts];
    const uint32_t half = Q.rcap / 2;
    const uint32_t want = (nr + half - 1) / half;
    uint32_t g = 1;
    while (g < want && g < parts) g <<= 1;
    return BatchGroups{g, parts / g};
}
__device__ __forceinline__ uint4 batch_group_rows(const ProbeParams &Q, uint32_t parts, uint32_t j, uint32_t g, uint32_t merge) {
    const size_t p0 = (size_t)j * parts + (size_t)g * merge, p1 = p0 + merge - 1;
    return make_uint4(Q.r_begin[p0], Q.r_end[p1], Q.s_begin[p0], Q.s_end[p1]);
}
__device__ __forceinline__ uint32_t batch_group_items(const ProbeParams &Q, const uint4 &d) {
    if (d.y <= d.x || d.w <= d.z) return 0;
    return ((d.y - d.x + Q.rcap - 1) / Q.rcap) * ((d.w - d.z + Q.schunk - 1) / Q.schunk);
}

// Join j by the whole block. COUNT: its items -> cnt[j]. !COUNT: its item descriptors from
// base[j] on (none past item_cap). s_warp: 32 words of block scratch.
template <bool COUNT>
__device__ __forceinline__ void batch_items_join(const ProbeParams &Q, uint32_t parts, uint32_t *cnt, const uint32_t *base, uint32_t j, uint32_t *s_warp) {
    const BatchGroups bg = batch_groups(Q, parts, j);
    uint32_t run = COUNT ? 0u : base[j];
    for (uint32_t g0 = 0; g0 < bg.groups; g0 += blockDim.x) {
        const uint32_t g = g0 + threadIdx.x;
        uint4 d = make_uint4(0, 0, 0, 0);
        uint32_t n = 0;
        if (g < bg.groups) {
            d = batch_group_rows(Q, parts, j, g, bg.merge);
            n = batch_group_items(Q, d);
        }
        uint32_t total = 0;
        const uint32_t excl = block_exclusive_scan<uint32_t>(n, s_warp, &total);
        if (!COUNT && n) {
            uint32_t k = run + excl;
            for (uint32_t r0 = d.x; r0 < d.y; r0 += Q.rcap) {
                for (uint32_t s0 = d.z; s0 < d.w; s0 += Q.schunk) {
                    if (k < Q.item_cap) {
                        Q.item_desc[k] = make_uint4(r0, min(d.y, r0 + Q.rcap), s0, min(d.w, s0 + Q.schunk));
                        Q.item_join[k] = j;
                    }
                    k++;
                }
            }
        }
        run += total;
        __syncthreads();
    }
    if (COUNT && threadIdx.x == 0) cnt[j] = run;
}

// Grid: one block per join.
template <bool COUNT>
__global__ void __launch_bounds__(256) batch_items_kernel(ProbeParams Q, uint32_t parts, uint32_t *cnt, const uint32_t *base) {
    __shared__ uint32_t s_warp[32];
    batch_items_join<COUNT>(Q, parts, cnt, base, blockIdx.x, s_warp);
}

// One block of PLAN_THREADS: item offset of every join, the item total, the counters reset.
// A batch with more items than item_desc holds is refused (error flag 2, no items).
__device__ __forceinline__ void batch_scan_block(const ProbeParams &Q, uint32_t *cnt_base) {
    __shared__ unsigned long long s_warp[32];
    const uint32_t per = (Q.joins + PLAN_THREADS - 1) / PLAN_THREADS;
    const uint32_t j0 = threadIdx.x * per;
    unsigned long long mine = 0;
    for (uint32_t j = j0; j < j0 + per && j < Q.joins; j++) mine += cnt_base[j];
    unsigned long long total = 0;
    unsigned long long run = block_exclusive_scan<unsigned long long>(mine, s_warp, &total);
    for (uint32_t j = j0; j < j0 + per && j < Q.joins; j++) {
        const uint32_t c = cnt_base[j];
        cnt_base[j] = (uint32_t)(run < 0xffffffffull ? run : 0xffffffffull);
        run += c;
        Q.out_counts[j] = 0;
    }
    if (threadIdx.x == 0) {
        const bool fits = total <= Q.item_cap;
        if (!fits) atomicOr(Q.error, 2u);
        Q.item_begin[Q.np] = fits ? (uint32_t)total : 0u;
        Q.item_begin[Q.np + 1] = 1u;
        *Q.ticket = 0;
        *Q.out_count = 0;
    }
}

static __global__ void __launch_bounds__(PLAN_THREADS) batch_scan_kernel(ProbeParams Q, uint32_t *cnt_base) { batch_scan_block(Q, cnt_base); }

template <int PB>
struct Pair;
template <>
struct Pair<4> {
    using T = uint2;
    static __device__ __forceinline__ T make(uint32_t a, uint32_t b) { return make_uint2(a, b); }
};
template <>
struct Pair<8> {
    using T = ulonglong2;
    static __device__ __forceinline__ T make(unsigned long long a, unsigned long long b) { return make_ulonglong2(a, b); }
};

// ------------------------------------------------------------------ probe kernel
//
// Persistent, one block per SM: PROBE_THREADS - 32 "consumer" threads build and probe, the
// last warp ("producer") runs up to two work items ahead of them and never probes.
//
//   producer, item k (buffer b = k & 1):
//     wait empty[b] (the consumers are done with item k - 2)
//     bulk-copy item k's build rows into rbuf[b]            (full[b]: arrival 1 + bytes)
//     flush item k - 2's staged pairs: one atomic on the output counter, one bulk store
//     publish item k's descriptor, clear its pair count     (full[b]: arrival 2)
//     claim item k + 1 by ticket, L2-prefetch its build and probe rows
//   consumers, item k:
//     wait full[b]; insert the build rows into table[b] (u16 slots: tag << 11 | row,
//     atomicCAS, the slot from a mix of the key: table_slot); load their first probe rows
//     into registers (without payloads for row-contiguous rows; in flight at the barrier)
//     named barrier over the consumers: the table is complete (the only block-level wait)
//     probe: rows straight from global memory, J per thread per round, matches staged per
//     item in stage[b] (one shared-memory reservation per warp and round)
//     arrive empty[b]
//
// Tables are cleared once every 31 uses: a slot belongs to the current item when its 5-bit
// tag equals the item's tag (the use count of the table buffer, mod 31, plus 1), so stale
// slots read as empty. Tables hold up to 2048 build rows at 8 slots per row by default
// (load <= 1/8): a warp walks as far as its longest probe sequence, and at load 1/2 that
// is about ten slots for a 32-lane miss. Staged pairs
// leave with one bulk store per item in the order of an atomic reservation; pairs past the
// stage's capacity (only when an item has more matches than it holds) are written directly
// with a per-warp reservation.

constexpr int PROBE_THREADS = 1024;
constexpr int PROBE_J = 5;  // probe rows per consumer thread per round (4960 per block)
constexpr uint32_t TAG_SHIFT = 11;  // table slot: tag << TAG_SHIFT | build row (rows < 2048)
constexpr uint32_t ROW_MASK = (1u << TAG_SHIFT) - 1;
constexpr uint32_t TAGS = 31;        // tags 1..31

template <int KW, int PB, int HS>
struct ProbeRow {
    Key<KW> key;
    typename PayloadType<PB>::T pay;
    uint64_t hash;
};

// Probe row s, straight from global memory (read once: streaming loads).
template <int KW, int PB, int HS, bool AOS>
__device__ __forceinline__ void load_probe_row(const ProbeParams &Q, uint32_t s, ProbeRow<KW, PB, HS> &r) {
    using L = Layout<KW, PB, HS>;
    using Pt = typename PayloadType<PB>::T;
    if (AOS) {
        const unsigned char *p = (const unsigned char *)Q.s_rows_in + (size_t)s * L::STRIDE;
        uint32_t w[L::STRIDE / 4];
        if (L::STRIDE % 16 == 0) {
#pragma unroll
            for (int o = 0; o < L::STRIDE / 16; o++) {
                const uint4 v = __ldcs((const uint4 *)p + o);
                w[4 * o] = v.x;
                w[4 * o + 1] = v.y;
                w[4 * o + 2] = v.z;
                w[4 * o + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int o = 0; o < L::STRIDE / 8; o++) {
                const uint2 v = __ldcs((const uint2 *)p + o);
                w[2 * o] = v.x;
                w[2 * o + 1] = v.y;
            }
        }
#pragma unroll
        for (int i = 0; i < KW; i++) r.key.w[i] = w[i];
        if (PB == 8) r.pay = (Pt)(((unsigned long long)w[L::PAY_OFF / 4 + 1] << 32) | w[L::PAY_OFF / 4]);
        else r.pay = (Pt)w[L::PAY_OFF / 4];
        if (HS == 8) r.hash = ((uint64_t)w[L::HASH_OFF / 4 + 1] << 32) | w[L::HASH_OFF / 4];
        else if (HS == 4) r.hash = w[L::HASH_OFF / 4];
        else r.hash = 0;
    } else {
        r.key = load_key_stream<KW>(Q.s_keys, s);
        r.pay = __ldcs((const Pt *)Q.s_pay + s);
        if (HS == 8) r.hash = __ldcs((const unsigned long long *)Q.s_hash + s);
        else if (HS == 4) r.hash = __ldcs((const uint32_t *)Q.s_hash + s);
        else r.hash = 0;
    }
}

// Probe rows in a row-contiguous buffer are loaded without their payload (key, and the hash
// where rows carry one), through L1 -- the probe walk needs nothing else; a matching row's
// payload is read from the same row when its pair is staged, mostly an L1 or L2 hit.
// Holding five rows' payloads in registers through the walk made the probe spill
// (2^27 x 2^29 int64 join's probe: 3.77 -> 3.61 ms).
template <int KW, int PB, int HS, bool AOS>
constexpr bool probe_key_only() {
    return AOS;
}
template <int KW, int PB, int HS>
__device__ __forceinline__ void load_probe_key(const ProbeParams &Q, uint32_t s, ProbeRow<KW, PB, HS> &r) {
    // rows are 8-byte aligned (their stride is a multiple of 8) and start with the key
    const unsigned char *p = (const unsigned char *)Q.s_rows_in + (size_t)s * Layout<KW, PB, HS>::STRIDE;
    if constexpr (KW % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KW / 2; i++) {
            const uint2 v = *((const uint2 *)p + i);
            r.key.w[2 * i] = v.x;
            r.key.w[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < KW; i++) r.key.w[i] = *((const uint32_t *)p + i);
    }
    r.pay = 0;
    if constexpr (HS == 8) r.hash = *(const unsigned long long *)(p + Layout<KW, PB, HS>::HASH_OFF);
    else if constexpr (HS == 4) r.hash = *(const uint32_t *)(p + Layout<KW, PB, HS>::HASH_OFF);
    else r.hash = 0;
}
template <int KW, int PB, int HS, bool AOS>
__device__ __forceinline__ void load_probe(const ProbeParams &Q, uint32_t s, ProbeRow<KW, PB, HS> &r) {
    if constexpr (probe_key_only<KW, PB, HS, AOS>()) load_probe_key<KW, PB, HS>(Q, s, r);
    else load_probe_row<KW, PB, HS, AOS>(Q, s, r);
}
// The payload of probe row s for its pair: from the row (key-only loads) or as loaded.
template <int KW, int PB, int HS, bool AOS>
__device__ __forceinline__ typename PayloadType<PB>::T probe_pay(const ProbeParams &Q, uint32_t s, const ProbeRow<KW, PB, HS> &r) {
    using L = Layout<KW, PB, HS>;
    if constexpr (probe_key_only<KW, PB, HS, AOS>()) return *(const typename PayloadType<PB>::T *)((const unsigned char *)Q.s_rows_in + (size_t)s * L::STRIDE + L::PAY_OFF);
    else return r.pay;
}

// Rows of work item `it`: build rows [x, y), probe rows [z, w) -- from the planner's
// descriptor, or (plans too large for the descriptor array) from a search of the prefix.
__device__ __forceinline__ uint4 item_rows(const ProbeParams &Q, uint32_t it, bool direct) {
    if (direct) return Q.item_desc[it];
    int lo = 0, hi = Q.np - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (Q.item_begin[mid] <= it) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t p = (uint32_t)lo;
    const uint32_t rb = Q.r_begin ? Q.r_begin[p] : 0, re = Q.r_begin ? Q.r_end[p] : Q.r_rows;
    const uint32_t sb = Q.s_begin ? Q.s_begin[p] : 0, se = Q.s_begin ? Q.s_end[p] : Q.s_rows;
    const uint32_t nsc = (se - sb + Q.schunk - 1) / Q.schunk;
    const uint32_t k = it - Q.item_begin[p];
    const uint32_t r0 = rb + (k / nsc) * Q.rcap;
    const uint32_t s0 = sb + (k % nsc) * Q.schunk;
    return make_uint4(r0, min(re, r0 + Q.rcap), s0, min(se, s0 + Q.schunk));
}

// Shared memory of the probe kernel (dynamic part): barriers, two build-row buffers, two
// tables, two output stages.
template <int KW, int PB, int HS, bool AOS>
struct ProbeSmem {
    using C = Chunk<KW, PB, HS, AOS>;
    using PT = typename Pair<PB>::T;
    __host__ __device__ static size_t rbuf_bytes(uint32_t rcap) { return (C::bytes(rcap) + 127) / 128 * 128; }
    __host__ __device__ static size_t bytes(uint32_t rcap, uint32_t tcap, uint32_t scap) {
        return 128 + 2 * rbuf_bytes(rcap) + 2 * (size_t)tcap * 2 + 2 * (size_t)scap * sizeof(PT);
    }
};

// Pairs of one warp's group of matches: lanes with `want` write `pair` at stage positions
// pos0 + (rank among the group); positions past the stage go straight to the output with
// their own reservation.
template <int PB, bool BATCH>
__device__ __forceinline__ void stage_pairs(const ProbeParams &Q, typename Pair<PB>::T *stage, uint32_t pos, bool want, const typename Pair<PB>::T &pair, uint32_t join, unsigned long long o_first,
                                            unsigned long long o_cap) {
    using PT = typename Pair<PB>::T;
    const bool over = want && pos >= Q.scap;
    const uint32_t ob = __ballot_sync(0xffffffffu, over);
    if (ob) {
        const int leader = __ffs(ob) - 1;
        unsigned long long g0 = 0;
        if ((int)(threadIdx.x & 31) == leader) g0 = atomicAdd(out_counter<BATCH>(Q, join), (unsigned long long)__popc(ob));
        g0 = __shfl_sync(0xffffffffu, g0, leader);
        if (over) {
            const unsigned long long g = g0 + __popc(ob & lanemask_lt());
            if (g < o_cap) ((PT *)Q.out)[o_first + g] = pair;
        }
    }
    if (want && !over) stage[pos] = pair;
}

// Producer: the n_staged pairs an item of join `join` staged in `stage` go to the output
// behind one reservation on the join's counter. Whole warp; n_staged and join are lane 0's
// values, the other lanes take them from it.
template <int PB, bool BATCH>
__device__ __forceinline__ void flush_stage(const ProbeParams &Q, const typename Pair<PB>::T *stage, uint32_t n_staged, uint32_t join) {
    using PT = typename Pair<PB>::T;
    const uint32_t lane = threadIdx.x & 31;
    join = __shfl_sync(0xffffffffu, join, 0);
    const uint32_t n = min(__shfl_sync(0xffffffffu, n_staged, 0), Q.scap);
    if (n == 0) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(out_counter<BATCH>(Q, join), (unsigned long long)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    unsigned long long first, cap;
    out_range<BATCH>(Q, join, &first, &cap);
    if (base >= cap) return;
    const uint32_t m = (uint32_t)min((unsigned long long)n, cap - base);
    PT *dst = (PT *)Q.out + first + base;
    if (sizeof(PT) == 16 && ((uintptr_t)dst & 15) == 0) {
        if (lane == 0) {
            bulk_s2g(dst, stage, m * 16u);
            bulk_commit();
            bulk_wait_read();
        }
    } else {
        for (uint32_t i = lane; i < m; i += 32) __stcs(dst + i, stage[i]);
    }
    __syncwarp();
}

// The probe by the whole block (blockDim.x threads, the last warp the producer) until the
// items run out; s_raw is the block's ProbeSmem bytes of dynamic shared memory. BATCH: a
// batch of joins; each item's pairs go to its join's output range.
template <int KW, int PB, int HS, bool AOS, bool BATCH>
__device__ __forceinline__ void probe_run(const ProbeParams &Q, unsigned char *s_raw) {
    using C = Chunk<KW, PB, HS, AOS>;
    using Pt = typename PayloadType<PB>::T;
    using PT = typename Pair<PB>::T;
    using SM = ProbeSmem<KW, PB, HS, AOS>;
    using Row = ProbeRow<KW, PB, HS>;
    constexpr int J = PROBE_J;
    uint64_t *full = (uint64_t *)s_raw;  // [2]: build rows landed + descriptor published
    uint64_t *empty = full + 2;          // [2]: consumers done with the item
    const size_t rbytes = SM::rbuf_bytes(Q.rcap);
    unsigned char *rbuf0 = s_raw + 128;
    uint16_t *tab0 = (uint16_t *)(rbuf0 + 2 * rbytes);
    PT *stage0 = (PT *)(tab0 + 2 * (size_t)Q.tcap);
    __shared__ uint4 s_desc[2];
    __shared__ uint32_t s_item[2], s_join[2], s_dups[2], s_out_n[2];
    __shared__ uint32_t s_rdelta[2][3];

    const uint32_t NC = blockDim.x - 32;  // consumer threads (a multiple of 32)
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = Q.item_begin[Q.np];
    const bool direct = Q.item_begin[Q.np + 1] != 0;

    if (threadIdx.x == 0) {
        mbar_init(&full[0], 2);
        mbar_init(&full[1], 2);
        mbar_init(&empty[0], NC / 32);
        mbar_init(&empty[1], NC / 32);
        s_out_n[0] = s_out_n[1] = 0;
        s_dups[0] = s_dups[1] = 0;
        fence_proxy_async();
    }
    for (uint32_t i = threadIdx.x; i < 2 * Q.tcap / 8; i += blockDim.x) ((uint4 *)tab0)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();

    if (warp == NC / 32) {
        // ---------------------------------------------------------------- producer warp
        const bool l0 = lane == 0;
        uint32_t t_cur = 0, t_nxt = 0, j_cur = 0;
        uint4 d_cur = make_uint4(0, 0, 0, 0);
        if (l0) {
            t_cur = atomicAdd(Q.ticket, 1u);
            if (t_cur < total) {
                d_cur = item_rows(Q, t_cur, direct);
                if constexpr (BATCH) j_cur = Q.item_join[t_cur];
                C::prefetch(Q.s_keys, Q.s_pay, Q.s_hash, Q.s_rows_in, d_cur.z, d_cur.w);
            }
            t_nxt = atomicAdd(Q.ticket, 1u);
        }
        uint32_t k = 0;
        bool ok = true;
        for (;; k++) {
            const uint32_t b = k & 1;
            if (k >= 2) {
                bool w = true;
                if (l0) w = mbar_wait(&empty[b], ((k - 2) >> 1) & 1);
                __syncwarp();  // the other lanes read the stage after lane 0's wait
                if (!__shfl_sync(0xffffffffu, (uint32_t)w, 0)) {
                    ok = false;
                    break;
                }
            }
            const bool valid = __shfl_sync(0xffffffffu, (uint32_t)(t_cur < total), 0) != 0;
            if (l0) {
                if (valid) {
                    fence_proxy_async();
                    C::issue(Q.r_keys, Q.r_pay, Q.r_hash, Q.r_rows_in, d_cur.x, d_cur.y, Q.rcap, rbuf0 + b * rbytes, &full[b], s_rdelta[b]);
                } else {
                    mbar_arrive(&full[b]);
                }
            }
            if (k >= 2) flush_stage<PB, BATCH>(Q, stage0 + (size_t)b * Q.scap, s_out_n[b], s_join[b]);
            if (l0) {
                s_item[b] = t_cur;
                s_desc[b] = d_cur;
                s_join[b] = j_cur;
                s_out_n[b] = 0;
                mbar_arrive(&full[b]);
            }
            if (!valid) break;
            if (l0) {
                t_cur = t_nxt;
                if (t_cur < total) {
                    d_cur = item_rows(Q, t_cur, direct);
                    if constexpr (BATCH) j_cur = Q.item_join[t_cur];
                    C::prefetch(Q.r_keys, Q.r_pay, Q.r_hash, Q.r_rows_in, d_cur.x, d_cur.y);
                    C::prefetch(Q.s_keys, Q.s_pay, Q.s_hash, Q.s_rows_in, d_cur.z, d_cur.w);
                }
                t_nxt = atomicAdd(Q.ticket, 1u);
            }
        }
        if (ok && k >= 1) {
            // the item before the end mark: its pairs are still staged
            const uint32_t b = (k - 1) & 1;
            bool w = true;
            if (l0) w = mbar_wait(&empty[b], ((k - 1) >> 1) & 1);
            __syncwarp();
            if (__shfl_sync(0xffffffffu, (uint32_t)w, 0)) flush_stage<PB, BATCH>(Q, stage0 + (size_t)b * Q.scap, s_out_n[b], s_join[b]);
            else ok = false;
        }
        if (l0) {
            if (!ok) atomicOr(Q.error, 4u);
            bulk_wait_all();
        }
        return;
    }

    // -------------------------------------------------------------------- consumer warps
    const uint32_t c = threadIdx.x;
    Row rows[J];
    for (uint32_t k = 0;; k++) {
        const uint32_t b = k & 1;
        const bool got = mbar_wait(&full[b], (k >> 1) & 1);
        const uint32_t item = got ? s_item[b] : 0xffffffffu;
        const bool stop = !got || item >= total;
        const uint32_t use = k >> 1;                  // uses of table b before this one
        const uint32_t tag = use % TAGS + 1u;         // 1..31
        uint16_t *T = tab0 + (size_t)b * Q.tcap;
        if (use > 0 && use % TAGS == 0) {
            // the tag wraps: clear the table (its last item finished before the previous
            // item's table barrier)
            for (uint32_t i = c; i < Q.tcap / 8; i += NC) ((uint4 *)T)[i] = make_uint4(0, 0, 0, 0);
            bar_sync(1, NC);
        }
        uint4 d = make_uint4(0, 0, 0, 0);
        uint32_t join = 0;
        if (!stop) {
            d = s_desc[b];
            if constexpr (BATCH) join = s_join[b];
        }
        const uint32_t nr = d.y - d.x, ns = d.w - d.z;
        uint32_t cap = 64;
        while (cap < nr * Q.tmul && cap < Q.tcap) cap <<= 1;
        const uint32_t cmask = cap - 1;
        const C R = C::view(rbuf0 + b * rbytes, Q.rcap, s_rdelta[b]);
        // ---- build: slot = tag << 11 | row; an equal key met on the way marks the item as
        // having duplicate build keys. Build rows go to the consumers in reverse order: the
        // rows past the first NC land on the last warps, while the probe rows past a whole
        // number of rounds land on the first ones, so no warp carries both extras to the
        // table barrier (4.81 -> 4.54 ms for the 2^27 x 2^29 join's probe).
        // one probe row's load before the build, the first round's others after it (below);
        // batches issue all five after it (the fused batch launch: 45.7 against 45.1 ms with
        // one before)
        if (!BATCH && c < ns) load_probe<KW, PB, HS, AOS>(Q, d.z + c, rows[0]);
        bool dup = false;
        for (uint32_t i = NC - 1 - c; i < nr; i += NC) {
            const Key<KW> key = R.key(i);
            uint32_t slot = table_slot<KW, HS>(key, HS ? R.hash(i) : 0ull, Q.slot_shift) & cmask;
            const unsigned short val = (unsigned short)((tag << TAG_SHIFT) | i);
            uint32_t cur = T[slot];
            for (uint32_t tries = 0;;) {
                if ((cur >> TAG_SHIFT) != tag) {
                    const uint32_t prev = atomicCAS((unsigned short *)&T[slot], (unsigned short)cur, val);
                    if (prev == cur) break;
                    cur = prev;
                    continue;
                }
                dup |= key_equal<KW>(R.key(cur & ROW_MASK), key);
                if (++tries > cap) {  // cannot happen: at most 1/tmul of the slots are used
                    atomicOr(Q.error, 1u);
                    break;
                }
                slot = (slot + 1) & cmask;
                cur = T[slot];
            }
        }
        if (dup) s_dups[b] = tag;
        // the rest of the first round of probe rows, issued after the build: they are in
        // flight during the table barrier, and the build does not wait behind ~5000 loads
        // queued at once (the 2^27 x 2^29 join's probe: all five before the build 4.33 ms,
        // all after 4.03; with key-only loads all after 3.604, one before 3.584, two 3.586,
        // three 3.66)
#pragma unroll
        for (int j = BATCH ? 0 : 1; j < J; j++) {
            const uint32_t i = c + (uint32_t)j * NC;
            if (i < ns) load_probe<KW, PB, HS, AOS>(Q, d.z + i, rows[j]);
        }
        if (bar_or(1, NC, stop)) {
            if (!got) atomicOr(Q.error, 4u);
            break;
        }
        const bool dups = s_dups[b] == tag;
        unsigned long long o_first, o_cap;  // this item's output range (direct writes)
        out_range<BATCH>(Q, join, &o_first, &o_cap);
        PT *stage = stage0 + (size_t)b * Q.scap;
        const uint32_t lt = lanemask_lt();

        for (uint32_t r0 = 0; r0 < ns; r0 += J * NC) {
            if (r0 > 0) {
#pragma unroll
                for (int j = 0; j < J; j++) {
                    const uint32_t i = r0 + c + (uint32_t)j * NC;
                    if (i < ns) load_probe<KW, PB, HS, AOS>(Q, d.z + i, rows[j]);
                }
            }
            if (!dups) {
                // Unique build keys: a probe row matches at most one build row. Every lane
                // resolves its J rows, then the warp stages all its matches behind one
                // shared-memory reservation.
                // (the ballots are taken again when staging rather than kept in an array:
                // fewer registers live across the reservation)
                int m[J];
                uint32_t cnt = 0;
#pragma unroll
                for (int j = 0; j < J; j++) {
                    m[j] = -1;
                    if (r0 + c + (uint32_t)j * NC < ns) {
                        const uint64_t h = HS ? rows[j].hash : 0ull;
                        uint32_t slot = table_slot<KW, HS>(rows[j].key, h, Q.slot_shift) & cmask;
                        for (uint32_t t = 0; t < cap; t++) {
                            const uint32_t e = T[slot];
                            if ((e >> TAG_SHIFT) != tag) break;
                            const uint32_t bi = e & ROW_MASK;
                            if (key_equal<KW>(R.key(bi), rows[j].key) && (!HS || R.hash(bi) == h)) {
                                m[j] = (int)bi;
                                break;
                            }
                            slot = (slot + 1) & cmask;
                        }
                    }
                    cnt += __popc(__ballot_sync(0xffffffffu, m[j] >= 0));
                }
                if (cnt) {
                    uint32_t pos0 = 0;
                    if (lane == 0) pos0 = atomicAdd(&s_out_n[b], cnt);
                    pos0 = __shfl_sync(0xffffffffu, pos0, 0);
                    if (pos0 + cnt <= Q.scap) {
                        // the warp's reservation fits the stage: no per-row overflow check
                        // (one per row and round cost the probe 4.66 against 4.37 ms)
#pragma unroll
                        for (int j = 0; j < J; j++) {
                            const uint32_t bj = __ballot_sync(0xffffffffu, m[j] >= 0);
                            if (m[j] >= 0) stage[pos0 + __popc(bj & lt)] = Pair<PB>::make(R.pay((uint32_t)m[j]), probe_pay<KW, PB, HS, AOS>(Q, d.z + r0 + c + (uint32_t)j * NC, rows[j]));
                            pos0 += __popc(bj);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < J; j++) {
                            const uint32_t bj = __ballot_sync(0xffffffffu, m[j] >= 0);
                            if (bj) {
                                const bool want = m[j] >= 0;
                                const PT pr = Pair<PB>::make(want ? R.pay((uint32_t)m[j]) : Pt(0), want ? probe_pay<KW, PB, HS, AOS>(Q, d.z + r0 + c + (uint32_t)j * NC, rows[j]) : Pt(0));
                                stage_pairs<PB, BATCH>(Q, stage, pos0 + __popc(bj & lt), want, pr, join, o_first, o_cap);
                                pos0 += __popc(bj);
                            }
                        }
                    }
                }
            } else {
                // Duplicate build keys: lanes walk their probe sequences in lock step and
                // stage every match, one reservation per warp and step.
#pragma unroll
                for (int j = 0; j < J; j++) {
                    bool active = r0 + c + (uint32_t)j * NC < ns;
                    uint64_t h = 0;
                    uint32_t slot = 0;
                    if (active) {
                        h = HS ? rows[j].hash : 0ull;
                        slot = table_slot<KW, HS>(rows[j].key, h, Q.slot_shift) & cmask;
                    }
                    uint32_t steps = 0;
                    while (__any_sync(0xffffffffu, active)) {
                        bool match = false;
                        Pt rp = 0;
                        if (active) {
                            const uint32_t e = T[slot];
                            if ((e >> TAG_SHIFT) != tag || ++steps > cap) {
                                active = false;
                            } else {
                                const uint32_t bi = e & ROW_MASK;
                                if (key_equal<KW>(R.key(bi), rows[j].key) && (!HS || R.hash(bi) == h)) {
                                    match = true;
                                    rp = R.pay(bi);
                                }
                                slot = (slot + 1) & cmask;
                            }
                        }
                        const uint32_t mb = __ballot_sync(0xffffffffu, match);
                        if (mb) {
                            uint32_t pos0 = 0;
                            if (lane == 0) pos0 = atomicAdd(&s_out_n[b], (uint32_t)__popc(mb));
                            pos0 = __shfl_sync(0xffffffffu, pos0, 0);
                            stage_pairs<PB, BATCH>(Q, stage, pos0 + __popc(mb & lt), match, Pair<PB>::make(rp, match ? probe_pay<KW, PB, HS, AOS>(Q, d.z + r0 + c + (uint32_t)j * NC, rows[j]) : Pt(0)), join, o_first, o_cap);
                        }
                    }
                }
            }
        }
        // staged pairs -> visible to the producer's bulk store; then hand the item back
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);
    }
}

template <int KW, int PB, int HS, bool AOS, bool BATCH>
__global__ void __launch_bounds__(PROBE_THREADS, 1) probe_kernel(ProbeParams Q) {
    extern __shared__ __align__(128) unsigned char s_raw[];
    probe_run<KW, PB, HS, AOS, BATCH>(Q, s_raw);
}


// ------------------------------------------------------------------ fused batch of joins
//
// A batch of joins as one persistent launch (cooperative: every block resident, one per
// SM, PROBE_THREADS threads): the phases of the separate launches run back to back inside
// the kernel, each over the whole grid, with a grid barrier between them --
//   segments      every join's row ranges, clamped into the tables (flag 16 if clamped)
//   plan          block 0: the output ranges made non-decreasing; the pass's unit plan
//   histogram     (one radix pass) the units' counts, the partition bounds
//   scatter       (one radix pass) rows into partitions, 4096-row tiles
//   items         per join: items counted; block 0: their offsets; per join: descriptors
//   probe         build and probe, pairs into each join's output range
// A block whose barrier wait runs out (WAIT_NS) sets error flag 64 and leaves; the others'
// waits then run out too, so the launch always ends.

// Row ranges of join j of a batch from the caller's offsets, each clamped into its table
// (and the output range into the output buffer) so that no later phase can leave its
// buffers; error flag 16 when an offset had to be clamped. j in [0, joins].
__device__ __forceinline__ void batch_segment(uint32_t j, uint32_t joins, const unsigned long long *ro, const unsigned long long *so, const unsigned long long *po, uint32_t r_rows,
                                              uint32_t s_rows, unsigned long long pair_cap, uint32_t *seg_begin, uint32_t *seg_end, unsigned long long *out_begin, uint32_t *error) {
    bool bad = false;
    auto clamp = [&](unsigned long long v, unsigned long long lo, unsigned long long hi) -> unsigned long long {
        const unsigned long long c = v < lo ? lo : (v > hi ? hi : v);
        bad |= c != v;
        return c;
    };
    // ranges start at 0, end at the table's rows and never decrease
    out_begin[j] = clamp(po[j], 0, pair_cap);
    if (j < joins) {
        const unsigned long long rb = j == 0 ? clamp(ro[0], 0, 0) : clamp(ro[j], 0, r_rows);
        const unsigned long long sb = j == 0 ? clamp(so[0], 0, 0) : clamp(so[j], 0, s_rows);
        const unsigned long long re = j + 1 == joins ? clamp(ro[j + 1], r_rows, r_rows) : clamp(ro[j + 1], rb, r_rows);
        const unsigned long long se = j + 1 == joins ? clamp(so[j + 1], s_rows, s_rows) : clamp(so[j + 1], sb, s_rows);
        bad |= po[j + 1] < po[j];
        seg_begin[j] = (uint32_t)rb;
        seg_end[j] = (uint32_t)(re < rb ? rb : re);
        seg_begin[joins + j] = (uint32_t)sb;
        seg_end[joins + j] = (uint32_t)(se < sb ? sb : se);
    }
    if (bad) atomicOr(error, 16u);
}

// Whole block: out_begin[0..joins] made non-decreasing (a running maximum).
__device__ __forceinline__ void out_monotone_block(uint32_t joins, unsigned long long *out_begin) {
    __shared__ unsigned long long s_max[32];
    const uint32_t n = joins + 1, per = (n + blockDim.x - 1) / blockDim.x, a = threadIdx.x * per;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    unsigned long long m = 0;
    for (uint32_t i = a; i < a + per && i < n; i++) m = max(m, out_begin[i]);
    // exclusive maximum over the threads before this one
    unsigned long long x = m;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane >= o) x = max(x, y);
    }
    if (lane == 31) s_max[warp] = x;
    __syncthreads();
    unsigned long long run = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) run = 0;
    for (uint32_t w = 0; w < warp && w < nwarps; w++) run = max(run, s_max[w]);
    for (uint32_t i = a; i < a + per && i < n; i++) {
        run = max(run, out_begin[i]);
        out_begin[i] = run;
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) { asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory"); }

// Grid barrier of a cooperative launch: words[0] counts arrivals (zero at launch, back to
// zero after every barrier), words[1] is the generation. False (error flag 64 set) when
// the wait ran out.
__device__ __forceinline__ bool grid_sync(uint32_t *words, uint32_t *error) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = true;
        const uint32_t gen = ld_acquire_u32(words + 1);
        __threadfence();  // this block's writes before its arrival
        if (atomicAdd(words, 1u) + 1u == gridDim.x) {
            words[0] = 0;
            __threadfence();
            st_release_u32(words + 1, gen + 1u);
        } else {
            const uint64_t t0 = global_ns();
            while (ld_acquire_u32(words + 1) == gen) {
                if (global_ns() - t0 > WAIT_NS) {
                    atomicOr(error, 64u);
                    ok = false;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

struct BatchFusedParams {
    PassParams P;   // the radix pass (passes == 1)
    ProbeParams Q;  // the probe; Q.error is the batch's error word
    uint32_t passes, joins, r_rows, s_rows, parts;
    const unsigned long long *ro, *so, *po;
    unsigned long long pair_cap;
    uint32_t *seg_begin, *seg_end;  // [2 * joins]: join rows per side
    unsigned long long *out_begin;  // [joins + 1]
    uint32_t *plan;                 // the pass's unit plan
    uint32_t *cnt;                  // [joins]: items per join, then their offsets
    uint32_t *sync;                 // grid barrier words (zero at launch)
};

// Dynamic shared memory the fused launch may take: the 227 KB a block may opt into, less
// room for the phases' static shared memory.
constexpr size_t FUSED_SMEM = 227 * 1024 - 4096;

// Rows per thread of the fused launch's scatter tiles: the largest of 4, 2, 1 whose tile
// fits FUSED_SMEM with the widest pass (2^MAX_RADIX_BITS buckets).
template <int KW, int PB, int HS>
constexpr int fused_scatter_items() {
    return ScatterSmem<KW, PB, HS, false, 4, PROBE_THREADS>::bytes(1u << MAX_RADIX_BITS) <= FUSED_SMEM   ? 4
           : ScatterSmem<KW, PB, HS, false, 2, PROBE_THREADS>::bytes(1u << MAX_RADIX_BITS) <= FUSED_SMEM ? 2
                                                                                                        : 1;
}

template <int KW, int PB, int HS, bool AOS>
__global__ void __launch_bounds__(PROBE_THREADS, 1) batch_fused_kernel(BatchFusedParams F) {
    static_assert(PLAN_THREADS == PROBE_THREADS, "the fused launch's blocks run the block-wide planners");
    constexpr int ITEMS = fused_scatter_items<KW, PB, HS>();
    extern __shared__ __align__(128) unsigned char s_raw[];
    __shared__ HistShared hsh;
    __shared__ ScatterShared ssh;
    __shared__ uint32_t s_w32[32];
    uint32_t *error = F.Q.error;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j <= F.joins; j += nthreads)
        batch_segment(j, F.joins, F.ro, F.so, F.po, F.r_rows, F.s_rows, F.pair_cap, F.seg_begin, F.seg_end, F.out_begin, error);
    if (!grid_sync(F.sync, error)) return;
    if (blockIdx.x == 0) {
        out_monotone_block(F.joins, F.out_begin);
        if (AOS) plan_block(F.seg_begin, F.seg_end, 2 * F.joins, (uint32_t)F.P.max_units, F.P.min_unit_rows, F.P.split, F.plan);
    }
    if (!grid_sync(F.sync, error)) return;
    if (AOS) {
        const uint32_t units = plan_total(F.P);
        for (uint32_t u = blockIdx.x; u < units; u += gridDim.x) {
            histogram_unit<KW, PB, HS, false, PROBE_THREADS>(F.P, u, (uint32_t *)s_raw, hsh);
            __syncthreads();
        }
        if (!grid_sync(F.sync, error)) return;
        fence_proxy_async();  // the histogram's shared memory is refilled by bulk copies next
        scatter_run<KW, PB, HS, false, true, ITEMS, PROBE_THREADS>(F.P, s_raw, ssh);
        if (!grid_sync(F.sync, error)) return;
    }
    for (uint32_t j = blockIdx.x; j < F.joins; j += gridDim.x) batch_items_join<true>(F.Q, F.parts, F.cnt, nullptr, j, s_w32);
    if (!grid_sync(F.sync, error)) return;
    if (blockIdx.x == 0) batch_scan_block(F.Q, F.cnt);
    if (!grid_sync(F.sync, error)) return;
    for (uint32_t j = blockIdx.x; j < F.joins; j += gridDim.x) batch_items_join<false>(F.Q, F.parts, nullptr, F.cnt, j, s_w32);
    if (!grid_sync(F.sync, error)) return;
    fence_proxy_async();  // likewise the scatter's, before the probe's bulk copies
    __syncthreads();
    probe_run<KW, PB, HS, AOS, true>(F.Q, s_raw);
}

// Host launch of the fused batch (csrc/vj_batch.cu): cooperative, `grid` blocks of
// PROBE_THREADS with `smem` bytes of dynamic shared memory.
template <int KW, int PB, int HS>
int batch_fused_launch(const BatchFusedParams &F, int grid, size_t smem, cudaStream_t stream);

// Dynamic shared memory of the fused batch: the largest phase's.
template <int KW, int PB, int HS>
size_t batch_fused_smem(uint32_t bins, size_t probe_smem) {
    const size_t sc = ScatterSmem<KW, PB, HS, false, fused_scatter_items<KW, PB, HS>(), PROBE_THREADS>::bytes(bins);
    size_t m = probe_smem > sc ? probe_smem : sc;
    return m > (size_t)bins * 4 ? m : (size_t)bins * 4;
}

}  // namespace vj
