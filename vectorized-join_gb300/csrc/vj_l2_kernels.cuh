// vj_l2_kernels.cuh -- build/probe against per-partition tables that live in L2.
//
// After one radix pass a partition of the build side holds ~2^17 rows: too many for a
// shared-memory table, few enough that its table (8-byte slots, load <= 1/3) and its rows
// stay in the 129 MB L2 while the partition's probe rows stream past. This replaces the
// second radix pass of the shared-memory design: the probe side is read once after the
// first pass, and table accesses are L2 hits (random 8-byte L2 loads run at ~300 G/s on
// GB300, against ~45 G/s from HBM).
//
// Work is a sequence of "seqs": a seq is one build chunk (<= rc rows of one partition)
// together with all probe rows of that partition. Each seq owns one region of a ring of
// `ring` tables. A persistent, cooperatively launched kernel takes work items from a
// ticket in this order:
//     B(0) .. B(lag-1) | B(lag) P(0) | B(lag+1) P(1) | ...      (group g = B(g), P(g-lag))
// where B(q) are the build items of seq q and P(q) its probe items. A probe item waits
// until every build item of its seq is done; a build item waits until every probe item of
// the seq that used its ring region before (q - ring) is done. Both wait only for items
// with smaller tickets, all blocks are resident (cooperative launch), so the waits end;
// they are bounded anyway and report error bit 4 if they run out.
//
// Slot format: [tag:16 | fingerprint:16 | row:32]. tag = 1 + q / ring differs between the
// successive users of a region, so a slot whose tag is not the current seq's reads as
// empty: regions are cleared once per join, not per seq. row is the build row's offset in
// the seq's chunk; the fingerprint (16 hash bits not used for the partition or the slot)
// skips most key comparisons of rows that only share a slot.
//
// The reference builds chained tables in shared memory per bucket pair
// (src/join/join_provider.cu:382-442) after enough radix passes to make every bucket fit
// 48 KB (src/join/join_provider.cuh:566-715).
#pragma once

#include "vj_join_kernels.cuh"

namespace vj {

constexpr int L2_THREADS = 512;
constexpr int L2_WARPS = L2_THREADS / 32;
constexpr int L2_U = 4;                  // probe rows per lane in flight
constexpr int L2_BUILD_U = 4;            // build rows per thread in flight
constexpr uint32_t L2_WARP_STAGE = 256;  // staged output pairs per warp
constexpr uint32_t L2_WALK_LIMIT = 512;  // slots an insert may pass before it calls the seq degenerate

struct L2Params {
    const void *r_rows, *s_rows;       // row-contiguous partition buffers
    const uint32_t *r_begin, *r_end;   // [np] partition bounds (rows)
    const uint32_t *s_begin, *s_end;
    int np;
    int part_bits;                     // hash bits consumed by the partition pass
    uint32_t rc;                       // build rows per seq at most
    uint32_t build_rows, probe_rows;   // rows per work item
    int ring;                          // table regions
    int lag;                           // groups between a seq's build items and its probe items
    uint32_t region_slots;             // slots per region (a power of two >= 3 * rc)
    unsigned long long *tables;        // [ring * region_slots]
    uint4 *seq;                        // [max_seqs]: build rows [x, y), probe rows [z, w)
    uint32_t *group_start;             // [max_seqs + lag + 1]: first ticket of each group
    uint4 *items;                      // [item_cap]: (seq | probe << 31, first row, end row, 0)
    uint32_t item_cap;
    uint32_t *built, *probed;          // [max_seqs]: finished build / probe items
    uint32_t *nseq;                    // [0] seqs, [1] work items, [2] 1: items[] is filled
    uint32_t max_seqs;
    uint32_t *ticket;
    unsigned long long *out_count;
    void *out;
    unsigned long long capacity;
    uint32_t outcap;                   // unused (per-warp staging of L2_WARP_STAGE pairs)
    HashSpec hs;
    uint32_t *error;                   // 2: plan too large, 4: a wait ran out, 8: degenerate seq
};

__host__ __device__ __forceinline__ uint32_t l2_items(uint32_t rows, uint32_t per) { return (rows + per - 1) / per; }

// Table capacity of a seq with n build rows: a power of two >= 3n (load <= 1/3).
__host__ __device__ __forceinline__ uint32_t l2_cap(uint32_t n) {
    uint32_t c = 64;
    while (c < 3 * n) c <<= 1;
    return c;
}

__device__ __forceinline__ uint32_t l2_fingerprint(uint64_t h) { return (uint32_t)(h ^ (h >> 29) ^ (h >> 47)) & 0xffffu; }

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Spin (one thread) until *p >= want; false if the bounded wait ran out.
__device__ __forceinline__ bool l2_wait_count(const uint32_t *p, uint32_t want) {
    uint32_t ns = 32;
    for (uint32_t i = 0; i < (1u << 22); i++) {
        if (ld_acquire_u32(p) >= want) return true;
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
    }
    return false;
}

// L2 policy for table slots: keep them over the streaming probe rows.
__device__ __forceinline__ uint64_t l2_policy_keep() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ unsigned long long slot_load(const unsigned long long *a, uint64_t pol) {
    unsigned long long v;
    asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol) : "memory");
    return v;
}

// (atom.cas takes no L2 cache hint; the hinted loads of the probe mark the lines)
__device__ __forceinline__ unsigned long long slot_cas(unsigned long long *a, unsigned long long cmp, unsigned long long val, uint64_t) { return atomicCAS(a, cmp, val); }

// One row of a row-contiguous buffer in registers, as 32-bit words.
template <int KW, int PB, int HS>
struct GRow {
    using L = Layout<KW, PB, HS>;
    using P = typename PayloadType<PB>::T;
    static constexpr int WORDS = L::STRIDE / 4;
    uint32_t w[WORDS];
    template <bool STREAM>
    __device__ __forceinline__ void load(const void *base, uint64_t i) {
        const unsigned char *p = (const unsigned char *)base + i * L::STRIDE;
        if constexpr (L::STRIDE % 16 == 0) {
#pragma unroll
            for (int o = 0; o < L::STRIDE / 16; o++) {
                const uint4 v = STREAM ? __ldcs((const uint4 *)p + o) : __ldg((const uint4 *)p + o);
                w[4 * o] = v.x;
                w[4 * o + 1] = v.y;
                w[4 * o + 2] = v.z;
                w[4 * o + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int o = 0; o < L::STRIDE / 8; o++) {
                const uint2 v = STREAM ? __ldcs((const uint2 *)p + o) : __ldg((const uint2 *)p + o);
                w[2 * o] = v.x;
                w[2 * o + 1] = v.y;
            }
        }
    }
    __device__ __forceinline__ Key<KW> key() const {
        Key<KW> k;
#pragma unroll
        for (int i = 0; i < KW; i++) k.w[i] = w[i];
        return k;
    }
    __device__ __forceinline__ P pay() const {
        if constexpr (PB == 8) return (P)w[L::PAY_OFF / 4] | ((P)w[L::PAY_OFF / 4 + 1] << 32);
        else return w[L::PAY_OFF / 4];
    }
    __device__ __forceinline__ uint64_t hash() const {
        if constexpr (HS == 8) return (uint64_t)w[L::HASH_OFF / 4] | ((uint64_t)w[L::HASH_OFF / 4 + 1] << 32);
        else if constexpr (HS == 4) return w[L::HASH_OFF / 4];
        else return 0;
    }
};

// One block. Seqs of every partition, the ticket offset of every group, the work items
// (when they fit items[]), counters reset.
__global__ void __launch_bounds__(PLAN_THREADS) l2_plan_kernel(L2Params Q) {
    __shared__ unsigned long long s_warp64[32];
    // ---- seqs: ceil(build rows / rc) per partition that has rows on both sides
    const int per = (Q.np + PLAN_THREADS - 1) / PLAN_THREADS;
    const int p0 = threadIdx.x * per;
    unsigned long long mine = 0;
    for (int p = p0; p < p0 + per && p < Q.np; p++) {
        const uint32_t nr = Q.r_end[p] - Q.r_begin[p], ns = Q.s_end[p] - Q.s_begin[p];
        if (nr && ns) mine += (nr + Q.rc - 1) / Q.rc;
    }
    unsigned long long nseq = 0;
    unsigned long long q = block_exclusive_scan<unsigned long long>(mine, s_warp64, &nseq);
    if (nseq > Q.max_seqs) {
        if (threadIdx.x == 0) {
            atomicOr(Q.error, 2u);
            Q.nseq[0] = Q.nseq[1] = Q.nseq[2] = 0;
            *Q.ticket = 0;
            *Q.out_count = 0;
        }
        return;
    }
    for (int p = p0; p < p0 + per && p < Q.np; p++) {
        const uint32_t rb = Q.r_begin[p], re = Q.r_end[p], sb = Q.s_begin[p], se = Q.s_end[p];
        if (rb == re || sb == se) continue;
        for (uint32_t r = rb; r < re; r += Q.rc) {
            Q.seq[q] = make_uint4(r, min(re, r + Q.rc), sb, se);
            Q.built[q] = 0;
            Q.probed[q] = 0;
            q++;
        }
    }
    __syncthreads();
    // ---- groups: g holds the build items of seq g and the probe items of seq g - lag
    const uint32_t ns_ = (uint32_t)nseq;
    const uint32_t G = ns_ + (uint32_t)Q.lag;
    const uint32_t gper = (G + PLAN_THREADS - 1) / PLAN_THREADS;
    const uint32_t g0 = threadIdx.x * gper;
    auto builds = [&](uint32_t g) -> uint32_t {
        if (g >= ns_) return 0;
        const uint4 d = Q.seq[g];
        return l2_items(d.y - d.x, Q.build_rows);
    };
    auto probes = [&](uint32_t g) -> uint32_t {
        if (g < (uint32_t)Q.lag || g - Q.lag >= ns_) return 0;
        const uint4 d = Q.seq[g - Q.lag];
        return l2_items(d.w - d.z, Q.probe_rows);
    };
    unsigned long long gm = 0;
    for (uint32_t g = g0; g < g0 + gper && g < G; g++) gm += builds(g) + probes(g);
    unsigned long long items = 0;
    unsigned long long run = block_exclusive_scan<unsigned long long>(gm, s_warp64, &items);
    const bool fail = items >= (1ull << 31);
    const bool fill = !fail && items <= Q.item_cap;
    for (uint32_t g = g0; g < g0 + gper && g < G; g++) {
        Q.group_start[g] = (uint32_t)run;
        const uint32_t nb = builds(g), np = probes(g);
        if (fill) {
            if (nb) {
                const uint4 d = Q.seq[g];
                for (uint32_t k = 0; k < nb; k++) {
                    const uint32_t a = d.x + k * Q.build_rows;
                    Q.items[run + k] = make_uint4(g, a, min(d.y, a + Q.build_rows), 0u);
                }
            }
            if (np) {
                const uint4 d = Q.seq[g - Q.lag];
                for (uint32_t k = 0; k < np; k++) {
                    const uint32_t a = d.z + k * Q.probe_rows;
                    Q.items[run + nb + k] = make_uint4((g - Q.lag) | 0x80000000u, a, min(d.w, a + Q.probe_rows), 0u);
                }
            }
        }
        run += nb + np;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (fail) atomicOr(Q.error, 2u);
        Q.group_start[G] = fail ? 0u : (uint32_t)items;
        Q.nseq[0] = fail ? 0u : ns_;
        Q.nseq[1] = fail ? 0u : (uint32_t)items;
        Q.nseq[2] = fill ? 1u : 0u;
        *Q.ticket = 0;
        *Q.out_count = 0;
    }
}

// Work item t as (seq | probe << 31, first row, end row): from items[], or (plans larger
// than items[]) from a search of the group offsets.
__device__ __forceinline__ uint4 l2_item(const L2Params &Q, uint32_t t, uint32_t nseq, bool direct) {
    if (direct) return Q.items[t];
    const uint32_t G = nseq + (uint32_t)Q.lag;
    uint32_t lo = 0, hi = G - 1;
    while (lo < hi) {  // last group starting at or before t
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (Q.group_start[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t g = lo;
    uint32_t o = t - Q.group_start[g];
    uint32_t nb = 0;
    if (g < nseq) {
        const uint4 d = Q.seq[g];
        nb = l2_items(d.y - d.x, Q.build_rows);
        if (o < nb) {
            const uint32_t a = d.x + o * Q.build_rows;
            return make_uint4(g, a, min(d.y, a + Q.build_rows), 0u);
        }
    }
    o -= nb;
    const uint32_t q = g - Q.lag;
    const uint4 d = Q.seq[q];
    const uint32_t a = d.z + o * Q.probe_rows;
    return make_uint4(q | 0x80000000u, a, min(d.w, a + Q.probe_rows), 0u);
}

// Copy a warp's staged pairs to the output: one reservation for the warp.
template <int PB, typename PT>
__device__ __forceinline__ void l2_warp_flush(const L2Params &Q, const PT *stage, uint32_t n, int lane) {
    __syncwarp();
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(Q.out_count, (unsigned long long)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    PT *out = (PT *)Q.out;
    for (uint32_t i = lane; i < n; i += 32) {
        if (base + i < Q.capacity) __stcs(out + base + i, stage[i]);
    }
    __syncwarp();
}

template <int KW, int PB, int HS>
__global__ void __launch_bounds__(L2_THREADS) l2_join_kernel(L2Params Q) {
    using R = GRow<KW, PB, HS>;
    using L = Layout<KW, PB, HS>;
    using PT = typename Pair<PB>::T;
    using Pt = typename PayloadType<PB>::T;
    constexpr int U = L2_U;
    constexpr int BU = L2_BUILD_U;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PT *stage = (PT *)s_raw + (size_t)warp * L2_WARP_STAGE;  // this warp's staged pairs
    uint32_t staged = 0;                                      // warp-uniform

    __shared__ uint4 s_it, s_next;
    __shared__ uint32_t s_next_t;
    __shared__ uint32_t s_ok;
    const uint32_t nseq = Q.nseq[0];
    const uint32_t total = Q.nseq[1];
    const bool direct = Q.nseq[2] != 0;
    const uint64_t keep = l2_policy_keep();
    if (threadIdx.x == 0) {
        s_next_t = total ? atomicAdd(Q.ticket, 1u) : 0u;
        if (s_next_t < total) s_next = l2_item(Q, s_next_t, nseq, direct);
    }
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t t = s_next_t;
            const uint4 it = s_next;
            s_it = it;
            s_ok = t < total ? 1u : 0u;
            if (t < total) {
                // claim and resolve the next item now; its rows start moving into L2
                s_next_t = atomicAdd(Q.ticket, 1u);
                if (s_next_t < total) {
                    const uint4 nx = l2_item(Q, s_next_t, nseq, direct);
                    s_next = nx;
                    const ColWindow w = col_window((nx.x >> 31) ? Q.s_rows : Q.r_rows, L::STRIDE, nx.y, nx.z);
                    bulk_prefetch_l2(w.src, w.bytes);
                }
                // dependencies of this item
                const uint32_t q = it.x & 0x7fffffffu;
                bool ok = true;
                if (it.x >> 31) {
                    const uint4 d = Q.seq[q];
                    ok = l2_wait_count(&Q.built[q], l2_items(d.y - d.x, Q.build_rows));
                } else if (q >= (uint32_t)Q.ring) {
                    const uint4 d = Q.seq[q - Q.ring];
                    ok = l2_wait_count(&Q.probed[q - Q.ring], l2_items(d.w - d.z, Q.probe_rows));
                }
                if (!ok) {
                    atomicOr(Q.error, 4u);
                    s_ok = 0;
                }
            }
        }
        __syncthreads();
        if (!s_ok) break;
        const uint4 it = s_it;
        const bool probe = (it.x >> 31) != 0;
        const uint32_t q = it.x & 0x7fffffffu;
        const uint4 sq = Q.seq[q];
        const uint32_t cap = l2_cap(sq.y - sq.x);
        const uint32_t cmask = cap - 1;
        const int cap_bits = 31 - __clz(cap);
        const unsigned long long tag = 1ull + q / (uint32_t)Q.ring;
        unsigned long long *T = Q.tables + (size_t)(q % (uint32_t)Q.ring) * Q.region_slots;
        const int pb = Q.part_bits;
        auto slot_of = [&](uint64_t mixed) -> uint32_t { return (uint32_t)((mixed << pb) >> (64 - cap_bits)) & cmask; };

        if (!probe) {
            // ---- build rows [y, z) of the seq's chunk: BU rows per thread in flight
            for (uint32_t i0 = it.y + threadIdx.x; i0 < it.z; i0 += BU * blockDim.x) {
                uint32_t slot[BU];
                unsigned long long val[BU], prev[BU];
                bool act[BU];
#pragma unroll
                for (int u = 0; u < BU; u++) {
                    const uint32_t i = i0 + u * blockDim.x;
                    act[u] = i < it.z;
                    slot[u] = 0;
                    val[u] = 0;
                    if (act[u]) {
                        R row;
                        row.template load<false>(Q.r_rows, i);
                        const uint64_t h = HS ? row.hash() : row_hash<KW>(row.key(), Q.hs);
                        slot[u] = slot_of(mix_hash(h));
                        val[u] = (tag << 48) | ((unsigned long long)l2_fingerprint(h) << 32) | (unsigned long long)(i - sq.x);
                    }
                }
#pragma unroll
                for (int u = 0; u < BU; u++) prev[u] = act[u] ? slot_cas(&T[slot[u]], 0ull, val[u], keep) : 0ull;
#pragma unroll
                for (int u = 0; u < BU; u++) {
                    if (!act[u] || prev[u] == 0ull) continue;
                    // the home slot was taken or stale: walk on
                    unsigned long long e = prev[u];
                    uint32_t sl = slot[u], walk = 0;
                    for (;;) {
                        if ((e >> 48) == tag) {
                            if (++walk > L2_WALK_LIMIT) {
                                atomicOr(Q.error, 8u);  // long cluster: duplicate-heavy or degenerate hash
                                break;
                            }
                            sl = (sl + 1) & cmask;
                            e = slot_load(&T[sl], keep);
                            continue;
                        }
                        const unsigned long long p = slot_cas(&T[sl], e, val[u], keep);
                        if (p == e) break;
                        e = p;
                    }
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(&Q.built[q], 1u);
            }
            continue;
        }

        // ---- probe rows [y, z): each warp takes a contiguous slice; lanes walk U rows'
        // clusters in lock step and the warp stages its matches
        const uint32_t n = it.z - it.y;
        const uint32_t per_warp = (n + L2_WARPS - 1) / L2_WARPS;
        const uint32_t wb = it.y + min(n, warp * per_warp), we = it.y + min(n, (warp + 1) * per_warp);
        for (uint32_t base = wb; base < we; base += 32 * U) {
            R srow[U];
            uint64_t sh[U];
            uint32_t slot[U], fp[U];
            bool act[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint32_t i = base + u * 32 + lane;
                act[u] = i < we;
                sh[u] = 0;
                slot[u] = 0;
                fp[u] = 0;
                if (act[u]) srow[u].template load<true>(Q.s_rows, i);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (act[u]) {
                    sh[u] = HS ? srow[u].hash() : row_hash<KW>(srow[u].key(), Q.hs);
                    slot[u] = slot_of(mix_hash(sh[u]));
                    fp[u] = l2_fingerprint(sh[u]);
                }
            }
            bool any = false;
#pragma unroll
            for (int u = 0; u < U; u++) any |= act[u];
            while (__any_sync(0xffffffffu, any)) {
                unsigned long long e[U];
#pragma unroll
                for (int u = 0; u < U; u++) e[u] = act[u] ? slot_load(&T[slot[u]], keep) : 0ull;
                bool cand[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (act[u] && (e[u] >> 48) != tag) act[u] = false;  // end of the cluster
                    cand[u] = act[u] && ((uint32_t)(e[u] >> 32) & 0xffffu) == fp[u];
                    slot[u] = (slot[u] + 1) & cmask;
                }
                R rrow[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (cand[u]) rrow[u].template load<false>(Q.r_rows, (uint64_t)sq.x + (uint32_t)e[u]);
                }
                bool m[U];
                uint32_t bal[U];
                uint32_t tot = 0;
#pragma unroll
                for (int u = 0; u < U; u++) {
                    m[u] = cand[u] && key_equal<KW>(rrow[u].key(), srow[u].key()) && (!HS || rrow[u].hash() == sh[u]);
                    bal[u] = __ballot_sync(0xffffffffu, m[u]);
                    tot += __popc(bal[u]);
                }
                if (tot) {
                    if (staged + tot > L2_WARP_STAGE) {
                        l2_warp_flush<PB>(Q, stage, staged, lane);
                        staged = 0;
                    }
                    const uint32_t lt = lanemask_lt();
                    uint32_t before = staged;
#pragma unroll
                    for (int u = 0; u < U; u++) {
                        if (m[u]) stage[before + __popc(bal[u] & lt)] = Pair<PB>::make((Pt)rrow[u].pay(), (Pt)srow[u].pay());
                        before += __popc(bal[u]);
                    }
                    staged += tot;
                }
                any = false;
#pragma unroll
                for (int u = 0; u < U; u++) any |= act[u];
            }
            if (staged >= L2_WARP_STAGE / 2) {
                l2_warp_flush<PB>(Q, stage, staged, lane);
                staged = 0;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&Q.probed[q], 1u);
        }
    }
    if (staged) l2_warp_flush<PB>(Q, stage, staged, lane);
}

}  // namespace vj
