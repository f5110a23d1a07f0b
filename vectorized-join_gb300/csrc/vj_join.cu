// vj_join.cu -- host orchestration of the join path: planning, workspace carving and the
// kernel sequence of vj_join / vj_partition / vj_build_probe / vj_join_host.
//
// The reference drives its pipeline from host threads: one std::thread per bucket and
// level (src/join/join_provider.cuh:566-715), a host synchronisation per partition level
// (:595) and per bucket pair (src/join/join_provider.cu:803), and a |R_b|*|S_b| probe
// buffer per pair (:694). Here one stream carries a fixed sequence of launches; every
// decision that depends on data (unit split, partition bounds, work items) is made on
// the device, and the host synchronises once, to read the match count.
#include "vj_join_kernels.cuh"

#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <tuple>

namespace vj {

namespace {

// ------------------------------------------------------------------ workspace carving

struct Carver {
    char *base = nullptr;
    size_t off = 0;
    template <typename T>
    T *take(size_t count, size_t align = 256) {
        off = (off + align - 1) / align * align;
        T *p = base ? (T *)(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

// ------------------------------------------------------------------ plan

struct Plan {
    int passes = 0;
    int bits[2] = {0, 0};
    uint32_t rcap = 2048;     // build rows per table
    uint32_t schunk = 8192;   // probe rows per work item
    uint32_t tmul = 2;        // table slots per build row (load <= 1/tmul)
    uint32_t tcap = 4096;     // table slots per table buffer
    uint32_t scap = 4096;     // staged output pairs per item
    int threads = PROBE_THREADS;  // probe block size (one producer warp + consumers)
    int max_units[2] = {0, 0};
};

int ceil_log2(uint64_t x) {
    int b = 0;
    while ((1ull << b) < x) b++;
    return b;
}

// Shared memory the probe block may use (one block per SM), minus its static shared memory.
size_t probe_smem_budget(const DeviceInfo &info) {
    const size_t per_block = info.smem_optin ? info.smem_optin : 48 * 1024;
    return per_block > 1024 ? per_block - 1024 : per_block;
}

// Table slots per build row for a requested load (percent): 2, 4 or 8 (0: 8, load <= 1/8).
uint32_t table_mul(int load_pct) {
    if (load_pct <= 0) return 8;
    uint32_t m = 2;
    while (m < 8 && (int)(100 / m) > load_pct) m <<= 1;
    return m;
}

// Units of a pass over `rows` rows in G segments: at most 48 per SM (short units keep the
// SMs busy as blocks finish, but each unit publishes a look-back word per bucket; on the
// 2^27 x 2^29 join 48 per SM took 15.71 ms against 15.80 with 64 and 15.74 with 32, and 16
// per SM, before the pass tails were cut in quarter units, 0.26 ms more than 64), none
// shorter than MIN_UNIT_ROWS, and one more per segment (every segment has a unit, whose
// block writes the segment's bounds).
constexpr uint32_t MIN_UNIT_ROWS = 4096;
// Whole units cut in four at the end of a join's pass: two for each SM, so that the blocks
// finishing the pass (two scatter blocks per SM) take quarter units.
uint32_t tail_split(const DeviceInfo &info) { return 2u * (uint32_t)info.sms; }
// split: the plan's whole units cut in four at its end (each adds three units)
int pass_units(const DeviceInfo &info, uint64_t rows, int G, uint32_t split = 0) {
    const uint64_t by_rows = (rows + MIN_UNIT_ROWS - 1) / MIN_UNIT_ROWS;
    const uint64_t cap = (uint64_t)info.sms * 48;
    return (int)((by_rows < cap ? by_rows : cap) + (uint64_t)G + 1 + 3ull * split);
}

// The unit plan of a pass over one or two whole tables (plan_block's rule, on the host).
void host_plan(PassParams &P, const uint32_t *rows, int nsides) {
    uint64_t total = 0;
    for (int sd = 0; sd < nsides; sd++) total += rows[sd];
    const uint64_t reserved = (uint64_t)nsides + 3ull * P.split;
    const uint64_t room = (uint64_t)P.max_units > reserved ? (uint64_t)P.max_units - reserved : 1ull;
    uint64_t t = (total + room - 1) / room;
    if (t < P.min_unit_rows) t = P.min_unit_rows;
    if (t < 1) t = 1;
    const uint32_t target = (uint32_t)(t < 0x7fffffffull ? t : 0x7fffffffull);
    uint32_t first[3] = {0, 0, 0};
    for (int sd = 0; sd < nsides; sd++) {
        const uint32_t n = rows[sd] ? (uint32_t)((rows[sd] + (uint64_t)target - 1) / target) : 1u;
        first[1 + sd] = first[sd] + n;
    }
    const uint32_t units = first[nsides];
    const uint32_t from = units - std::min(P.split, units / 4);
    P.plan = nullptr;
    P.hplan[0] = target;
    for (int g = 0; g <= nsides; g++) P.hplan[1 + g] = split_index(first[g], from);
    P.hplan[2 + nsides] = from;
}

template <int KW, int PB, int HS>
Plan make_plan(uint64_t nr, uint64_t ns, const DeviceInfo &info, const vj_join_options *opt) {
    using SMf = ProbeSmem<KW, PB, HS, true>;  // row-contiguous chunks are never smaller than columnar ones
    using PT = typename Pair<PB>::T;
    Plan pl;
    if (opt && opt->probe_threads > 0) {
        int t = opt->probe_threads / 32 * 32;
        pl.threads = t < 64 ? 64 : (t > PROBE_THREADS ? PROBE_THREADS : t);
    }
    pl.tmul = table_mul(opt ? opt->table_load_pct : 0);
    const size_t budget = probe_smem_budget(info);
    // largest build chunk (a power of two, at most 2048: table slots hold 11-bit rows) whose
    // buffers, tables and a stage of one pair per build row fit one block
    pl.rcap = 64;
    for (uint32_t rcap = 2048; rcap >= 64; rcap >>= 1) {
        uint32_t tcap = 64;
        while (tcap < rcap * pl.tmul) tcap <<= 1;
        if (tcap <= (1u << SLOT_BITS) && SMf::bytes(rcap, tcap, rcap) <= budget) {
            pl.rcap = rcap;
            break;
        }
    }
    if (opt && opt->build_rows > 0) {
        uint32_t want = 64;
        while (want < (uint32_t)opt->build_rows && want < pl.rcap) want <<= 1;
        pl.rcap = want;
    }
    pl.tcap = 64;
    while (pl.tcap < pl.rcap * pl.tmul) pl.tcap <<= 1;
    // the stage takes the rest of the block's shared memory
    const size_t fixed = SMf::bytes(pl.rcap, pl.tcap, 0);
    const size_t room = budget > fixed ? (budget - fixed) / (2 * sizeof(PT)) : 0;
    pl.scap = (uint32_t)std::min<size_t>(room, 16384);
    if (opt && opt->probe_rows > 0) pl.schunk = (uint32_t)std::max(32, opt->probe_rows);
    // passes / bits: the average build partition should fill about half a table
    int total_bits = 0;
    if (nr > pl.rcap) {
        total_bits = ceil_log2((nr + pl.rcap / 2 - 1) / (pl.rcap / 2));
    }
    // A probe side much smaller than the build side is cheaper to stream against
    // every build chunk than to partition: cost in probe steps.
    const uint64_t chunks0 = (nr + pl.rcap - 1) / pl.rcap;
    if (total_bits > 0 && chunks0 * ns <= 2 * (nr + ns)) total_bits = 0;
    if (total_bits > 2 * MAX_RADIX_BITS) total_bits = 2 * MAX_RADIX_BITS;
    if (total_bits == 0) {
        pl.passes = 0;
    } else if (total_bits <= 10) {
        pl.passes = 1;
        pl.bits[0] = total_bits;
    } else {
        pl.passes = 2;
        // the first pass scatters over the whole table, the second within small segments:
        // give the extra bit to the second
        pl.bits[0] = total_bits / 2;
        pl.bits[1] = total_bits - pl.bits[0];
    }
    if (opt && (opt->flags & VJ_JOIN_FIXED_PASSES)) {
        pl.passes = opt->passes < 0 ? 0 : (opt->passes > 2 ? 2 : opt->passes);
        pl.bits[0] = pl.passes >= 1 ? (opt->radix_bits[0] > 0 ? opt->radix_bits[0] : 8) : 0;
        pl.bits[1] = pl.passes >= 2 ? (opt->radix_bits[1] > 0 ? opt->radix_bits[1] : 8) : 0;
    }
    for (int p = 0; p < 2; p++) {
        if (pl.bits[p] > MAX_RADIX_BITS) pl.bits[p] = MAX_RADIX_BITS;
    }
    pl.max_units[0] = pass_units(info, nr + ns, 2, tail_split(info));
    pl.max_units[1] = pass_units(info, nr + ns, 2 << pl.bits[0], tail_split(info));
    return pl;
}

// ------------------------------------------------------------------ kernel attributes

// Per (kernel, device): the dynamic shared memory already allowed, and occupancies already
// asked for -- driver calls a join would otherwise repeat on every call.
std::mutex g_attr_mutex;
std::map<std::pair<const void *, int>, size_t> g_smem_allowed;
std::map<std::tuple<const void *, int, int, size_t>, int> g_occupancy;

template <typename K>
int ensure_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return VJ_OK;
    int dev = 0;
    VJ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    size_t &allowed = g_smem_allowed[std::make_pair((const void *)kernel, dev)];
    if (allowed >= bytes) return VJ_OK;
    VJ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    allowed = bytes;
    return VJ_OK;
}

template <typename K>
int blocks_per_sm(K kernel, int threads, size_t smem, int *per_sm) {
    int dev = 0;
    VJ_CUDA(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lock(g_attr_mutex);
        auto it = g_occupancy.find(std::make_tuple((const void *)kernel, dev, threads, smem));
        if (it != g_occupancy.end()) {
            *per_sm = it->second;
            return VJ_OK;
        }
    }
    VJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kernel, threads, smem));
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    g_occupancy[std::make_tuple((const void *)kernel, dev, threads, smem)] = *per_sm;
    return VJ_OK;
}


// Bookkeeping of one pass (workspace).
struct PassBufs {
    uint32_t *plan = nullptr;              // [G + 3]: the pass's unit plan when the previous pass writes it
    uint32_t *ctl = nullptr;               // [4]: counters and the scatter's ticket \  cleared
    uint32_t *seg_done = nullptr;          // [G]: units counted per segment          |  before
    uint32_t *seg_tot = nullptr;           // [G * bins]: bucket totals per segment   /  the pass
    unsigned long long *look = nullptr;    // [max_units * bins]: look-back words
    uint32_t *part_begin = nullptr, *part_end = nullptr;  // [G * bins]
    int max_units = 0;
    int G = 0;
};

PassBufs carve_pass(Carver &c, int G, int bins, int max_units) {
    PassBufs b;
    b.plan = c.take<uint32_t>((size_t)G + 3);
    b.ctl = c.take<uint32_t>(4);
    b.seg_done = c.take<uint32_t>((size_t)G, 16);
    b.seg_tot = c.take<uint32_t>((size_t)G * bins, 16);
    b.look = c.take<unsigned long long>((size_t)max_units * bins);
    b.part_begin = c.take<uint32_t>((size_t)G * bins);
    b.part_end = c.take<uint32_t>((size_t)G * bins);
    b.max_units = max_units;
    b.G = G;
    return b;
}

// One radix pass: histogram (per-unit counts, partition bounds, the next pass's plan) and
// scatter (look-back cursors, bucket-sorted tiles). P's plan (device or host), sides,
// segments, bucket rule and next_plan are the caller's; the bookkeeping comes from b.
// The pass's bookkeeping in P; its counters, ticket and the segments' totals set to zero
// (the histogram writes every unit's look-back words).
int pass_setup(PassParams &P, const PassBufs &b, cudaStream_t stream) {
    const uint32_t bins = 1u << P.bits;
    P.ctl = b.ctl;
    P.seg_done = b.seg_done;
    P.seg_tot = b.seg_tot;
    P.look = b.look;
    P.part_begin = b.part_begin;
    P.part_end = b.part_end;
    P.max_units = b.max_units;
    VJ_CUDA(cudaMemsetAsync(b.ctl, 0, (size_t)((char *)(b.seg_tot + (size_t)b.G * bins) - (char *)b.ctl), stream));
    return VJ_OK;
}

template <int KW, int PB, int HS, bool IN_AOS, bool OUT_AOS>
int run_pass(vj_ctx *ctx, int sms, int pass, PassParams P, const PassBufs &b, cudaStream_t stream) {
    const uint32_t bins = 1u << P.bits;
    profile_mark(ctx, PM_PASS0 + 4 * pass, stream);
    VJ_TRY(pass_setup(P, b, stream));
    if (ctx && ctx->sm_reserve) {
        // SMs reserved: at most 4 blocks for each SM the join may use, looping over units
        histogram_kernel<KW, PB, HS, IN_AOS, true><<<std::min(b.max_units, sms * 4), PART_THREADS, bins * sizeof(uint32_t), stream>>>(P);
    } else {
        histogram_kernel<KW, PB, HS, IN_AOS><<<b.max_units, PART_THREADS, bins * sizeof(uint32_t), stream>>>(P);
    }
    VJ_CUDA(cudaGetLastError());
    profile_mark(ctx, PM_HIST_END + 4 * pass, stream);
    profile_mark(ctx, PM_SCAN_END + 4 * pass, stream);
    constexpr int ITEMS = scatter_items<KW, PB, HS, IN_AOS>();
    const size_t sc_smem = ScatterSmem<KW, PB, HS, IN_AOS, ITEMS>::bytes(bins);
    VJ_TRY(ensure_smem(scatter_kernel<KW, PB, HS, IN_AOS, OUT_AOS, ITEMS>, sc_smem));
    int per_sm = 0;
    VJ_TRY(blocks_per_sm(scatter_kernel<KW, PB, HS, IN_AOS, OUT_AOS, ITEMS>, PART_THREADS, sc_smem, &per_sm));
    VJ_CHECK(per_sm >= 1, VJ_ERR_UNSUPPORTED, "scatter kernel does not fit an SM (%zu bytes of shared memory)", sc_smem);
    scatter_kernel<KW, PB, HS, IN_AOS, OUT_AOS, ITEMS><<<sms * per_sm, PART_THREADS, sc_smem, stream>>>(P);
    VJ_CUDA(cudaGetLastError());
    profile_mark(ctx, PM_SCATTER_END + 4 * pass, stream);
    if (ctx) ctx->launches += 2;
    return VJ_OK;
}

template <int KW, int PB, int HS, bool AOS, bool BATCH>
int probe_grid(int sms, int threads, size_t smem, int *grid) {
    int per_sm = 0;
    VJ_TRY(blocks_per_sm(probe_kernel<KW, PB, HS, AOS, BATCH>, threads, smem, &per_sm));
    if (per_sm < 1) per_sm = 1;
    *grid = sms * per_sm;
    return VJ_OK;
}

// Device pointers of both tables, in and out of the partition passes.
struct Tables {
    const void *keys[2], *pay[2], *hash[2];
    uint32_t rows[2];
    // a batch of independent joins (r_offsets set): join j is build rows
    // [r_offsets[j], r_offsets[j+1]) and probe rows [s_offsets[j], s_offsets[j+1]); its
    // pairs go to pair_offsets[j] .. pair_offsets[j+1] of the output, counted in counts[j]
    uint32_t joins = 1;
    const unsigned long long *r_offsets = nullptr, *s_offsets = nullptr, *pair_offsets = nullptr;
    unsigned long long pair_capacity = 0;
    unsigned long long *counts = nullptr;
};

// Segments of a batch from the caller's offsets, each range clamped into its table (and
// the output ranges into the output buffer) so that no later kernel can leave its buffers;
// error flag 16 when an offset had to be clamped.
__global__ void batch_segments_kernel(uint32_t joins, const unsigned long long *ro, const unsigned long long *so, const unsigned long long *po, uint32_t r_rows, uint32_t s_rows,
                                      unsigned long long pair_cap, uint32_t *seg_begin, uint32_t *seg_end, unsigned long long *out_begin, uint32_t *error) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j <= joins; j += gridDim.x * blockDim.x) {
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
}

// Output ranges must not decrease: a running maximum over the (clamped) pair offsets.
__global__ void batch_out_monotone_kernel(uint32_t joins, unsigned long long *out_begin) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long m = 0;
        for (uint32_t j = 0; j <= joins; j++) {
            if (out_begin[j] < m) out_begin[j] = m;
            m = out_begin[j];
        }
    }
}

struct JoinRun {
    // results
    unsigned long long *d_out_count;
    uint32_t *d_error;
    // probe inputs prepared by the partition passes
    ProbeParams probe;
    bool aos;          // probe reads row-contiguous partition buffers
    int threads;       // probe block size
    size_t probe_smem;
    int probe_grid;
    unsigned long long *plan_blocks = nullptr;  // per-block item offsets of the item planner
    // batches of joins: per-join item counts, partitions per join
    bool batch = false;
    uint32_t *batch_cnt = nullptr;
    uint32_t batch_parts = 1;
    bool plant_flag = false;  // VJ_JOIN_TEST_DEVICE_FLAG
    // a batch as one fused launch (set before prepare): its parameters, grid and shared memory
    bool fused = false;
    BatchFusedParams fusedp{};
    int fused_grid = 0;
    size_t fused_smem = 0;
};

// VJ_JOIN_TEST_DEVICE_FLAG: sets a flag bit in the error word as a kernel that ran out of a
// bounded wait would, so that tests can follow it to the call's status.
__global__ void plant_flag_kernel(uint32_t *error, uint32_t bit) { atomicOr(error, bit); }

template <int KW, int PB, int HS, bool AOS, bool BATCH>
int probe_setup(vj_ctx *ctx, const Plan &pl, JoinRun *run) {
    run->aos = AOS;
    run->batch = BATCH;
    run->threads = pl.threads;
    run->probe_smem = ProbeSmem<KW, PB, HS, AOS>::bytes(pl.rcap, pl.tcap, pl.scap);
    VJ_TRY(ensure_smem(probe_kernel<KW, PB, HS, AOS, BATCH>, run->probe_smem));
    return probe_grid<KW, PB, HS, AOS, BATCH>(ctx->info.sms - ctx->sm_reserve, pl.threads, run->probe_smem, &run->probe_grid);
}

// Everything up to (not including) the probe launch. Returns probe parameters whose
// output fields the caller fills in.
template <int KW, int PB, int HS>
int prepare(vj_ctx *ctx, const Tables &in, const Plan &pl, const HashSpec &hs, cudaStream_t stream, JoinRun *run) {
    using L = Layout<KW, PB, HS>;
    const int bins0 = 1 << pl.bits[0];
    const int bins1 = 1 << pl.bits[1];
    const bool batch = in.r_offsets != nullptr;
    const int J = batch ? (int)in.joins : 1;  // segments per side entering the first pass
    const int G0 = 2 * J, G1 = 2 * J * bins0;
    const int np = J * (pl.passes == 0 ? 1 : (pl.passes == 1 ? bins0 : bins0 * bins1));
    int max_units[2] = {pl.max_units[0], pl.max_units[1]};
    if (batch) {
        max_units[0] = pass_units(ctx->info, (uint64_t)in.rows[0] + in.rows[1], G0, tail_split(ctx->info));
        max_units[1] = pass_units(ctx->info, (uint64_t)in.rows[0] + in.rows[1], G1, tail_split(ctx->info));
    }

    // ---- workspace layout (dry run, then carve): per pass one row-contiguous buffer per side
    const uint64_t item_cap = batch ? 2ull * ((uint64_t)np + in.rows[1] / pl.schunk + in.rows[0] / pl.rcap) + 4096 : (uint64_t)np + in.rows[1] / pl.schunk + in.rows[0] / pl.rcap + 4096;
    uint32_t *b_seg_begin = nullptr, *b_seg_end = nullptr, *b_cnt = nullptr;
    unsigned long long *plan_blocks = nullptr;
    uint16_t *bids[2] = {nullptr, nullptr};  // pass-2 buckets written by pass 1
    unsigned long long *b_out_begin = nullptr;
    uint32_t *item_join = nullptr;
    uint32_t *gsync = nullptr;  // the fused batch's grid-barrier words, right after the error word
    const bool fused = run->fused;
    auto layout = [&](Carver &c, void *bufs[2][2], PassBufs *pb0, PassBufs *pb1, uint32_t **item_begin, uint4 **item_desc, uint32_t **ticket, unsigned long long **out_count, uint32_t **error) {
        for (int pass = 0; pass < 2; pass++) {
            for (int sd = 0; sd < 2; sd++) {
                bufs[pass][sd] = pl.passes > pass ? c.take<char>((size_t)in.rows[sd] * L::STRIDE + 64) : nullptr;
            }
        }
        for (int sd = 0; sd < 2; sd++) bids[sd] = pl.passes >= 2 ? c.take<uint16_t>((size_t)in.rows[sd] + 8) : nullptr;
        if (batch) {
            b_seg_begin = c.take<uint32_t>((size_t)2 * J);
            b_seg_end = c.take<uint32_t>((size_t)2 * J);
            b_cnt = c.take<uint32_t>((size_t)J);
            b_out_begin = c.take<unsigned long long>((size_t)J + 1);
        }
        if (pl.passes >= 1) *pb0 = carve_pass(c, G0, bins0, max_units[0]);
        if (pl.passes >= 2) *pb1 = carve_pass(c, G1, bins1, max_units[1]);
        *item_begin = c.take<uint32_t>((size_t)np + 2);
        plan_blocks = c.take<unsigned long long>(((size_t)np + PLAN_BLOCK - 1) / PLAN_BLOCK);
        *item_desc = c.take<uint4>(item_cap);
        item_join = batch ? c.take<uint32_t>(item_cap) : nullptr;
        *ticket = c.take<uint32_t>(1);
        *out_count = c.take<unsigned long long>(1);
        *error = c.take<uint32_t>(1);
        gsync = c.take<uint32_t>(2, 4);
    };
    void *bufs[2][2];
    PassBufs pb0{}, pb1{};
    uint32_t *item_begin, *ticket, *error;
    uint4 *item_desc;
    unsigned long long *out_count;
    Carver dry;
    layout(dry, bufs, &pb0, &pb1, &item_begin, &item_desc, &ticket, &out_count, &error);
    void *ws = nullptr;
    VJ_TRY(workspace_reserve(ctx, dry.off + 256, stream, &ws));
    Carver c;
    c.base = (char *)ws;
    layout(c, bufs, &pb0, &pb1, &item_begin, &item_desc, &ticket, &out_count, &error);
    VJ_CUDA(cudaMemsetAsync(error, 0, fused ? 3 * sizeof(uint32_t) : sizeof(uint32_t), stream));
    ctx->launches = 0;

    const uint32_t *seg_begin = nullptr, *seg_end = nullptr;
    int Q = 1;
    if (batch && fused) {
        seg_begin = b_seg_begin;
        seg_end = b_seg_end;
        Q = J;
    } else if (batch) {
        batch_segments_kernel<<<(J + 256) / 256, 256, 0, stream>>>(in.joins, in.r_offsets, in.s_offsets, in.pair_offsets, in.rows[0], in.rows[1], in.pair_capacity, b_seg_begin, b_seg_end, b_out_begin,
                                                                     error);
        VJ_CUDA(cudaGetLastError());
        batch_out_monotone_kernel<<<1, 1, 0, stream>>>(in.joins, b_out_begin);
        VJ_CUDA(cudaGetLastError());
        ctx->launches += 2;
        seg_begin = b_seg_begin;
        seg_end = b_seg_end;
        Q = J;
    }
    int consumed_bits = 0;
    for (int pass = 0; pass < pl.passes; pass++) {
        PassParams P{};
        for (int sd = 0; sd < 2; sd++) {
            P.side[sd].keys_in = in.keys[sd];
            P.side[sd].pay_in = in.pay[sd];
            P.side[sd].hash_in = in.hash[sd];
            P.side[sd].rows_in = pass > 0 ? bufs[pass - 1][sd] : nullptr;
            P.side[sd].rows_out = bufs[pass][sd];
            P.side[sd].rows = in.rows[sd];
            P.side[sd].bid_out = pass == 0 && pl.passes >= 2 ? bids[sd] : nullptr;
            P.side[sd].bid_in = pass == 1 ? bids[sd] : nullptr;
        }
        P.next_shift = 64 - (pl.bits[0] + pl.bits[1]);
        P.next_bits = pl.bits[1];
        P.nsides = 2;
        P.Q = Q;
        P.seg_begin = seg_begin;
        P.seg_end = seg_end;
        P.bits = pl.bits[pass];
        consumed_bits += pl.bits[pass];
        P.shift = 64 - consumed_bits;  // top bits of the mixed hash, pass 1 first
        P.hs = hs;
        P.max_units = max_units[pass];
        P.min_unit_rows = MIN_UNIT_ROWS;
        P.split = tail_split(ctx->info);
        P.next_split = tail_split(ctx->info);
        P.error = error;
        const PassBufs &pb = pass == 0 ? pb0 : pb1;
        if (pass == 0 && !batch) {
            host_plan(P, in.rows, 2);
        } else {
            P.plan = pb.plan;  // written by the previous pass, or by plan_kernel for a batch
            if (pass == 0 && !fused) {
                plan_kernel<<<1, PLAN_THREADS, 0, stream>>>(P, pb.plan);
                VJ_CUDA(cudaGetLastError());
                ctx->launches += 1;
            }
        }
        if (pass == 0 && pl.passes >= 2) {
            P.next_plan = pb1.plan;
            P.next_max_units = pb1.max_units;
        }
        if (fused) {
            VJ_TRY(pass_setup(P, pb, stream));  // the fused launch runs the pass itself
            run->fusedp.P = P;
        } else if (pass == 0) {
            VJ_TRY((run_pass<KW, PB, HS, false, true>(ctx, ctx->info.sms, pass, P, pb, stream)));
        } else {
            VJ_TRY((run_pass<KW, PB, HS, true, true>(ctx, ctx->info.sms, pass, P, pb, stream)));
        }
        seg_begin = pb.part_begin;
        seg_end = pb.part_end;
        Q = Q << pl.bits[pass];
    }

    ProbeParams Pq{};
    Pq.r_keys = in.keys[0];
    Pq.r_pay = in.pay[0];
    Pq.r_hash = in.hash[0];
    Pq.s_keys = in.keys[1];
    Pq.s_pay = in.pay[1];
    Pq.s_hash = in.hash[1];
    if (pl.passes == 0) {
        Pq.r_rows_in = Pq.s_rows_in = nullptr;
        Pq.r_begin = seg_begin;  // a batch: one partition per join; else the whole tables
        Pq.r_end = seg_end;
        Pq.s_begin = seg_begin ? seg_begin + np : nullptr;
        Pq.s_end = seg_end ? seg_end + np : nullptr;
    } else {
        Pq.r_rows_in = bufs[pl.passes - 1][0];
        Pq.s_rows_in = bufs[pl.passes - 1][1];
        Pq.r_begin = seg_begin;
        Pq.r_end = seg_end;
        Pq.s_begin = seg_begin + np;
        Pq.s_end = seg_end + np;
    }
    Pq.r_rows = in.rows[0];
    Pq.s_rows = in.rows[1];
    Pq.np = np;
    Pq.rcap = pl.rcap;
    Pq.schunk = pl.schunk;
    Pq.tcap = pl.tcap;
    Pq.tmul = pl.tmul;
    Pq.scap = pl.scap;
    // slot bits: the 14 bits right below the partition bits (tables hold at most 2^14 slots)
    Pq.slot_shift = 64 - (pl.bits[0] + pl.bits[1]) - 14;
    Pq.item_begin = item_begin;
    Pq.item_desc = item_desc;
    Pq.item_join = item_join;
    Pq.item_cap = (uint32_t)(item_cap < 0xffffffffull ? item_cap : 0xffffffffull);
    Pq.ticket = ticket;
    Pq.out_count = out_count;
    Pq.hs = hs;
    Pq.error = error;
    Pq.joins = (uint32_t)J;
    if (batch) {
        Pq.out_begin = b_out_begin;
        Pq.out_counts = in.counts;
        run->batch_cnt = b_cnt;
        run->batch_parts = (uint32_t)(np / J);
    }
    run->probe = Pq;
    run->plan_blocks = plan_blocks;
    run->d_out_count = out_count;
    run->d_error = error;
    if (fused) {
        BatchFusedParams &F = run->fusedp;
        F.passes = (uint32_t)pl.passes;
        F.joins = (uint32_t)J;
        F.r_rows = in.rows[0];
        F.s_rows = in.rows[1];
        F.parts = (uint32_t)(np / J);
        F.ro = in.r_offsets;
        F.so = in.s_offsets;
        F.po = in.pair_offsets;
        F.pair_cap = in.pair_capacity;
        F.seg_begin = b_seg_begin;
        F.seg_end = b_seg_end;
        F.out_begin = b_out_begin;
        F.plan = pl.passes ? pb0.plan : nullptr;
        F.cnt = b_cnt;
        F.sync = gsync;
        const size_t probe_smem = ProbeSmem<KW, PB, HS, true>::bytes(pl.rcap, pl.tcap, pl.scap);
        run->fused_smem = batch_fused_smem<KW, PB, HS>(1u << pl.bits[0], probe_smem);
        run->fused_grid = ctx->info.sms;
        run->threads = PROBE_THREADS;
        return VJ_OK;
    }
    if (pl.passes == 0) {
        return batch ? probe_setup<KW, PB, HS, false, true>(ctx, pl, run) : probe_setup<KW, PB, HS, false, false>(ctx, pl, run);
    }
    return batch ? probe_setup<KW, PB, HS, true, true>(ctx, pl, run) : probe_setup<KW, PB, HS, true, false>(ctx, pl, run);
}

template <int KW, int PB, int HS>
int launch_probe(vj_ctx *ctx, const JoinRun &run, cudaStream_t stream) {
    profile_mark(ctx, PM_PROBE_BEGIN, stream);
    if (run.probe.out_begin) {
        const ProbeParams &Q = run.probe;
        batch_items_kernel<true><<<Q.joins, 256, 0, stream>>>(Q, run.batch_parts, run.batch_cnt, nullptr);
        VJ_CUDA(cudaGetLastError());
        batch_scan_kernel<<<1, PLAN_THREADS, 0, stream>>>(Q, run.batch_cnt);
        VJ_CUDA(cudaGetLastError());
        batch_items_kernel<false><<<Q.joins, 256, 0, stream>>>(Q, run.batch_parts, nullptr, run.batch_cnt);
        VJ_CUDA(cudaGetLastError());
        ctx->launches += 3;
    } else {
        const int nb = (run.probe.np + PLAN_BLOCK - 1) / PLAN_BLOCK;
        items_count_kernel<<<nb, PLAN_BLOCK, 0, stream>>>(run.probe, run.plan_blocks);
        VJ_CUDA(cudaGetLastError());
        items_scan_kernel<<<1, PLAN_THREADS, 0, stream>>>(run.probe, run.plan_blocks, nb);
        VJ_CUDA(cudaGetLastError());
        items_write_kernel<<<nb, PLAN_BLOCK, 0, stream>>>(run.probe, run.plan_blocks);
        VJ_CUDA(cudaGetLastError());
        ctx->launches += 3;
    }
    if (run.aos) {
        if (run.batch) probe_kernel<KW, PB, HS, true, true><<<run.probe_grid, run.threads, run.probe_smem, stream>>>(run.probe);
        else probe_kernel<KW, PB, HS, true, false><<<run.probe_grid, run.threads, run.probe_smem, stream>>>(run.probe);
    } else {
        if (run.batch) probe_kernel<KW, PB, HS, false, true><<<run.probe_grid, run.threads, run.probe_smem, stream>>>(run.probe);
        else probe_kernel<KW, PB, HS, false, false><<<run.probe_grid, run.threads, run.probe_smem, stream>>>(run.probe);
    }
    VJ_CUDA(cudaGetLastError());
    ctx->launches += 1;
    if (run.plant_flag) {
        plant_flag_kernel<<<1, 1, 0, stream>>>(run.d_error, 32u);
        VJ_CUDA(cudaGetLastError());
        ctx->launches += 1;
    }
    profile_mark(ctx, PM_PROBE_END, stream);
    return VJ_OK;
}

// After the stream has been synchronised: stage times of a profiled join.
void finish_profile(vj_ctx *ctx, const Plan &pl, uint64_t nr, uint64_t ns, uint64_t matches) {
    vj_profile &p = ctx->last;
    memset(&p, 0, sizeof(p));
    p.passes = pl.passes;
    p.kernel_launches = ctx->launches;
    p.radix_bits[0] = pl.bits[0];
    p.radix_bits[1] = pl.bits[1];
    p.build_rows = pl.rcap;
    p.probe_rows = pl.schunk;
    p.tables = VJ_TABLES_SHARED;
    p.fallbacks = 0;
    p.rows[0] = nr;
    p.rows[1] = ns;
    p.matches = matches;
    if (!ctx->profiling || !ctx->events_ready) return;
    auto ms = [&](int a, int b) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ctx->events[a], ctx->events[b]) != cudaSuccess) {
            cudaGetLastError();
            t = 0.f;
        }
        return t;
    };
    for (int pass = 0; pass < pl.passes; pass++) {
        p.ms_histogram[pass] = ms(PM_PASS0 + 4 * pass, PM_HIST_END + 4 * pass);
        p.ms_plan[pass] = ms(PM_HIST_END + 4 * pass, PM_SCAN_END + 4 * pass);
        p.ms_scatter[pass] = ms(PM_SCAN_END + 4 * pass, PM_SCATTER_END + 4 * pass);
    }
    p.ms_probe = ms(PM_PROBE_BEGIN, PM_PROBE_END);
    p.ms_total = ms(pl.passes ? PM_PASS0 : PM_PROBE_BEGIN, PM_PROBE_END);
}

// Match count and error flags of a probe, stored by one thread into page-locked host memory
// (the copy engines' small copies to the host stalled now and then for tens of ms).
__global__ void read_count_kernel(const unsigned long long *count, const uint32_t *error, volatile unsigned long long *host) {
    host[0] = *count;
    host[1] = *error;
}

// Per host thread: the page-locked words read_count_kernel stores into, freed when the
// thread ends.
struct CountWords {
    unsigned long long *host = nullptr, *mapped = nullptr;
    ~CountWords() {
        if (host) cudaFreeHost(host);
    }
};

// Match count and the kernels' error flags of the probe just launched (synchronises).
int read_count(vj_ctx *ctx, const JoinRun &run, cudaStream_t stream, uint64_t *count, uint32_t *flags) {
    static thread_local CountWords words;
    if (!words.host) {
        unsigned long long *h = nullptr;
        VJ_CUDA(cudaHostAlloc((void **)&h, 2 * sizeof(unsigned long long), cudaHostAllocMapped | cudaHostAllocPortable));
        note_allocation();
        unsigned long long *d = nullptr;
        const cudaError_t e = cudaHostGetDevicePointer((void **)&d, h, 0);
        if (e != cudaSuccess) {
            cudaFreeHost(h);
            return cuda_error(e, "read_count: mapped host words");
        }
        words.host = h;
        words.mapped = d;
    }
    unsigned long long *pinned = words.host, *mapped = words.mapped;
    read_count_kernel<<<1, 1, 0, stream>>>(run.d_out_count, run.d_error, mapped);
    VJ_CUDA(cudaGetLastError());
    ctx->launches += 1;
    VJ_CUDA(cudaStreamSynchronize(stream));
    const volatile unsigned long long *h = pinned;
    *count = h[0];
    *flags = (uint32_t)h[1];
    return VJ_OK;
}

int check_flags(uint32_t flags) {
    VJ_CHECK(flags == 0, VJ_ERR_DEVICE, "probe kernel reported an internal limit (flags %x)", flags);
    return VJ_OK;
}

// Plan, partition and probe once into (out, capacity). On return `run` holds the partitions
// (for a second probe into a larger buffer).
template <int KW, int PB, int HS>
int probe_once(vj_ctx *ctx, const Tables &t, const HashSpec &hs, const vj_join_options *opt, void *out, uint64_t capacity, cudaStream_t stream, JoinRun *run, Plan *plan, uint64_t *count) {
    Plan pl = make_plan<KW, PB, HS>(t.rows[0], t.rows[1], ctx->info, opt);
    *run = JoinRun{};
    VJ_TRY((prepare<KW, PB, HS>(ctx, t, pl, hs, stream, run)));
    run->plant_flag = opt && (opt->flags & VJ_JOIN_TEST_DEVICE_FLAG);
    run->probe.out = out;
    run->probe.capacity = capacity;
    VJ_TRY((launch_probe<KW, PB, HS>(ctx, *run, stream)));
    uint32_t flags = 0;
    VJ_TRY(read_count(ctx, *run, stream, count, &flags));
    VJ_TRY(check_flags(flags));
    *plan = pl;
    return VJ_OK;
}

// ------------------------------------------------------------------ typed entry points

template <int KW, int PB, int HS>
int join_typed(vj_ctx *ctx, const Tables &t, const HashSpec &hs, const vj_join_options *opt, vj_result *res, cudaStream_t stream) {
    const bool caller_buffer = res->pairs != nullptr && res->capacity > 0 && !res->owned;
    if (!caller_buffer) {
        uint64_t cap = t.rows[1] ? t.rows[1] : 1;
        void *p = nullptr;
        VJ_TRY(owned_alloc(ctx, (size_t)cap * 2 * PB, stream, &p));
        res->pairs = p;
        res->capacity = cap;
        res->owned = 1;
    }
    res->payload_bytes = PB;
    Plan pl;
    JoinRun run;
    uint64_t count = 0;
    VJ_TRY((probe_once<KW, PB, HS>(ctx, t, hs, opt, res->pairs, res->capacity, stream, &run, &pl, &count)));
    finish_profile(ctx, pl, t.rows[0], t.rows[1], count);
    if (count > res->capacity) {
        if (!res->owned) {
            res->count = count;
            return set_error(VJ_ERR_CAPACITY, "join produced %llu pairs, output capacity is %llu", (unsigned long long)count, (unsigned long long)res->capacity);
        }
        // library-owned output: grow to the exact count and probe again (the partitions are
        // still in the workspace)
        VJ_CUDA(cudaFreeAsync(res->pairs, stream));
        owned_release(ctx, (size_t)res->capacity * 2 * PB);
        res->pairs = nullptr;
        res->capacity = 0;
        void *p = nullptr;
        VJ_TRY(owned_alloc(ctx, (size_t)count * 2 * PB, stream, &p));
        res->pairs = p;
        res->capacity = count;
        run.probe.out = p;
        run.probe.capacity = count;
        VJ_TRY((launch_probe<KW, PB, HS>(ctx, run, stream)));
        uint64_t again = 0;
        uint32_t flags = 0;
        VJ_TRY(read_count(ctx, run, stream, &again, &flags));
        VJ_TRY(check_flags(flags));
        VJ_CHECK(again == count, VJ_ERR_DEVICE, "second probe gave %llu pairs, first %llu", (unsigned long long)again, (unsigned long long)count);
    }
    res->count = count;
    return VJ_OK;
}

template <int KW, int PB, int HS>
int partition_typed(vj_ctx *ctx, const vj_table *in, const void *hashes_in, const HashSpec &hs, void *keys_out, void *pay_out, void *hash_out, int shift, int bits, uint64_t *d_hist, uint64_t *d_off,
                    uint64_t *h_hist, uint64_t *h_off, cudaStream_t stream);

}  // namespace

// Export of a single-segment pass result as the reference's index_t histogram/offsets; when a
// kernel of the pass set an error flag, every histogram entry is UINT64_MAX instead.
__global__ void export_hist_kernel(const uint32_t *begin, const uint32_t *end, int bins, unsigned long long *hist, unsigned long long *off, const uint32_t *error) {
    const bool bad = *error != 0;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bins; b += gridDim.x * blockDim.x) {
        if (hist) hist[b] = bad ? ~0ull : (unsigned long long)(end[b] - begin[b]);
        if (off) off[b] = begin[b];
    }
}

namespace {

template <int KW, int PB, int HS>
int partition_typed(vj_ctx *ctx, const vj_table *in, const void *hashes_in, const HashSpec &hs, void *keys_out, void *pay_out, void *hash_out, int shift, int bits, uint64_t *d_hist, uint64_t *d_off,
                    uint64_t *h_hist, uint64_t *h_off, cudaStream_t stream) {
    const int bins = 1 << bits;
    const int G = 1;
    const int max_units = pass_units(ctx->info, in->rows, G);
    auto layout = [&](Carver &c, PassBufs *pb, unsigned long long **hist, unsigned long long **off, uint32_t **err) {
        *pb = carve_pass(c, G, bins, max_units);
        *hist = c.take<unsigned long long>(bins);
        *off = c.take<unsigned long long>(bins);
        *err = c.take<uint32_t>(1);
    };
    PassBufs pb;
    unsigned long long *dh, *doff;
    uint32_t *derr;
    Carver dry;
    layout(dry, &pb, &dh, &doff, &derr);
    void *ws = nullptr;
    VJ_TRY(workspace_reserve(ctx, dry.off + 256, stream, &ws));
    Carver c;
    c.base = (char *)ws;
    layout(c, &pb, &dh, &doff, &derr);
    VJ_CUDA(cudaMemsetAsync(derr, 0, sizeof(uint32_t), stream));
    PassParams P{};
    P.side[0].keys_in = in->keys;
    P.side[0].pay_in = in->payloads;
    P.side[0].hash_in = hashes_in;
    P.side[0].rows_in = nullptr;
    P.side[0].rows_out = nullptr;
    P.side[0].keys_out = keys_out;
    P.side[0].pay_out = pay_out;
    P.side[0].hash_out = hash_out;
    P.side[0].rows = (uint32_t)in->rows;
    P.nsides = 1;
    P.Q = 1;
    P.seg_begin = P.seg_end = nullptr;
    P.shift = shift;
    P.bits = bits;
    P.hs = hs;
    P.max_units = max_units;
    P.min_unit_rows = MIN_UNIT_ROWS;
    P.error = derr;
    const uint32_t rows = (uint32_t)in->rows;
    host_plan(P, &rows, 1);
    // an empty table still has one (empty) unit, which writes the empty bounds
    VJ_TRY((run_pass<KW, PB, HS, false, false>(ctx, ctx->info.sms, 0, P, pb, stream)));
    export_hist_kernel<<<(bins + 255) / 256, 256, 0, stream>>>(pb.part_begin, pb.part_end, bins, d_hist ? (unsigned long long *)d_hist : dh, d_off ? (unsigned long long *)d_off : doff, derr);
    VJ_CUDA(cudaGetLastError());
    if (h_hist || h_off) {
        if (h_hist) VJ_CUDA(cudaMemcpyAsync(h_hist, d_hist ? (void *)d_hist : (void *)dh, bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
        if (h_off) VJ_CUDA(cudaMemcpyAsync(h_off, d_off ? (void *)d_off : (void *)doff, bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
        uint32_t herr = 0;
        VJ_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        VJ_CUDA(cudaStreamSynchronize(stream));
        VJ_CHECK(herr == 0, VJ_ERR_DEVICE, "vj_partition: a kernel reported an internal limit (flags %x)", herr);
    }
    return VJ_OK;
}

// ------------------------------------------------------------------ dispatch

int check_table(const vj_table *t, const char *name) {
    VJ_CHECK(t != nullptr, VJ_ERR_INVALID_ARGUMENT, "%s: null table", name);
    VJ_CHECK(t->key_words == 1 || t->key_words == 2 || t->key_words == 4 || t->key_words == 6 || t->key_words == 8, VJ_ERR_UNSUPPORTED, "%s: key_words must be 1, 2, 4, 6 or 8 (got %d)", name, t->key_words);
    VJ_CHECK(t->payload_bytes == 4 || t->payload_bytes == 8, VJ_ERR_UNSUPPORTED, "%s: payload_bytes must be 4 or 8 (got %d)", name, t->payload_bytes);
    VJ_CHECK(t->rows < (1ull << 32), VJ_ERR_UNSUPPORTED, "%s: at most 2^32-1 rows", name);
    if (t->rows) {
        VJ_CHECK(t->keys && t->payloads, VJ_ERR_INVALID_ARGUMENT, "%s: null column", name);
        const uintptr_t ka = t->key_words == 1 ? 4 : 8;
        VJ_CHECK((uintptr_t)t->keys % ka == 0, VJ_ERR_INVALID_ARGUMENT, "%s: keys must be %d-byte aligned", name, (int)ka);
        VJ_CHECK((uintptr_t)t->payloads % t->payload_bytes == 0, VJ_ERR_INVALID_ARGUMENT, "%s: payloads must be aligned to their size", name);
    }
    return VJ_OK;
}

// Calls F::template run<KW, PB, HS>() for the supported layouts.
template <typename F>
int dispatch(int kw, int pb, int hs, F &&f) {
#define VJ_D(K, B, H) \
    if (kw == K && pb == B && hs == H) return f.template run<K, B, H>();
    VJ_D(1, 4, 0)
    VJ_D(1, 8, 0)
    VJ_D(2, 4, 0)
    VJ_D(2, 8, 0)
    VJ_D(4, 4, 0)
    VJ_D(4, 8, 0)
    VJ_D(6, 4, 0)
    VJ_D(6, 8, 0)
    VJ_D(8, 4, 0)
    VJ_D(8, 8, 0)
    VJ_D(2, 8, 4)
    VJ_D(2, 8, 8)
    VJ_D(4, 8, 4)
    VJ_D(4, 8, 8)
    VJ_D(6, 8, 4)
    VJ_D(6, 8, 8)
    VJ_D(8, 8, 4)
    VJ_D(8, 8, 8)
#undef VJ_D
    return set_error(VJ_ERR_UNSUPPORTED, "unsupported layout: key_words %d, payload_bytes %d, hash array bytes %d", kw, pb, hs);
}

int check_options(const vj_join_options *opt, const char *name) {
    VJ_CHECK(!opt || !(opt->flags & VJ_JOIN_L2_TABLES), VJ_ERR_UNSUPPORTED, "%s: VJ_JOIN_L2_TABLES is no longer offered (shared-memory tables only)", name);
    return VJ_OK;
}

HashSpec spec_from(const vj_join_options *opt, int mix) {
    HashSpec hs;
    hs.algo = opt && opt->hash_algo > 0 && opt->hash_algo < VJ_HASH_COUNT ? opt->hash_algo : VJ_HASH_FNV;
    hs.hash_bits = opt && opt->hash_bits == 32 ? 32 : 64;
    hs.mix = mix;
    return hs;
}

struct JoinCall {
    vj_ctx *ctx;
    Tables t;
    HashSpec hs;
    const vj_join_options *opt;
    vj_result *res;
    cudaStream_t stream;
    template <int KW, int PB, int HS>
    int run() {
        return join_typed<KW, PB, HS>(ctx, t, hs, opt, res, stream);
    }
};

struct PartitionCall {
    vj_ctx *ctx;
    const vj_table *in;
    const void *hashes;
    HashSpec hs;
    void *ko, *po, *ho;
    int shift, bits;
    uint64_t *dh, *doff, *hh, *hoff;
    cudaStream_t stream;
    template <int KW, int PB, int HS>
    int run() {
        return partition_typed<KW, PB, HS>(ctx, in, hashes, hs, ko, po, ho, shift, bits, dh, doff, hh, hoff, stream);
    }
};

// build_and_probe: the plan never reallocates the caller's buffer; count only past capacity.
struct BuildProbeCall {
    JoinCall &c;
    template <int KW, int PB, int HS>
    int run() {
        vj_result &rr = *c.res;
        Plan pl;
        JoinRun run;
        uint64_t n = 0;
        VJ_TRY((probe_once<KW, PB, HS>(c.ctx, c.t, c.hs, c.opt, rr.pairs, rr.capacity, c.stream, &run, &pl, &n)));
        finish_profile(c.ctx, pl, c.t.rows[0], c.t.rows[1], n);
        rr.count = n;
        return VJ_OK;
    }
};

// A batch of joins, no host synchronisation. At most one radix pass (the second pass's
// bookkeeping would grow with joins x buckets x buckets). By default one fused,
// cooperative launch runs it all (batch_fused_kernel); VJ_JOIN_BATCH_LAUNCHES runs the same
// phases as separate launches.
template <int KW, int PB, int HS>
int batch_typed(vj_ctx *ctx, const Tables &t, const HashSpec &hs, const vj_join_options *opt, uint64_t max_build_rows, bool launches, void *pairs, uint32_t *d_status, cudaStream_t stream) {
    const bool fused = HS == 0 && !launches;
    DeviceInfo info = ctx->info;
    if (fused && info.smem_optin > FUSED_SMEM + 1024) info.smem_optin = FUSED_SMEM + 1024;  // room for the phases' static shared memory
    Plan pl = make_plan<KW, PB, HS>(max_build_rows, 4 * max_build_rows, info, opt);
    if (pl.passes == 2) {
        pl.passes = 1;
        pl.bits[0] = pl.bits[0] + pl.bits[1] > MAX_RADIX_BITS ? MAX_RADIX_BITS : pl.bits[0] + pl.bits[1];
        pl.bits[1] = 0;
    }
    if (fused) pl.threads = PROBE_THREADS;  // the fused launch's blocks are PROBE_THREADS wide
    const bool prof = ctx->profiling;
    ctx->profiling = false;  // stage events need a synchronisation this call does not make
    JoinRun run;
    run.fused = fused;
    int st = prepare<KW, PB, HS>(ctx, t, pl, hs, stream, &run);
    if (st == VJ_OK) {
        run.probe.out = pairs;
        run.probe.capacity = t.pair_capacity;
        if (fused) {
            if constexpr (HS == 0) {
                run.fusedp.Q = run.probe;
                st = batch_fused_launch<KW, PB, HS>(run.fusedp, run.fused_grid, run.fused_smem, stream);
                ctx->launches = 1;
            }
        } else {
            st = launch_probe<KW, PB, HS>(ctx, run, stream);
        }
    }
    ctx->profiling = prof;
    VJ_TRY(st);
    if (d_status) VJ_CUDA(cudaMemcpyAsync(d_status, run.d_error, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
    // the plan the batch ran (no stage times: nothing synchronises)
    vj_profile &p = ctx->last;
    memset(&p, 0, sizeof(p));
    p.passes = pl.passes;
    p.kernel_launches = ctx->launches;
    p.radix_bits[0] = pl.bits[0];
    p.radix_bits[1] = pl.bits[1];
    p.build_rows = pl.rcap;
    p.probe_rows = pl.schunk;
    p.rows[0] = t.rows[0];
    p.rows[1] = t.rows[1];
    return VJ_OK;
}

struct BatchCall {
    vj_ctx *ctx;
    Tables t;
    HashSpec hs;
    const vj_join_options *opt;
    uint64_t max_build_rows;
    bool launches;  // VJ_JOIN_BATCH_LAUNCHES: separate launches instead of the fused one
    void *pairs;
    uint32_t *status;
    cudaStream_t stream;
    template <int KW, int PB, int HS>
    int run() {
        return batch_typed<KW, PB, HS>(ctx, t, hs, opt, max_build_rows, launches, pairs, status, stream);
    }
};

struct FootprintCall {
    const vj_ctx *ctx;
    uint64_t nr, ns;
    const vj_join_options *opt;
    uint64_t *bytes;
    template <int KW, int PB, int HS>
    int run() {
        const Plan pl = make_plan<KW, PB, HS>(nr, ns, ctx->info, opt);
        using L = Layout<KW, PB, HS>;
        // partition buffers of every pass (grown by an eighth), bookkeeping, owned output of |S| pairs
        const uint64_t bufs = (uint64_t)pl.passes * (nr + ns) * L::STRIDE;
        *bytes = bufs + bufs / 8 + ns * 2 * PB + (64ull << 20);
        return VJ_OK;
    }
};

}  // namespace

// Device bytes a vj_join of these tables takes from a context: its workspace (partition
// buffers and bookkeeping) and a library-owned output of |S| pairs -- an upper estimate
// for admission by memory budget.
int join_footprint(const vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *opt, uint64_t *bytes) {
    VJ_TRY(check_table(r, "join_footprint: r"));
    VJ_TRY(check_table(s, "join_footprint: s"));
    FootprintCall call{ctx, r->rows, s->rows, opt, bytes};
    return dispatch(r->key_words, r->payload_bytes, 0, call);
}

}  // namespace vj

using namespace vj;

extern "C" int vj_join_batch(vj_ctx *ctx, const vj_table *r, const vj_table *s, uint32_t joins, const uint64_t *d_r_offsets, const uint64_t *d_s_offsets, uint64_t max_build_rows,
                             const vj_join_options *options, void *d_pairs, const uint64_t *d_pair_offsets, uint64_t pair_capacity, uint64_t *d_counts, uint32_t *d_status, vj_stream_t stream) {
    VJ_CHECK(ctx != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_join_batch: null context");
    VJ_TRY(check_table(r, "vj_join_batch: r"));
    VJ_TRY(check_table(s, "vj_join_batch: s"));
    VJ_CHECK(r->key_words == s->key_words && r->payload_bytes == s->payload_bytes, VJ_ERR_INVALID_ARGUMENT, "vj_join_batch: r and s must have the same key_words and payload_bytes");
    VJ_TRY(check_options(options, "vj_join_batch"));
    // the pass's unit scan keeps one shared-memory word per unit, two units per join at least
    VJ_CHECK(joins >= 1 && joins <= 16384, VJ_ERR_UNSUPPORTED, "vj_join_batch: joins must be in [1, 16384] (got %u)", joins);
    VJ_CHECK(d_r_offsets && d_s_offsets && d_pair_offsets && d_counts, VJ_ERR_INVALID_ARGUMENT, "vj_join_batch: null offsets or counts");
    VJ_CHECK(d_pairs != nullptr || pair_capacity == 0, VJ_ERR_INVALID_ARGUMENT, "vj_join_batch: null output with capacity > 0");
    VJ_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    if (r->rows == 0 || s->rows == 0) {  // nothing matches: zero counts, ok status
        VJ_CUDA(cudaMemsetAsync(d_counts, 0, (size_t)joins * sizeof(uint64_t), st));
        if (d_status) VJ_CUDA(cudaMemsetAsync(d_status, 0, sizeof(uint32_t), st));
        return VJ_OK;
    }
    BatchCall call;
    call.ctx = ctx;
    call.t.keys[0] = r->keys;
    call.t.keys[1] = s->keys;
    call.t.pay[0] = r->payloads;
    call.t.pay[1] = s->payloads;
    call.t.hash[0] = call.t.hash[1] = nullptr;
    call.t.rows[0] = (uint32_t)r->rows;
    call.t.rows[1] = (uint32_t)s->rows;
    call.t.joins = joins;
    call.t.r_offsets = (const unsigned long long *)d_r_offsets;
    call.t.s_offsets = (const unsigned long long *)d_s_offsets;
    call.t.pair_offsets = (const unsigned long long *)d_pair_offsets;
    call.t.pair_capacity = pair_capacity;
    call.t.counts = (unsigned long long *)d_counts;
    call.hs = spec_from(options, 1);
    call.opt = options;
    call.max_build_rows = max_build_rows && max_build_rows < r->rows ? max_build_rows : r->rows;
    // a tuned plan for the class of the batch's largest join, if any (probe rows in the
    // batch's ratio)
    vj_table rmax = *r, smax = *s;
    rmax.rows = call.max_build_rows;
    smax.rows = (uint64_t)((double)call.max_build_rows * ((double)s->rows / (double)r->rows)) + 1;
    call.opt = tuned_options(ctx, &rmax, &smax, options);
    call.launches = options && (options->flags & VJ_JOIN_BATCH_LAUNCHES);
    call.pairs = d_pairs;
    call.status = d_status;
    call.stream = st;
    return dispatch(r->key_words, r->payload_bytes, 0, call);
}

extern "C" int vj_join(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, vj_result *result, vj_stream_t stream) {
    VJ_CHECK(ctx && result, VJ_ERR_INVALID_ARGUMENT, "vj_join: null argument");
    VJ_TRY(check_table(r, "vj_join: r"));
    VJ_TRY(check_table(s, "vj_join: s"));
    VJ_CHECK(r->key_words == s->key_words && r->payload_bytes == s->payload_bytes, VJ_ERR_INVALID_ARGUMENT, "vj_join: r and s must have the same key_words and payload_bytes");
    VJ_TRY(check_options(options, "vj_join"));
    VJ_CUDA(cudaSetDevice(ctx->device));
    result->count = 0;
    if (!(result->pairs && result->capacity > 0)) {
        result->pairs = nullptr;
        result->capacity = 0;
        result->owned = 0;
    } else {
        result->owned = 0;
    }
    JoinCall call;
    call.ctx = ctx;
    call.t.keys[0] = r->keys;
    call.t.keys[1] = s->keys;
    call.t.pay[0] = r->payloads;
    call.t.pay[1] = s->payloads;
    call.t.hash[0] = call.t.hash[1] = nullptr;
    call.t.rows[0] = (uint32_t)r->rows;
    call.t.rows[1] = (uint32_t)s->rows;
    call.hs = spec_from(options, 1);
    call.opt = options;
    call.res = result;
    call.stream = (cudaStream_t)stream;
    result->payload_bytes = r->payload_bytes;
    if (r->rows == 0 || s->rows == 0) {
        return VJ_OK;  // empty join: count 0, no buffer needed
    }
    call.opt = tuned_options(ctx, r, s, options);  // a vj_tune result for this shape class, if any
    return dispatch(r->key_words, r->payload_bytes, 0, call);
}

extern "C" int vj_build_probe(vj_ctx *ctx, const vj_table *r, const void *d_r_hashes, const vj_table *s, const void *d_s_hashes, int hash_bits, int key_offset, void *d_pairs, uint64_t capacity, uint64_t *count,
                              vj_stream_t stream) {
    (void)key_offset;
    VJ_CHECK(ctx && count, VJ_ERR_INVALID_ARGUMENT, "vj_build_probe: null argument");
    VJ_TRY(check_table(r, "vj_build_probe: r"));
    VJ_TRY(check_table(s, "vj_build_probe: s"));
    VJ_CHECK(r->key_words == s->key_words && r->payload_bytes == s->payload_bytes, VJ_ERR_INVALID_ARGUMENT, "vj_build_probe: r and s must have the same layout");
    VJ_CHECK((d_r_hashes == nullptr) == (d_s_hashes == nullptr), VJ_ERR_INVALID_ARGUMENT, "vj_build_probe: give hashes for both tables or neither");
    VJ_CHECK(hash_bits == 32 || hash_bits == 64, VJ_ERR_INVALID_ARGUMENT, "vj_build_probe: hash_bits must be 32 or 64");
    VJ_CUDA(cudaSetDevice(ctx->device));
    *count = 0;
    if (r->rows == 0 || s->rows == 0) return VJ_OK;
    VJ_CHECK(d_pairs != nullptr || capacity == 0, VJ_ERR_INVALID_ARGUMENT, "vj_build_probe: null output with capacity > 0");
    vj_result res{};
    res.pairs = d_pairs;
    res.capacity = capacity;
    res.owned = 0;
    // capacity 0 counts only: the kernels never write at or past the capacity
    JoinCall call;
    call.ctx = ctx;
    call.t.keys[0] = r->keys;
    call.t.keys[1] = s->keys;
    call.t.pay[0] = r->payloads;
    call.t.pay[1] = s->payloads;
    call.t.hash[0] = d_r_hashes;
    call.t.hash[1] = d_s_hashes;
    call.t.rows[0] = (uint32_t)r->rows;
    call.t.rows[1] = (uint32_t)s->rows;
    vj_join_options o{};
    o.hash_bits = hash_bits;
    call.hs = spec_from(&o, 1);
    call.opt = nullptr;
    call.res = &res;
    call.stream = (cudaStream_t)stream;
    // a caller buffer is never reallocated: mark it as caller-owned even at capacity 0
    res.owned = 0;
    BuildProbeCall cc{call};
    const int hs = d_r_hashes ? hash_bits / 8 : 0;
    VJ_TRY(dispatch(r->key_words, r->payload_bytes, hs, cc));
    *count = res.count;
    if (res.count > capacity) {
        return set_error(VJ_ERR_CAPACITY, "vj_build_probe: %llu pairs, capacity %llu", (unsigned long long)res.count, (unsigned long long)capacity);
    }
    return VJ_OK;
}

extern "C" int vj_partition(vj_ctx *ctx, const vj_table *in, const void *d_hashes_in, int hash_bits, int hash_algo, void *d_keys_out, void *d_payloads_out, void *d_hashes_out, int radix_shift, int radix_bits,
                            uint64_t *d_histogram, uint64_t *d_offsets, uint64_t *h_histogram, uint64_t *h_offsets, vj_stream_t stream) {
    VJ_CHECK(ctx != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_partition: null context");
    VJ_TRY(check_table(in, "vj_partition: in"));
    VJ_CHECK(radix_bits >= 1 && radix_bits <= MAX_RADIX_BITS, VJ_ERR_UNSUPPORTED, "vj_partition: radix_bits must be in [1, %d]", MAX_RADIX_BITS);
    VJ_CHECK(hash_bits == 32 || hash_bits == 64, VJ_ERR_INVALID_ARGUMENT, "vj_partition: hash_bits must be 32 or 64");
    VJ_CHECK(radix_shift >= 0 && radix_shift < 64, VJ_ERR_INVALID_ARGUMENT, "vj_partition: radix_shift must be in [0, 63]");
    VJ_CHECK(hash_algo >= 0 && hash_algo < VJ_HASH_COUNT, VJ_ERR_INVALID_ARGUMENT, "vj_partition: unknown hash algorithm %d", hash_algo);
    VJ_CHECK(in->rows == 0 || (d_keys_out && d_payloads_out), VJ_ERR_INVALID_ARGUMENT, "vj_partition: null output column");
    VJ_CUDA(cudaSetDevice(ctx->device));
    PartitionCall call;
    call.ctx = ctx;
    call.in = in;
    call.hashes = d_hashes_in;
    call.hs.algo = hash_algo;
    call.hs.hash_bits = hash_bits;
    call.hs.mix = 0;
    call.ko = d_keys_out;
    call.po = d_payloads_out;
    call.ho = d_hashes_in ? d_hashes_out : nullptr;
    call.shift = radix_shift;
    call.bits = radix_bits;
    call.dh = d_histogram;
    call.doff = d_offsets;
    call.hh = h_histogram;
    call.hoff = h_offsets;
    call.stream = (cudaStream_t)stream;
    return dispatch(in->key_words, in->payload_bytes, d_hashes_in ? hash_bits / 8 : 0, call);
}

// Copies n words between the device and page-locked, mapped host memory with SM loads and
// stores, eight loads in flight per thread. The copy engines' transfers to and from host
// memory stall now and then on this platform (1 GB taking 40-60 ms instead of 5 at times,
// with or without other GPU work), and a copy to the host can hold the calling thread until
// it ends; loads and stores from a few SMs, which keep many host pages in flight at once,
// hold the link rate (~210 GB/s in, ~190 out) throughout and never block the host.
template <typename V>
__global__ void __launch_bounds__(512) host_copy_kernel(const V *__restrict__ src, V *__restrict__ dst, size_t n) {
    constexpr int U = 8;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < n; i += U * stride) {
        V v[U];
#pragma unroll
        for (int u = 0; u < U; u++) v[u] = src[i + u * stride];
#pragma unroll
        for (int u = 0; u < U; u++) dst[i + u * stride] = v[u];
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

namespace {

// Blocks of host_copy_kernel: 16 x 512 threads x 8 loads of 16 bytes (1 MB in flight) fill
// the link alone; beside the joins they overlap, 32 keep more of it (the 2^27 x 2^29 join
// from host tables: 71.6 ms with 32, 75.7 with 16, no better with 64), and the other SMs
// stay with the joins.
constexpr int HOST_COPY_BLOCKS = 32;
// SMs vj_join_host's joins leave to the copy kernels: both directions' blocks at 4 a SM
constexpr int HOST_COPY_SMS = 2 * HOST_COPY_BLOCKS / 4;

// Device address of host memory [p, p + bytes) that the GPU can load from (page-locked and
// mapped, both ends in the same mapping), or null.
const char *mapped_host(const void *p, size_t bytes) {
    if (!p || bytes == 0) return nullptr;
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    if (cudaPointerGetAttributes(&b, (const char *)p + bytes - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (b.type != cudaMemoryTypeHost || (const char *)b.devicePointer != (const char *)a.devicePointer + bytes - 1) return nullptr;
    return (const char *)a.devicePointer;
}

// SM copy of bytes between device addresses (one side a host mapping), in the widest words
// that the addresses and the size allow.
cudaError_t sm_copy(void *dst, const void *dsrc, size_t bytes, cudaStream_t stream) {
    const uintptr_t al = (uintptr_t)dsrc | (uintptr_t)dst | (uintptr_t)bytes;
    const dim3 grid(HOST_COPY_BLOCKS), block(512);
    if ((al & 15) == 0) {
        host_copy_kernel<uint4><<<grid, block, 0, stream>>>((const uint4 *)dsrc, (uint4 *)dst, bytes / 16);
    } else if ((al & 7) == 0) {
        host_copy_kernel<uint2><<<grid, block, 0, stream>>>((const uint2 *)dsrc, (uint2 *)dst, bytes / 8);
    } else if ((al & 3) == 0) {
        host_copy_kernel<uint32_t><<<grid, block, 0, stream>>>((const uint32_t *)dsrc, (uint32_t *)dst, bytes / 4);
    } else {
        host_copy_kernel<uint8_t><<<grid, block, 0, stream>>>((const uint8_t *)dsrc, (uint8_t *)dst, bytes);
    }
    return cudaGetLastError();
}

// Host-to-device copy: SM loads for mapped page-locked memory, the copy engine otherwise
// (pageable memory, which it stages itself).
cudaError_t copy_in(void *dst, const void *src, size_t bytes, cudaStream_t stream) {
    if (bytes == 0) return cudaSuccess;
    const char *dsrc = mapped_host(src, bytes);
    if (!dsrc) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
    return sm_copy(dst, dsrc, bytes, stream);
}

// Device-to-host copy: SM stores for mapped page-locked memory, the copy engine otherwise.
cudaError_t copy_out(void *dst, const void *src, size_t bytes, cudaStream_t stream) {
    if (bytes == 0) return cudaSuccess;
    char *ddst = (char *)mapped_host(dst, bytes);
    if (!ddst) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream);
    return sm_copy(ddst, src, bytes, stream);
}

// A join into a caller's device buffer that is never reallocated, capacity 0 included
// (counts only: the kernels write nothing at or past the capacity).
int join_into(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, void *d_pairs, uint64_t capacity, uint64_t *count, cudaStream_t stream) {
    *count = 0;
    if (r->rows == 0 || s->rows == 0) return VJ_OK;
    vj_result res{};
    res.pairs = d_pairs;
    res.capacity = capacity;
    res.owned = 0;
    JoinCall call;
    call.ctx = ctx;
    call.t.keys[0] = r->keys;
    call.t.keys[1] = s->keys;
    call.t.pay[0] = r->payloads;
    call.t.pay[1] = s->payloads;
    call.t.hash[0] = call.t.hash[1] = nullptr;
    call.t.rows[0] = (uint32_t)r->rows;
    call.t.rows[1] = (uint32_t)s->rows;
    call.hs = spec_from(options, 1);
    call.opt = tuned_options(ctx, r, s, options);
    call.res = &res;
    call.stream = stream;
    BuildProbeCall cc{call};
    VJ_TRY(dispatch(r->key_words, r->payload_bytes, 0, cc));
    *count = res.count;
    return VJ_OK;
}

// ------------------------------------------------------------------ chunked probe side
//
// vj_join_host's pipeline joins the whole build side with one probe-side chunk at a time.
// The build side is partitioned once, when it has landed; each chunk is partitioned on its
// own (the plan's passes, one side per launch) and probed against the build side's
// partitions. Partitions p of both sides hold the same hash range whichever launch made
// them, so the items of partition p pair the build rows [r_begin[p], r_end[p]) with the
// chunk's rows [s_begin[p], s_end[p]).

struct ChunkJoiner {
    virtual ~ChunkJoiner() = default;
    // plans the join of r with a probe side of s_rows rows in chunks of at most max_chunk
    // rows, and partitions r (r's rows must be on the device in stream order)
    virtual int build(cudaStream_t stream) = 0;
    // joins r with one chunk into (out, room); *count = all its pairs (synchronises)
    virtual int probe(const vj_table &chunk, void *out, uint64_t room, uint64_t *count, cudaStream_t stream) = 0;
};

// Workspace of one side's passes.
struct SideBufs {
    void *rows[2] = {nullptr, nullptr};  // partition buffer of each pass
    uint16_t *bids = nullptr;             // pass-2 buckets written by pass 1
    PassBufs pb[2] = {};
};

template <int KW, int PB, int HS>
struct ChunkJoinerT final : ChunkJoiner {
    using L = Layout<KW, PB, HS>;
    vj_ctx *ctx;
    vj_table r;
    uint64_t s_rows;
    uint32_t max_chunk;
    HashSpec hs;
    const vj_join_options *opt;
    Plan pl;
    bool direct = false;  // no radix pass: each chunk is joined whole
    int np = 1;
    SideBufs rb, sb;
    const uint32_t *r_begin = nullptr, *r_end = nullptr;
    uint32_t *item_begin = nullptr, *ticket = nullptr, *error = nullptr;
    uint4 *item_desc = nullptr;
    unsigned long long *plan_blocks = nullptr, *out_count = nullptr;
    uint64_t item_cap = 0;

    void carve_side(Carver &c, uint32_t rows, SideBufs *b) const {
        for (int pass = 0; pass < 2; pass++) b->rows[pass] = pl.passes > pass ? c.take<char>((size_t)rows * L::STRIDE + 64) : nullptr;
        b->bids = pl.passes >= 2 ? c.take<uint16_t>((size_t)rows + 8) : nullptr;
        for (int pass = 0; pass < pl.passes; pass++) {
            const int G = pass == 0 ? 1 : 1 << pl.bits[0];
            b->pb[pass] = carve_pass(c, G, 1 << pl.bits[pass], pass_units(ctx->info, rows, G, tail_split(ctx->info)));
        }
    }

    void layout(Carver &c) {
        carve_side(c, (uint32_t)r.rows, &rb);
        carve_side(c, max_chunk, &sb);
        item_begin = c.take<uint32_t>((size_t)np + 2);
        plan_blocks = c.take<unsigned long long>(((size_t)np + PLAN_BLOCK - 1) / PLAN_BLOCK);
        item_desc = c.take<uint4>(item_cap);
        ticket = c.take<uint32_t>(1);
        out_count = c.take<unsigned long long>(1);
        error = c.take<uint32_t>(1);
    }

    // The plan's passes over one table; its partitions are rows [begin[p], end[p]) of the
    // last pass's buffer.
    int partition(const void *keys, const void *pay, uint32_t rows, const SideBufs &b, cudaStream_t stream, const uint32_t **begin, const uint32_t **end) {
        const uint32_t *seg_begin = nullptr, *seg_end = nullptr;
        int Q = 1, consumed = 0;
        for (int pass = 0; pass < pl.passes; pass++) {
            PassParams P{};
            P.side[0].keys_in = keys;
            P.side[0].pay_in = pay;
            P.side[0].hash_in = nullptr;
            P.side[0].rows_in = pass > 0 ? b.rows[pass - 1] : nullptr;
            P.side[0].rows_out = b.rows[pass];
            P.side[0].rows = rows;
            P.side[0].bid_out = pass == 0 && pl.passes >= 2 ? b.bids : nullptr;
            P.side[0].bid_in = pass == 1 ? b.bids : nullptr;
            P.next_shift = 64 - (pl.bits[0] + pl.bits[1]);
            P.next_bits = pl.bits[1];
            P.nsides = 1;
            P.Q = Q;
            P.seg_begin = seg_begin;
            P.seg_end = seg_end;
            P.bits = pl.bits[pass];
            consumed += pl.bits[pass];
            P.shift = 64 - consumed;
            P.hs = hs;
            P.max_units = b.pb[pass].max_units;
            P.min_unit_rows = MIN_UNIT_ROWS;
            P.split = tail_split(ctx->info);
            P.next_split = tail_split(ctx->info);
            P.error = error;
            if (pass == 0) {
                host_plan(P, &rows, 1);
                if (pl.passes >= 2) {
                    P.next_plan = b.pb[1].plan;
                    P.next_max_units = b.pb[1].max_units;
                }
                VJ_TRY((run_pass<KW, PB, HS, false, true>(ctx, ctx->info.sms - ctx->sm_reserve, pass, P, b.pb[0], stream)));
            } else {
                P.plan = b.pb[1].plan;
                VJ_TRY((run_pass<KW, PB, HS, true, true>(ctx, ctx->info.sms - ctx->sm_reserve, pass, P, b.pb[1], stream)));
            }
            seg_begin = b.pb[pass].part_begin;
            seg_end = b.pb[pass].part_end;
            Q <<= pl.bits[pass];
        }
        *begin = seg_begin;
        *end = seg_end;
        return VJ_OK;
    }

    int build(cudaStream_t stream) override {
        pl = make_plan<KW, PB, HS>(r.rows, s_rows, ctx->info, opt);
        if (pl.passes == 0) {
            direct = true;
            return VJ_OK;
        }
        np = pl.passes == 1 ? 1 << pl.bits[0] : 1 << (pl.bits[0] + pl.bits[1]);
        item_cap = (uint64_t)np + max_chunk / pl.schunk + r.rows / pl.rcap + 4096;
        Carver dry;
        layout(dry);
        void *ws = nullptr;
        VJ_TRY(workspace_reserve(ctx, dry.off + 256, stream, &ws));
        Carver c;
        c.base = (char *)ws;
        layout(c);
        VJ_CUDA(cudaMemsetAsync(error, 0, sizeof(uint32_t), stream));
        return partition(r.keys, r.payloads, (uint32_t)r.rows, rb, stream, &r_begin, &r_end);
    }

    int probe(const vj_table &chunk, void *out, uint64_t room, uint64_t *count, cudaStream_t stream) override {
        *count = 0;
        if (direct) return join_into(ctx, &r, &chunk, opt, out, room, count, stream);
        if (chunk.rows == 0 || r.rows == 0) return VJ_OK;
        ctx->launches = 0;
        const uint32_t *s_begin = nullptr, *s_end = nullptr;
        VJ_TRY(partition(chunk.keys, chunk.payloads, (uint32_t)chunk.rows, sb, stream, &s_begin, &s_end));
        ProbeParams Pq{};
        Pq.r_keys = r.keys;
        Pq.r_pay = r.payloads;
        Pq.s_keys = chunk.keys;
        Pq.s_pay = chunk.payloads;
        Pq.r_rows_in = rb.rows[pl.passes - 1];
        Pq.s_rows_in = sb.rows[pl.passes - 1];
        Pq.r_begin = r_begin;
        Pq.r_end = r_end;
        Pq.s_begin = s_begin;
        Pq.s_end = s_end;
        Pq.r_rows = (uint32_t)r.rows;
        Pq.s_rows = (uint32_t)chunk.rows;
        Pq.np = np;
        Pq.rcap = pl.rcap;
        Pq.schunk = pl.schunk;
        Pq.tcap = pl.tcap;
        Pq.tmul = pl.tmul;
        Pq.scap = pl.scap;
        Pq.slot_shift = 64 - (pl.bits[0] + pl.bits[1]) - 14;
        Pq.item_begin = item_begin;
        Pq.item_desc = item_desc;
        Pq.item_cap = (uint32_t)(item_cap < 0xffffffffull ? item_cap : 0xffffffffull);
        Pq.ticket = ticket;
        Pq.out_count = out_count;
        Pq.hs = hs;
        Pq.error = error;
        Pq.joins = 1;
        Pq.out = out;
        Pq.capacity = room;
        JoinRun run;
        run.probe = Pq;
        run.plan_blocks = plan_blocks;
        run.d_out_count = out_count;
        run.d_error = error;
        VJ_TRY((probe_setup<KW, PB, HS, true, false>(ctx, pl, &run)));
        VJ_TRY((launch_probe<KW, PB, HS>(ctx, run, stream)));
        uint32_t flags = 0;
        VJ_TRY(read_count(ctx, run, stream, count, &flags));
        VJ_TRY(check_flags(flags));
        finish_profile(ctx, pl, r.rows, chunk.rows, *count);
        return VJ_OK;
    }
};

struct MakeChunkJoiner {
    vj_ctx *ctx;
    const vj_table *r;
    uint64_t s_rows;
    uint32_t max_chunk;
    const vj_join_options *opt;
    std::unique_ptr<ChunkJoiner> *out;
    template <int KW, int PB, int HS>
    int run() {
        auto j = std::make_unique<ChunkJoinerT<KW, PB, HS>>();
        j->ctx = ctx;
        j->r = *r;
        j->s_rows = s_rows;
        j->max_chunk = max_chunk;
        j->hs = spec_from(opt, 1);
        j->opt = opt;
        *out = std::move(j);
        return VJ_OK;
    }
};

// Probe-side chunks of vj_join_host's pipeline. A chunk's join (the whole build side and
// the chunk) takes about as long as the copy of one build side's worth of probe rows, so
// chunks of about |R| rows keep the link busy; 1 (no pipeline) for a probe side under
// twice the build side or a join too small to gain from it.
int host_chunks(uint64_t r_rows, uint64_t s_rows) {
    const uint64_t min_chunk = 1ull << 22;
    if (r_rows == 0 || s_rows < 2 * r_rows || s_rows < 2 * min_chunk) return 1;
    uint64_t c = (s_rows + r_rows / 2) / r_rows;
    if (s_rows / c < min_chunk) c = s_rows / min_chunk;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(c, 16));
}

int host_streams(vj_ctx *ctx) {
    if (ctx->host_ready) return VJ_OK;
    cudaStream_t in = nullptr, out = nullptr;
    cudaEvent_t ev[sizeof(ctx->host_ev) / sizeof(ctx->host_ev[0])] = {};
    const int n = (int)(sizeof(ev) / sizeof(ev[0]));
    // copies at the highest priority: their few blocks are scheduled ahead of the joins'
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&in, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&out, cudaStreamNonBlocking, greatest);
    for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (int i = 0; i < n; i++)
            if (ev[i]) cudaEventDestroy(ev[i]);
        if (in) cudaStreamDestroy(in);
        if (out) cudaStreamDestroy(out);
        return cuda_error(e, "vj_join_host: copy streams");
    }
    ctx->host_in = in;
    ctx->host_out = out;
    for (int i = 0; i < n; i++) ctx->host_ev[i] = ev[i];
    ctx->host_ready = true;
    return VJ_OK;
}

// vj_join_host with the probe side in chunks: the build side and the chunks are copied in
// on one stream, each chunk is joined with the whole build side on the caller's stream as
// soon as it has landed, and each chunk's pairs are copied out on a third stream while the
// next chunk is joined. The host link carries both directions at once, so copies in, joins
// and copies out overlap. R ⋈ S is the union of the R ⋈ S_i; each chunk's pairs follow the
// previous chunks' in the output.
int join_host_chunked(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, void *h_pairs, uint64_t capacity, uint64_t *count, cudaStream_t st, int chunks, char *rk,
                      char *rp, char *sk, char *sp, char *dpairs) {
    VJ_TRY(host_streams(ctx));
    // The join kernels leave HOST_COPY_SMS SMs to the copy kernels: persistent join kernels
    // fill every SM's registers, and copy blocks that cannot start stall the host link.
    struct Reserve {
        vj_ctx *c;
        explicit Reserve(vj_ctx *x) : c(x) { c->sm_reserve = std::min(HOST_COPY_SMS, c->info.sms / 4); }
        ~Reserve() { c->sm_reserve = 0; }
    } reserve(ctx);
    const size_t kb = (size_t)r->key_words * 4, pb = (size_t)r->payload_bytes;
    cudaEvent_t ev_start = ctx->host_ev[0], ev_in = ctx->host_ev[1], ev_out = ctx->host_ev[2], ev_r = ctx->host_ev[3];
    cudaEvent_t *ev_s = ctx->host_ev + 4, *ev_j = ctx->host_ev + 4 + 16;
    cudaStream_t in = ctx->host_in, out = ctx->host_out;
    // Chunk i weighs 2 (chunks + 1) - i: later chunks are smaller, so the join and the copy
    // out left after the last chunk has landed are short (4 chunks of 29, 26, 24 and 21 % of
    // the probe side: 71.6 ms for the 2^27 x 2^29 join, 4 equal chunks 73.9 ms). Bounds on
    // multiples of 64 rows keep every chunk's copy as aligned as the table.
    const uint64_t C = (uint64_t)chunks;
    auto weight_below = [&](uint64_t i) -> uint64_t { return i * (4 * (C + 1) - i + 1) / 2; };
    auto begin = [&](int i) -> uint64_t { return i == chunks ? s->rows : (s->rows * weight_below((uint64_t)i) / weight_below(C)) & ~(uint64_t)63; };
    // copies in: the build side, then the chunks (ev_s[i]: chunk i and all before it landed)
    VJ_CUDA(cudaEventRecord(ev_start, st));  // after whatever the caller queued before
    cudaError_t e = cudaStreamWaitEvent(in, ev_start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(out, ev_start, 0);
    if (e == cudaSuccess) e = copy_in(rk, r->keys, r->rows * kb, in);
    if (e == cudaSuccess) e = copy_in(rp, r->payloads, r->rows * pb, in);
    if (e == cudaSuccess) e = cudaEventRecord(ev_r, in);
    uint32_t max_chunk = 0;
    for (int i = 0; i < chunks && e == cudaSuccess; i++) {
        const uint64_t a = begin(i), n = begin(i + 1) - a;
        max_chunk = std::max<uint32_t>(max_chunk, (uint32_t)n);
        e = copy_in(sk + a * kb, (const char *)s->keys + a * kb, n * kb, in);
        if (e == cudaSuccess) e = copy_in(sp + a * pb, (const char *)s->payloads + a * pb, n * pb, in);
        if (e == cudaSuccess) e = cudaEventRecord(ev_s[i], in);
    }
    int status = e == cudaSuccess ? VJ_OK : cuda_error(e, "vj_join_host: copies to the device");
    vj_table dr = *r;
    dr.keys = rk;
    dr.payloads = rp;
    // the build side is partitioned once, as soon as it has landed
    std::unique_ptr<ChunkJoiner> joiner;
    if (status == VJ_OK) {
        MakeChunkJoiner mk{ctx, &dr, s->rows, max_chunk, tuned_options(ctx, r, s, options), &joiner};
        status = dispatch(r->key_words, r->payload_bytes, 0, mk);
    }
    if (status == VJ_OK) {
        e = cudaStreamWaitEvent(st, ev_r, 0);
        status = e == cudaSuccess ? joiner->build(st) : cuda_error(e, "vj_join_host: stream order");
    }
    uint64_t off = 0, total = 0;
    bool over = false;
    for (int i = 0; i < chunks && status == VJ_OK; i++) {
        const uint64_t a = begin(i);
        vj_table ds = *s;
        ds.keys = sk + a * kb;
        ds.payloads = sp + a * pb;
        ds.rows = begin(i + 1) - a;
        e = cudaStreamWaitEvent(st, ev_s[i], 0);
        if (e != cudaSuccess) {
            status = cuda_error(e, "vj_join_host: stream order");
            break;
        }
        // once the output is full the remaining chunks are counted only
        const uint64_t room = over ? 0 : capacity - off;
        uint64_t n = 0;
        status = joiner->probe(ds, dpairs + off * 2 * pb, room, &n, st);
        if (status != VJ_OK) break;
        total += n;
        if (over || n > room) {
            over = true;
            continue;
        }
        if (n) {
            e = cudaEventRecord(ev_j[i], st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(out, ev_j[i], 0);
            if (e == cudaSuccess) e = copy_out((char *)h_pairs + off * 2 * pb, dpairs + off * 2 * pb, n * 2 * pb, out);
            if (e != cudaSuccess) status = cuda_error(e, "vj_join_host: copy of pairs to the host");
        }
        off += n;
    }
    // the caller's stream takes over the completion of both copy streams, after an error
    // too, so that no copy into the staging buffer outlives the call
    e = cudaEventRecord(ev_in, in);
    if (e == cudaSuccess) e = cudaEventRecord(ev_out, out);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_in, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_out, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (status != VJ_OK) return status;
    if (e != cudaSuccess) return cuda_error(e, "vj_join_host: pipeline");
    *count = total;
    if (over) {
        return set_error(VJ_ERR_CAPACITY, "vj_join_host: %llu pairs, capacity %llu", (unsigned long long)total, (unsigned long long)capacity);
    }
    return VJ_OK;
}

}  // namespace

extern "C" int vj_join_host(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *options, void *h_pairs, uint64_t capacity, uint64_t *count, vj_stream_t stream) {
    VJ_CHECK(ctx && count, VJ_ERR_INVALID_ARGUMENT, "vj_join_host: null argument");
    VJ_TRY(check_table(r, "vj_join_host: r"));
    VJ_TRY(check_table(s, "vj_join_host: s"));
    VJ_CHECK(r->key_words == s->key_words && r->payload_bytes == s->payload_bytes, VJ_ERR_INVALID_ARGUMENT, "vj_join_host: r and s must have the same layout");
    VJ_TRY(check_options(options, "vj_join_host"));
    VJ_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    *count = 0;
    const size_t kb = (size_t)r->key_words * 4, pb = (size_t)r->payload_bytes;
    // one cached device buffer holds both tables and the output pairs
    const size_t need = (r->rows + s->rows) * (kb + pb) + (size_t)capacity * 2 * pb + 6 * 256;
    if (ctx->stage_bytes < need) {
        if (ctx->stage) {
            VJ_CUDA(cudaFreeAsync(ctx->stage, st));
            ctx->stage = nullptr;
            ctx->stage_bytes = 0;
        }
        VJ_CHECK(!ctx->budget || ctx->owned_bytes + ctx->workspace_bytes + need <= ctx->budget, VJ_ERR_BUDGET, "vj_join_host: staging exceeds the context budget");
        VJ_CUDA(cudaMallocAsync(&ctx->stage, need, st));
        note_allocation();
        ctx->stage_bytes = need;
    }
    Carver c;
    c.base = (char *)ctx->stage;
    void *rk = c.take<char>(r->rows * kb), *rp = c.take<char>(r->rows * pb);
    void *sk = c.take<char>(s->rows * kb), *sp = c.take<char>(s->rows * pb);
    void *dpairs = c.take<char>((size_t)capacity * 2 * pb);
    const int chunks = capacity > 0 ? host_chunks(r->rows, s->rows) : 1;
    if (chunks > 1) {
        VJ_CHECK(h_pairs != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_join_host: null output");
        return join_host_chunked(ctx, r, s, options, h_pairs, capacity, count, st, chunks, (char *)rk, (char *)rp, (char *)sk, (char *)sp, (char *)dpairs);
    }
    VJ_CUDA(copy_in(rk, r->keys, r->rows * kb, st));
    VJ_CUDA(copy_in(rp, r->payloads, r->rows * pb, st));
    VJ_CUDA(copy_in(sk, s->keys, s->rows * kb, st));
    VJ_CUDA(copy_in(sp, s->payloads, s->rows * pb, st));
    vj_table dr = *r, ds = *s;
    dr.keys = rk;
    dr.payloads = rp;
    ds.keys = sk;
    ds.payloads = sp;
    vj_result res{};
    if (capacity > 0) {
        res.pairs = dpairs;
        res.capacity = capacity;
    } else {
        res.pairs = nullptr;  // count only: library-owned buffer, never copied back
    }
    int status = vj_join(ctx, &dr, &ds, options, &res, stream);
    *count = res.count;
    if (status == VJ_ERR_CAPACITY) {
        return status;
    }
    VJ_TRY(status);
    if (res.count > capacity) {
        status = set_error(VJ_ERR_CAPACITY, "vj_join_host: %llu pairs, capacity %llu", (unsigned long long)res.count, (unsigned long long)capacity);
    } else if (res.count) {
        VJ_CHECK(h_pairs != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_join_host: null output");
        cudaError_t e = copy_out(h_pairs, res.pairs, res.count * 2 * pb, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) status = cuda_error(e, "vj_join_host: copy of pairs to the host");
    }
    if (res.owned) {
        vj_result_free(ctx, &res);
    }
    return status;
}

// ------------------------------------------------------------------ vj_partition_noalloc
//
// A radix pass for callers that cannot allocate device memory (an engine whose own pool
// holds all of HBM, or one that cannot let cudaFree synchronise a device its other streams
// are using). The pass's working memory lives in the static array below instead of a
// context workspace; everything else is the vj_partition sequence.

// Working memory of vj_partition_noalloc, one copy per device that loads the library. In
// host code this name stands for a host-side shadow, not for device memory: host code
// passes kernels the address cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[VJ_NOALLOC_SCRATCH_BYTES];

namespace vj {
namespace {

std::mutex g_noalloc_mutex;
char *g_noalloc_base[64];

// Device address of the scratch on `device` (the current device), looked up on the first
// call for that device and kept for the life of the process.
int noalloc_scratch(int device, char **out) {
    VJ_CHECK(device >= 0 && device < (int)(sizeof(g_noalloc_base) / sizeof(g_noalloc_base[0])), VJ_ERR_UNSUPPORTED, "vj_partition_noalloc: device %d is beyond the %d devices it keeps scratch addresses for", device,
             (int)(sizeof(g_noalloc_base) / sizeof(g_noalloc_base[0])));
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            return cuda_error(e, "vj_partition_noalloc: device address of the static scratch");
        }
        g_noalloc_base[device] = (char *)p;
    }
    *out = g_noalloc_base[device];
    return VJ_OK;
}

struct NoallocLayout {
    PassBufs pb;
    unsigned long long *hist, *off;
    uint32_t *err;
};

NoallocLayout noalloc_layout(Carver &c, int bins, int units) {
    NoallocLayout L;
    L.pb = carve_pass(c, 1, bins, units);
    L.hist = c.take<unsigned long long>(bins);
    L.off = c.take<unsigned long long>(bins);
    L.err = c.take<uint32_t>(1);
    return L;
}

// Work units of the pass: as many as vj_partition uses for these rows, fewer when their
// look-back words (8 bytes per bucket per unit) would not fit in the scratch.
// 0: not even two units fit.
int noalloc_units(const DeviceInfo &info, uint64_t rows, int bins) {
    Carver fixed;
    noalloc_layout(fixed, bins, 0);
    const size_t per_unit = sizeof(unsigned long long) * (size_t)bins;
    const size_t slack = 256;  // alignment of the per-unit array
    const size_t room = VJ_NOALLOC_SCRATCH_BYTES > fixed.off + slack ? VJ_NOALLOC_SCRATCH_BYTES - fixed.off - slack : 0;
    size_t units = room / per_unit;
    const size_t want = (size_t)pass_units(info, rows, 1);
    if (units > want) units = want;
    Carver check;
    noalloc_layout(check, bins, (int)units);
    return units >= 2 && check.off <= VJ_NOALLOC_SCRATCH_BYTES ? (int)units : 0;
}

template <int KW, int PB, int HS>
int partition_noalloc_typed(char *scratch, int sms, int units, const vj_table *in, const void *hashes_in, const HashSpec &hs, void *keys_out, void *pay_out, void *hash_out, int shift, int bits, uint64_t *d_hist,
                            uint64_t *d_off, uint64_t *h_hist, uint64_t *h_off, cudaStream_t stream) {
    const int bins = 1 << bits;
    Carver c;
    c.base = scratch;
    const NoallocLayout L = noalloc_layout(c, bins, units);
    // The scratch holds whatever the previous call left. The error flag must start at zero;
    // the pass clears its own counters and bucket totals and overwrites every other array
    // before use.
    VJ_CUDA(cudaMemsetAsync(L.err, 0, sizeof(uint32_t), stream));
    PassParams P{};
    P.side[0].keys_in = in->keys;
    P.side[0].pay_in = in->payloads;
    P.side[0].hash_in = hashes_in;
    P.side[0].rows_in = nullptr;
    P.side[0].rows_out = nullptr;
    P.side[0].keys_out = keys_out;
    P.side[0].pay_out = pay_out;
    P.side[0].hash_out = hash_out;
    P.side[0].rows = (uint32_t)in->rows;
    P.nsides = 1;
    P.Q = 1;
    P.seg_begin = P.seg_end = nullptr;
    P.shift = shift;
    P.bits = bits;
    P.hs = hs;
    P.max_units = units;
    P.min_unit_rows = MIN_UNIT_ROWS;
    P.error = L.err;
    const uint32_t rows = (uint32_t)in->rows;
    host_plan(P, &rows, 1);
    // an empty table still has one (empty) unit, which writes the empty bounds
    VJ_TRY((run_pass<KW, PB, HS, false, false>(nullptr, sms, 0, P, L.pb, stream)));
    unsigned long long *hist = d_hist ? (unsigned long long *)d_hist : L.hist;
    unsigned long long *off = d_off ? (unsigned long long *)d_off : L.off;
    export_hist_kernel<<<(bins + 255) / 256, 256, 0, stream>>>(L.pb.part_begin, L.pb.part_end, bins, hist, off, L.err);
    VJ_CUDA(cudaGetLastError());
    if (h_hist || h_off) {
        if (h_hist) VJ_CUDA(cudaMemcpyAsync(h_hist, hist, bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
        if (h_off) VJ_CUDA(cudaMemcpyAsync(h_off, off, bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
        uint32_t herr = 0;
        VJ_CUDA(cudaMemcpyAsync(&herr, L.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        VJ_CUDA(cudaStreamSynchronize(stream));
        VJ_CHECK(herr == 0, VJ_ERR_DEVICE, "vj_partition_noalloc: a kernel reported an internal limit (flags %x)", herr);
    }
    return VJ_OK;
}

struct NoallocPartitionCall {
    char *scratch;
    int sms;
    int units;
    const vj_table *in;
    const void *hashes;
    HashSpec hs;
    void *ko, *po, *ho;
    int shift, bits;
    uint64_t *dh, *doff, *hh, *hoff;
    cudaStream_t stream;
    template <int KW, int PB, int HS>
    int run() {
        return partition_noalloc_typed<KW, PB, HS>(scratch, sms, units, in, hashes, hs, ko, po, ho, shift, bits, dh, doff, hh, hoff, stream);
    }
};

}  // namespace
}  // namespace vj

extern "C" int vj_partition_noalloc(const vj_table *in, const void *d_hashes_in, int hash_bits, int hash_algo, void *d_keys_out, void *d_payloads_out, void *d_hashes_out, int radix_shift, int radix_bits,
                                    uint64_t *d_histogram, uint64_t *d_offsets, uint64_t *h_histogram, uint64_t *h_offsets, vj_stream_t stream) {
    // every argument is checked before the first CUDA call
    VJ_TRY(check_table(in, "vj_partition_noalloc: in"));
    VJ_CHECK(radix_bits >= 1 && radix_bits <= VJ_NOALLOC_MAX_RADIX_BITS, VJ_ERR_UNSUPPORTED,
             "vj_partition_noalloc: radix_bits %d is outside [1, %d], the buckets its %u-byte static scratch holds (vj_partition takes up to %d)", radix_bits, VJ_NOALLOC_MAX_RADIX_BITS,
             (unsigned)VJ_NOALLOC_SCRATCH_BYTES, MAX_RADIX_BITS);
    VJ_CHECK(hash_bits == 32 || hash_bits == 64, VJ_ERR_INVALID_ARGUMENT, "vj_partition_noalloc: hash_bits must be 32 or 64");
    VJ_CHECK(radix_shift >= 0 && radix_shift < 64, VJ_ERR_INVALID_ARGUMENT, "vj_partition_noalloc: radix_shift must be in [0, 63]");
    VJ_CHECK(hash_algo >= 0 && hash_algo < VJ_HASH_COUNT, VJ_ERR_INVALID_ARGUMENT, "vj_partition_noalloc: unknown hash algorithm %d", hash_algo);
    VJ_CHECK(in->rows == 0 || (d_keys_out && d_payloads_out), VJ_ERR_INVALID_ARGUMENT, "vj_partition_noalloc: null output column");
    int device = 0;
    VJ_CUDA(cudaGetDevice(&device));
    DeviceInfo info;
    VJ_TRY(device_info(device, &info));
    NoallocPartitionCall call;
    VJ_TRY(noalloc_scratch(device, &call.scratch));
    call.sms = info.sms;
    call.units = noalloc_units(info, in->rows, 1 << radix_bits);
    VJ_CHECK(call.units > 0, VJ_ERR_UNSUPPORTED, "vj_partition_noalloc: %d buckets do not fit the %u-byte static scratch", 1 << radix_bits, (unsigned)VJ_NOALLOC_SCRATCH_BYTES);
    call.in = in;
    call.hashes = d_hashes_in;
    call.hs.algo = hash_algo;
    call.hs.hash_bits = hash_bits;
    call.hs.mix = 0;
    call.ko = d_keys_out;
    call.po = d_payloads_out;
    call.ho = d_hashes_in ? d_hashes_out : nullptr;
    call.shift = radix_shift;
    call.bits = radix_bits;
    call.dh = d_histogram;
    call.doff = d_offsets;
    call.hh = h_histogram;
    call.hoff = h_offsets;
    call.stream = (cudaStream_t)stream;
    return dispatch(in->key_words, in->payload_bytes, d_hashes_in ? hash_bits / 8 : 0, call);
}
