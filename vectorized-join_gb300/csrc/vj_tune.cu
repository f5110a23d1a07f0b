// vj_tune.cu -- autotuner: times candidate plans of a join and keeps the fastest per shape
// class in the context; automatic joins of that class use it. The cache persists as text.
//
// The reference tunes by sweeping configuration grids from TOML files in separate benchmark
// runs (src/benchmark/configuration.hpp:200-305: bucket counts, vector sizes, kernel
// shapes); here the sweep runs on the caller's own tables, inside the library.
//
// Candidates: the planner's own choice; the same with a fuller table (load <= 1/4, 1/2)
// and with a smaller probe block (512 threads: one producer warp, 15 consumers); two
// passes with the bits split both ways around the total that fills shared-memory tables,
// and one bit more or less (with build tables sized to match); one pass where the total
// fits one pass.
#include "vj_internal.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace vj {

namespace {

int lg(uint64_t x) {
    int b = 0;
    while ((1ull << b) < x) b++;
    return b;
}

bool automatic(const vj_join_options *o) {
    if (!o) return true;
    return (o->flags & ~VJ_JOIN_BATCH_LAUNCHES) == 0 && o->passes == 0 && o->radix_bits[0] == 0 && o->radix_bits[1] == 0 && o->build_rows == 0 && o->probe_rows == 0 && o->probe_threads == 0 && o->probe_sub_rows == 0 &&
           o->table_load_pct == 0;
}

vj_join_options base_of(const vj_join_options *b) {
    vj_join_options o;
    memset(&o, 0, sizeof(o));
    if (b) {
        o.hash_algo = b->hash_algo;
        o.hash_bits = b->hash_bits;
    }
    return o;
}

std::vector<vj_join_options> candidates(const vj_table *r, const vj_join_options *base, int max_n) {
    std::vector<vj_join_options> c;
    const vj_join_options b = base_of(base);
    c.push_back(b);  // the planner's own choice
    for (int load : {25, 50}) {  // block shape and table load of the planner's plan
        vj_join_options o = b;
        o.table_load_pct = load;
        c.push_back(o);
    }
    {
        vj_join_options o = b;
        o.probe_threads = 512;
        c.push_back(o);
    }
    const int lr = lg(r->rows);
    const int total = lr > 10 ? lr - 10 : 0;  // partitions of ~1024 build rows: half a 2048-row table
    for (int t = total - 1; t <= total + 1; t++) {
        if (t < 2) continue;
        // build tables sized so the average partition fills about half of one
        const int rows_per_part = lr - t;
        int build = 1 << (rows_per_part + 1);
        if (build < 256) build = 256;
        if (build > 8192) build = 8192;
        if (t <= 12) {
            vj_join_options o = b;
            o.flags = VJ_JOIN_FIXED_PASSES | VJ_JOIN_SHARED_TABLES;
            o.passes = 1;
            o.radix_bits[0] = t;
            o.build_rows = build;
            c.push_back(o);
        }
        if (t >= 4 && t <= 24) {
            for (int first : {t / 2, t - t / 2}) {
                vj_join_options o = b;
                o.flags = VJ_JOIN_FIXED_PASSES | VJ_JOIN_SHARED_TABLES;
                o.passes = 2;
                o.radix_bits[0] = first;
                o.radix_bits[1] = t - first;
                o.build_rows = build;
                c.push_back(o);
                if (t % 2 == 0) break;  // an even total splits one way only
            }
        }
    }
    if ((int)c.size() > max_n) c.resize((size_t)max_n);
    return c;
}

}  // namespace

TuneKey tune_key(const vj_table *r, const vj_table *s, const vj_join_options *opt) {
    TuneKey k;
    k.kw = r->key_words;
    k.pb = r->payload_bytes;
    k.lg_r = lg(r->rows);
    k.lg_s = lg(s->rows);
    k.algo = opt && opt->hash_algo > 0 && opt->hash_algo < VJ_HASH_COUNT ? opt->hash_algo : VJ_HASH_FNV;
    k.hash_bits = opt && opt->hash_bits == 32 ? 32 : 64;
    return k;
}

const vj_join_options *tuned_options(const vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *opt) {
    if (!ctx || ctx->tuned.empty() || !automatic(opt)) return opt;
    const TuneKey k = tune_key(r, s, opt);
    for (const TuneEntry &e : ctx->tuned) {
        if (e.key == k) return &e.opt;
    }
    return opt;
}

}  // namespace vj

using namespace vj;

extern "C" int vj_tune(vj_ctx *ctx, const vj_table *r, const vj_table *s, const vj_join_options *base, void *d_pairs, uint64_t capacity, int max_candidates, vj_join_options *best, float *best_ms,
                       vj_stream_t stream) {
    VJ_CHECK(ctx && r && s, VJ_ERR_INVALID_ARGUMENT, "vj_tune: null argument");
    VJ_CHECK(r->rows > 0 && s->rows > 0, VJ_ERR_INVALID_ARGUMENT, "vj_tune: both tables need rows");
    VJ_CHECK(d_pairs != nullptr && capacity > 0, VJ_ERR_INVALID_ARGUMENT, "vj_tune: needs an output buffer");
    VJ_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    VJ_CUDA(cudaEventCreate(&e0));
    VJ_CUDA(cudaEventCreate(&e1));
    const std::vector<vj_join_options> cand = candidates(r, base, max_candidates > 0 ? max_candidates : 16);
    float top = INFINITY;
    vj_join_options win = cand[0];
    uint64_t first_count = UINT64_MAX;
    int status = VJ_OK;
    for (const vj_join_options &o : cand) {
        float t_min = INFINITY;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; rep++) {  // the first run warms the workspace
            vj_result res{};
            res.pairs = d_pairs;
            res.capacity = capacity;
            cudaEventRecord(e0, st);
            const int rc = vj_join(ctx, r, s, &o, &res, stream);  // explicit options: no cache lookup
            cudaEventRecord(e1, st);
            if (rc != VJ_OK) {
                ok = false;
                if (rc == VJ_ERR_CAPACITY) status = rc;  // the buffer is too small for this join
                break;
            }
            VJ_CUDA(cudaEventSynchronize(e1));
            if (first_count == UINT64_MAX) first_count = res.count;
            VJ_CHECK(res.count == first_count, VJ_ERR_DEVICE, "vj_tune: candidate plans disagree on the match count (%llu vs %llu)", (unsigned long long)res.count, (unsigned long long)first_count);
            float ms = 0.f;
            VJ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0 && ms < t_min) t_min = ms;
        }
        if (ok && t_min < top) {
            top = t_min;
            win = o;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status == VJ_ERR_CAPACITY && !std::isfinite(top)) return set_error(VJ_ERR_CAPACITY, "vj_tune: the output buffer holds fewer pairs than the join makes");
    VJ_CHECK(std::isfinite(top), VJ_ERR_DEVICE, "vj_tune: no candidate plan ran");
    const TuneKey k = tune_key(r, s, base);
    bool replaced = false;
    for (TuneEntry &e : ctx->tuned) {
        if (e.key == k) {
            e.opt = win;
            e.ms = top;
            replaced = true;
        }
    }
    if (!replaced) ctx->tuned.push_back(TuneEntry{k, win, top});
    if (best) *best = win;
    if (best_ms) *best_ms = top;
    return VJ_OK;
}

// One line per entry: key fields, then the options, then the time.
extern "C" int vj_tune_save(const vj_ctx *ctx, const char *path) {
    VJ_CHECK(ctx && path, VJ_ERR_INVALID_ARGUMENT, "vj_tune_save: null argument");
    FILE *f = fopen(path, "w");
    VJ_CHECK(f != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_tune_save: cannot write %s", path);
    fprintf(f, "# vj tuning cache: kw pb lg_r lg_s algo hash_bits | flags passes bits0 bits1 build_rows probe_rows threads table_load_pct | ms\n");
    for (const TuneEntry &e : ctx->tuned) {
        const vj_join_options &o = e.opt;
        fprintf(f, "%d %d %d %d %d %d | %d %d %d %d %d %d %d %d | %.4f\n", e.key.kw, e.key.pb, e.key.lg_r, e.key.lg_s, e.key.algo, e.key.hash_bits, o.flags, o.passes, o.radix_bits[0], o.radix_bits[1], o.build_rows,
                o.probe_rows, o.probe_threads, o.table_load_pct, e.ms);
    }
    const bool ok = fclose(f) == 0;
    VJ_CHECK(ok, VJ_ERR_INVALID_ARGUMENT, "vj_tune_save: cannot write %s", path);
    return VJ_OK;
}

extern "C" int vj_tune_load(vj_ctx *ctx, const char *path) {
    VJ_CHECK(ctx && path, VJ_ERR_INVALID_ARGUMENT, "vj_tune_load: null argument");
    FILE *f = fopen(path, "r");
    VJ_CHECK(f != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_tune_load: cannot read %s", path);
    char line[512];
    int loaded = 0, lineno = 0;
    while (fgets(line, sizeof line, f)) {
        lineno++;
        if (line[0] == '#' || line[0] == '\n') continue;
        TuneEntry e;
        memset(&e, 0, sizeof(e));
        vj_join_options &o = e.opt;
        const int n = sscanf(line, "%d %d %d %d %d %d | %d %d %d %d %d %d %d %d | %f", &e.key.kw, &e.key.pb, &e.key.lg_r, &e.key.lg_s, &e.key.algo, &e.key.hash_bits, &o.flags, &o.passes, &o.radix_bits[0],
                             &o.radix_bits[1], &o.build_rows, &o.probe_rows, &o.probe_threads, &o.table_load_pct, &e.ms);
        if (n != 15 || e.key.algo < 0 || e.key.algo >= VJ_HASH_COUNT || (e.key.hash_bits != 32 && e.key.hash_bits != 64)) {
            fclose(f);
            return set_error(VJ_ERR_INVALID_ARGUMENT, "vj_tune_load: %s line %d is not a tuning entry", path, lineno);
        }
        o.hash_algo = e.key.algo;
        o.hash_bits = e.key.hash_bits;
        bool replaced = false;
        for (TuneEntry &x : ctx->tuned) {
            if (x.key == e.key) {
                x = e;
                replaced = true;
            }
        }
        if (!replaced) ctx->tuned.push_back(e);
        loaded++;
    }
    fclose(f);
    return VJ_OK;
}
