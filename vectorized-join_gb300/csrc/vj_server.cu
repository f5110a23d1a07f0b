// vj_server.cu -- a join server: requests admitted by HBM budget, run concurrently.
//
// The reference bounds its own concurrency with per-device memory bookkeeping
// (DeviceConfig::memory_left / reserve_memory / is_out_of_memory,
// src/join/join_provider.cuh:138-150), a semaphore of probe threads (:453-480) and a pool
// of streams (:534-560), all inside one join. Here the unit is a whole join request:
//   - `slots` worker threads, each with its own context (its partition buffers and tables
//     stay resident between requests) and its own stream, so admitted joins overlap on the
//     GPU;
//   - a request is admitted when a slot is free and the memory held by all slots plus its
//     estimated footprint stays within the budget; idle slots give their workspace back
//     when a waiting request needs the room;
//   - admission follows arrival order, except that a request that fits may pass a head
//     that does not, at most kBypassLimit times per head (no starvation).
// Every request carries its submit / start / finish times for latency figures.
#include "vj_internal.cuh"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr int kBypassLimit = 8;

struct Request {
    uint64_t id = 0;
    vj_table r{}, s{};
    vj_join_options opt{};
    bool has_opt = false;
    void *pairs = nullptr;
    uint64_t capacity = 0;
    uint64_t need = 0;
    int bypassed = 0;
    bool done = false;
    bool claimed = false;  // a thread is waiting for it (a second waiter is refused)
    vj_request_result res{};
};

struct Slot {
    vj_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t held = 0;  // bytes this slot holds (its workspace) or has reserved (running)
    bool busy = false;
    std::thread thread;
};

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct vj_server {
    int device = 0;
    uint64_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::unordered_map<uint64_t, Request *> requests;
    uint64_t next_id = 1;
    std::vector<Slot> slots;
    bool stopping = false;
    std::chrono::steady_clock::time_point t0;
    vj_server_stats stats{};

    uint64_t held_except(size_t k) const {
        uint64_t h = 0;
        for (size_t j = 0; j < slots.size(); j++) {
            if (j != k) h += slots[j].held;
        }
        return h;
    }

    // Gives back the workspace of an idle slot (stream-ordered: no device-wide wait).
    void release_idle(Slot &sl) {
        vj_ctx *c = sl.ctx;
        if (c->workspace) cudaFreeAsync(c->workspace, sl.stream);
        if (c->stage) cudaFreeAsync(c->stage, sl.stream);
        c->workspace = nullptr;
        c->workspace_bytes = 0;
        c->stage = nullptr;
        c->stage_bytes = 0;
        sl.held = vj_ctx_memory_in_use(c);
    }

    // Under mu: the next request slot k may start, or null.
    Request *pick(size_t k) {
        for (int attempt = 0; attempt < 2; attempt++) {
            const uint64_t others = held_except(k);
            for (size_t i = 0; i < queue.size(); i++) {
                Request *r = queue[i];
                const uint64_t mine = r->need > slots[k].held ? r->need : slots[k].held;
                if (others + mine <= budget) {
                    queue.erase(queue.begin() + (long)i);
                    if (i > 0) queue.front()->bypassed++;
                    return r;
                }
                if (i == 0 && r->bypassed >= kBypassLimit) break;  // the head waits for room, nobody passes it
            }
            if (attempt == 0 && !queue.empty()) {
                // memory is short: idle slots give back their workspace, then try again
                bool freed = false;
                for (auto &sl : slots) {
                    if (!sl.busy && sl.held) {
                        release_idle(sl);
                        freed = true;
                    }
                }
                if (!freed) break;
            }
        }
        return nullptr;
    }

    void worker(size_t k) {
        Slot &sl = slots[k];
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lock(mu);
        for (;;) {
            Request *r = nullptr;
            cv_work.wait(lock, [&] { return (r = pick(k)) != nullptr || (stopping && queue.empty()); });
            if (!r) return;
            sl.busy = true;
            if (r->need > sl.held) sl.held = r->need;
            uint64_t total = 0;
            int running = 0;
            for (auto &x : slots) {
                total += x.held;
                running += x.busy ? 1 : 0;
            }
            if (total > stats.peak_bytes) stats.peak_bytes = total;
            if (running > stats.peak_running) stats.peak_running = running;
            r->res.slot = (int32_t)k;
            r->res.start_s = seconds_since(t0);
            lock.unlock();

            vj_result out{};
            out.pairs = r->pairs;
            out.capacity = r->capacity;
            const int st = vj_join(sl.ctx, &r->r, &r->s, r->has_opt ? &r->opt : nullptr, &out, (vj_stream_t)sl.stream);
            const double fin = seconds_since(t0);

            lock.lock();
            r->res.status = st;
            r->res.count = out.count;
            r->res.passes = sl.ctx->last.passes;
            r->res.radix_bits[0] = sl.ctx->last.radix_bits[0];
            r->res.radix_bits[1] = sl.ctx->last.radix_bits[1];
            r->res.build_rows = sl.ctx->last.build_rows;
            r->res.finish_s = fin;
            r->done = true;
            sl.busy = false;
            sl.held = vj_ctx_memory_in_use(sl.ctx);
            stats.completed++;
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" int vj_server_create(int device, uint64_t memory_budget_bytes, int slots, vj_server **out) {
    using namespace vj;
    VJ_CHECK(out != nullptr, VJ_ERR_INVALID_ARGUMENT, "vj_server_create: null output");
    VJ_CHECK(slots >= 1 && slots <= 64, VJ_ERR_INVALID_ARGUMENT, "vj_server_create: slots must be in [1, 64]");
    VJ_CUDA(cudaSetDevice(device));
    size_t free_b = 0, total_b = 0;
    VJ_CUDA(cudaMemGetInfo(&free_b, &total_b));
    auto *srv = new vj_server();
    srv->device = device;
    srv->budget = memory_budget_bytes ? memory_budget_bytes : (uint64_t)free_b;
    srv->t0 = std::chrono::steady_clock::now();
    srv->slots.resize((size_t)slots);
    for (auto &sl : srv->slots) {
        int st = vj_ctx_create(device, 0, &sl.ctx);
        if (st == VJ_OK && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) st = set_error(VJ_ERR_CUDA, "vj_server_create: stream");
        if (st != VJ_OK) {
            for (auto &x : srv->slots) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.ctx) vj_ctx_destroy(x.ctx);
            }
            delete srv;
            return st;
        }
    }
    srv->stats.slots = slots;
    srv->stats.budget = srv->budget;
    for (size_t k = 0; k < srv->slots.size(); k++) srv->slots[k].thread = std::thread(&vj_server::worker, srv, k);
    *out = srv;
    return VJ_OK;
}

extern "C" int vj_server_submit(vj_server *srv, const vj_table *r, const vj_table *s, const vj_join_options *options, void *d_pairs, uint64_t capacity, uint64_t *request_id) {
    using namespace vj;
    VJ_CHECK(srv && r && s && request_id, VJ_ERR_INVALID_ARGUMENT, "vj_server_submit: null argument");
    VJ_CHECK(d_pairs != nullptr || capacity == 0, VJ_ERR_INVALID_ARGUMENT, "vj_server_submit: null output with capacity > 0");
    uint64_t need = 0;
    VJ_TRY(join_footprint(srv->slots[0].ctx, r, s, options, &need));
    VJ_CHECK(need <= srv->budget, VJ_ERR_BUDGET, "vj_server_submit: the join needs about %llu bytes, the server's budget is %llu", (unsigned long long)need, (unsigned long long)srv->budget);
    auto *q = new Request();
    q->r = *r;
    q->s = *s;
    if (options) {
        q->opt = *options;
        q->has_opt = true;
    }
    q->pairs = d_pairs;
    q->capacity = capacity;
    q->need = need;
    std::lock_guard<std::mutex> lock(srv->mu);
    VJ_CHECK(!srv->stopping, VJ_ERR_INVALID_ARGUMENT, "vj_server_submit: server is stopping");
    q->id = srv->next_id++;
    q->res.submit_s = seconds_since(srv->t0);
    q->res.slot = -1;
    srv->requests[q->id] = q;
    srv->queue.push_back(q);
    srv->stats.submitted++;
    *request_id = q->id;
    srv->cv_work.notify_all();
    return VJ_OK;
}

extern "C" int vj_server_wait(vj_server *srv, uint64_t request_id, vj_request_result *out) {
    using namespace vj;
    VJ_CHECK(srv && out, VJ_ERR_INVALID_ARGUMENT, "vj_server_wait: null argument");
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->requests.find(request_id);
    VJ_CHECK(it != srv->requests.end(), VJ_ERR_INVALID_ARGUMENT, "vj_server_wait: unknown request %llu", (unsigned long long)request_id);
    Request *q = it->second;
    VJ_CHECK(!q->claimed, VJ_ERR_INVALID_ARGUMENT, "vj_server_wait: request %llu is already being waited for", (unsigned long long)request_id);
    q->claimed = true;
    srv->cv_done.wait(lock, [&] { return q->done; });
    *out = q->res;
    srv->requests.erase(request_id);  // the iterator may be stale after the wait
    delete q;
    return VJ_OK;
}

extern "C" int vj_server_share_tuning(vj_server *srv, const vj_ctx *ctx) {
    using namespace vj;
    VJ_CHECK(srv && ctx, VJ_ERR_INVALID_ARGUMENT, "vj_server_share_tuning: null argument");
    std::lock_guard<std::mutex> lock(srv->mu);
    VJ_CHECK(srv->queue.empty() && srv->stats.completed == srv->stats.submitted, VJ_ERR_INVALID_ARGUMENT, "vj_server_share_tuning: requests are queued or running");
    for (auto &sl : srv->slots) sl.ctx->tuned = ctx->tuned;
    return VJ_OK;
}

extern "C" int vj_server_stats_get(vj_server *srv, vj_server_stats *out) {
    using namespace vj;
    VJ_CHECK(srv && out, VJ_ERR_INVALID_ARGUMENT, "vj_server_stats_get: null argument");
    std::lock_guard<std::mutex> lock(srv->mu);
    *out = srv->stats;
    return VJ_OK;
}

extern "C" int vj_server_destroy(vj_server *srv) {
    if (!srv) return VJ_OK;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stopping = true;
    }
    srv->cv_work.notify_all();
    for (auto &sl : srv->slots) {
        if (sl.thread.joinable()) sl.thread.join();
    }
    for (auto &sl : srv->slots) {
        if (sl.stream) {
            cudaStreamSynchronize(sl.stream);
            cudaStreamDestroy(sl.stream);
        }
        if (sl.ctx) vj_ctx_destroy(sl.ctx);
    }
    for (auto &kv : srv->requests) delete kv.second;
    delete srv;
    return VJ_OK;
}
