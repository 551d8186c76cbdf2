// server.cpp — serving loop: resident scenes, admission by device memory,
// continuous batching of ray-query requests.
//
// The reference renders one frame at a time on one render thread
// (src/rt/raytracing_interface.cpp:144-254) and has no request path; this
// loop serves independent ray-query requests against scenes kept resident in
// HBM.  One scheduler thread owns the device work:
//   1. admission: requests wait in FIFO order until their ray, prev_hit and
//      result buffers fit into a device arena of `memory_cap_bytes` (one
//      cudaMalloc at start; sub-allocated first-fit, 256-byte aligned);
//   2. continuous batching: whenever one of `streams` stream slots is free,
//      every admitted request not yet launched (up to max_batch_rays /
//      max_batch_requests) is coalesced into one batched persistent launch
//      on that stream: uploads, the kernel, downloads, an event;
//   3. completion: finished events release the requests' arena blocks (so
//      waiting requests can be admitted) and wake their waiters.
// Requests that arrive while batches run are admitted and launched on the
// next free slot, so their work overlaps the running batches on the device.
// Every ray's result depends only on its own scene and ray, so a request's
// results are the same alone or in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

using namespace igxrt;

namespace {

using Clock = std::chrono::steady_clock;

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

// First-fit allocator over [0, size).
class Arena {
   public:
    explicit Arena(size_t size) { free_[0] = size; }
    bool alloc(size_t bytes, size_t& off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest)
                    free_[off + bytes] = rest;
                used_ += bytes;
                peak_ = std::max(peak_, used_);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t peak() const { return peak_; }

   private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0, peak_ = 0;
};

struct Request {
    igxrt_request r{};
    uint64_t ticket = 0;
    size_t bytes = 0, offset = 0;
    igxrt_request_stats st{};
    bool done = false;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t event = nullptr;
    BatchItemDev* d_table = nullptr;
    BatchItemDev* h_table = nullptr;  // pinned
    uint32_t* queue = nullptr;
    std::vector<Request*> reqs;
    bool busy = false;
};

}  // namespace

struct igxrt_server {
    igxrt_context* ctx = nullptr;
    igxrt_server_options opt{};
    igxrt_launch_params params{};
    Clock::time_point t0;
    char* d_arena = nullptr;
    std::unique_ptr<Arena> arena;
    std::vector<const igxrt_scene*> scenes;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::deque<Request*> pending;  // submitted, waiting for admission
    uint64_t next_ticket = 1;
    bool stopping = false;
    std::vector<double> latencies_ms;
    igxrt_server_stats stats{};

    std::deque<Request*> ready;  // admitted, not launched (scheduler thread only)
    uint32_t batch_seq = 0;
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
    void admit();
    bool launch_one();
    bool complete();
};

void igxrt_server::admit() {
    std::lock_guard<std::mutex> lock(mu);
    while (!pending.empty()) {
        Request* q = pending.front();
        size_t off = 0;
        if (!arena->alloc(q->bytes, off))
            break;  // FIFO: later requests wait behind the first one that does not fit
        q->offset = off;
        q->st.admitted = now();
        ready.push_back(q);
        pending.pop_front();
    }
    stats.peak_memory_bytes = arena->peak();
}

bool igxrt_server::launch_one() {
    if (ready.empty())
        return false;
    Slot* s = nullptr;
    for (auto& sl : slots)
        if (!sl.busy) {
            s = &sl;
            break;
        }
    if (!s)
        return false;
    s->reqs.clear();
    uint64_t rays = 0;
    uint32_t packets = 0;
    while (!ready.empty() && s->reqs.size() < opt.max_batch_requests) {
        Request* q = ready.front();
        if (!s->reqs.empty() && rays + q->r.count > opt.max_batch_rays)
            break;
        ready.pop_front();
        const igxrt_scene* sc = scenes[q->r.scene_id];
        char* base = d_arena + q->offset;
        const size_t rb = round256((size_t)q->r.count * sizeof(igxrt_ray));
        const size_t pb = q->r.prev_hit ? round256((size_t)q->r.count * 4) : 0;
        BatchItemDev& d = s->h_table[s->reqs.size()];
        d.nodes = reinterpret_cast<const float4*>(sc->nodes[params.layout]);
        d.prims = reinterpret_cast<const float4*>(sc->prims);
        d.rays = reinterpret_cast<const igxrt_ray*>(base);
        d.prev = q->r.prev_hit ? reinterpret_cast<const uint32_t*>(base + rb) : nullptr;
        d.out = base + rb + pb;
        d.count = q->r.count;
        d.mode = q->r.mode;
        d.node_count = sc->node_count[params.layout];
        d.packet_begin = packets;
        packets += (q->r.count + params.packet_size - 1) / params.packet_size;
        rays += q->r.count;
        cudaMemcpyAsync(base, q->r.rays, (size_t)q->r.count * sizeof(igxrt_ray),
                        cudaMemcpyHostToDevice, s->stream);
        if (q->r.prev_hit)
            cudaMemcpyAsync(base + rb, q->r.prev_hit, (size_t)q->r.count * 4, cudaMemcpyHostToDevice,
                            s->stream);
        s->reqs.push_back(q);
    }
    const uint32_t n = (uint32_t)s->reqs.size();
    const uint32_t seq = ++batch_seq;
    cudaMemcpyAsync(s->d_table, s->h_table, n * sizeof(BatchItemDev), cudaMemcpyHostToDevice, s->stream);
    igxrt_status st = launch_batch(ctx, s->d_table, n, packets, rays, params, s->queue, s->stream);
    const double t = now();
    for (Request* q : s->reqs) {
        const size_t rb = round256((size_t)q->r.count * sizeof(igxrt_ray));
        const size_t pb = q->r.prev_hit ? round256((size_t)q->r.count * 4) : 0;
        const size_t ob = (size_t)q->r.count * (q->r.mode ? sizeof(uint32_t) : sizeof(igxrt_hit));
        cudaMemcpyAsync(q->r.out, d_arena + q->offset + rb + pb, ob, cudaMemcpyDeviceToHost, s->stream);
        q->st.launched = t;
        q->st.batch = seq;
        q->st.status = st;
    }
    cudaEventRecord(s->event, s->stream);
    s->busy = true;
    {
        std::lock_guard<std::mutex> lock(mu);
        stats.batches++;
        uint32_t inflight = 0;
        for (auto& sl : slots)
            inflight += sl.busy;
        stats.peak_in_flight_batches = std::max(stats.peak_in_flight_batches, inflight);
    }
    return true;
}

bool igxrt_server::complete() {
    bool any = false;
    for (auto& s : slots) {
        if (!s.busy)
            continue;
        const cudaError_t e = cudaEventQuery(s.event);
        if (e == cudaErrorNotReady)
            continue;
        const double t = now();
        std::lock_guard<std::mutex> lock(mu);
        for (Request* q : s.reqs) {
            arena->release(q->offset, q->bytes);
            q->st.completed = t;
            if (e != cudaSuccess)
                q->st.status = IGXRT_ERROR_CUDA;
            q->done = true;
            stats.completed++;
            stats.rays_completed += q->r.count;
            stats.last_complete = t;
            latencies_ms.push_back(1e3 * (t - q->st.submitted));
        }
        s.reqs.clear();
        s.busy = false;
        any = true;
    }
    if (any)
        cv_done.notify_all();
    return any;
}

void igxrt_server::run() {
    cudaSetDevice(ctx->device);
    for (;;) {
        admit();
        bool progress = false;
        while (launch_one())
            progress = true;
        progress |= complete();
        std::unique_lock<std::mutex> lock(mu);
        bool busy = !ready.empty();
        for (auto& s : slots)
            busy |= s.busy;
        if (stopping && pending.empty() && !busy)
            break;
        if (!progress) {
            // in-flight work: poll its events often; otherwise sleep until a submit
            if (busy)
                cv_work.wait_for(lock, std::chrono::microseconds(20));
            else if (pending.empty() && !stopping)
                cv_work.wait_for(lock, std::chrono::milliseconds(2));
            else
                cv_work.wait_for(lock, std::chrono::microseconds(20));
        }
    }
}

extern "C" {

igxrt_status igxrt_server_create(igxrt_context* ctx, const igxrt_server_options* opts, igxrt_server** out) {
    if (!ctx || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    std::unique_ptr<igxrt_server> s(new (std::nothrow) igxrt_server());
    if (!s)
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "server object");
    s->ctx = ctx;
    if (opts)
        s->opt = *opts;
    if (!s->opt.memory_cap_bytes)
        s->opt.memory_cap_bytes = 24ull << 30;
    if (!s->opt.max_batch_rays)
        s->opt.max_batch_rays = 4u << 20;
    if (!s->opt.max_batch_requests)
        s->opt.max_batch_requests = 1024;
    if (!s->opt.streams)
        s->opt.streams = 2;
    if (s->opt.max_batch_requests > 4096 || s->opt.streams > 16)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "max_batch_requests <= 4096, streams <= 16");
    igxrt_status st = resolve_params(ctx, ctx->params, s->params);
    if (st != IGXRT_OK)
        return st;
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    s->opt.memory_cap_bytes = round256(s->opt.memory_cap_bytes);
    cudaError_t e = cudaMalloc(&s->d_arena, s->opt.memory_cap_bytes);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "server arena (memory_cap_bytes)");
    s->arena.reset(new Arena(s->opt.memory_cap_bytes));
    s->slots.resize(s->opt.streams);
    for (auto& sl : s->slots) {
        const size_t tb = round256(s->opt.max_batch_requests * sizeof(BatchItemDev));
        e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaMalloc(&sl.d_table, tb + 256);
        if (e == cudaSuccess)
            e = cudaMallocHost(&sl.h_table, tb);
        if (e != cudaSuccess) {
            igxrt_server_destroy(s.release());
            return cuda_fail(ctx, e, "server stream slots");
        }
        sl.queue = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(sl.d_table) + tb);
    }
    s->t0 = Clock::now();
    s->stats.first_submit = -1;
    igxrt_server* raw = s.release();
    raw->worker = std::thread([raw]() { raw->run(); });
    *out = raw;
    return IGXRT_OK;
}

igxrt_status igxrt_server_add_scene(igxrt_server* s, const igxrt_scene* scene, uint32_t* scene_id) {
    if (!s || !scene || !scene_id)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (scene->device != s->ctx->device)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    // the batched kernel the server launches traces triangle-only trees in
    // the server's layout
    if (scene->mixed || !scene->has_layout(s->params.layout))
        return IGXRT_ERROR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(s->mu);
    *scene_id = (uint32_t)s->scenes.size();
    s->scenes.push_back(scene);
    return IGXRT_OK;
}

igxrt_status igxrt_server_submit(igxrt_server* s, const igxrt_request* req, uint64_t* ticket) {
    if (!s || !req || !ticket)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::unique_ptr<Request> q(new (std::nothrow) Request());
    if (!q)
        return IGXRT_ERROR_OUT_OF_MEMORY;
    q->r = *req;
    const double t = s->now();
    q->st.submitted = t;
    std::lock_guard<std::mutex> lock(s->mu);
    if (req->scene_id >= s->scenes.size() || req->mode > 1 || (req->count && (!req->rays || !req->out)))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (((uintptr_t)req->rays % 16) || ((uintptr_t)req->prev_hit % 4) || ((uintptr_t)req->out % 4))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    q->bytes = round256((size_t)req->count * sizeof(igxrt_ray)) +
               (req->prev_hit ? round256((size_t)req->count * 4) : 0) +
               round256((size_t)req->count * (req->mode ? sizeof(uint32_t) : sizeof(igxrt_hit)));
    s->stats.submitted++;
    if (s->stats.first_submit < 0)
        s->stats.first_submit = t;
    if (q->bytes > s->opt.memory_cap_bytes) {
        s->stats.rejected++;
        return IGXRT_ERROR_ADMISSION;
    }
    q->ticket = s->next_ticket++;
    *ticket = q->ticket;
    Request* raw = q.get();
    s->reqs.emplace(q->ticket, std::move(q));
    if (raw->r.count == 0) {
        raw->st.admitted = raw->st.launched = raw->st.completed = t;
        raw->done = true;
        s->stats.completed++;
        s->latencies_ms.push_back(0.0);
        s->cv_done.notify_all();
        return IGXRT_OK;
    }
    s->pending.push_back(raw);
    s->stats.peak_pending = std::max<uint32_t>(s->stats.peak_pending, (uint32_t)s->pending.size());
    s->cv_work.notify_one();
    return IGXRT_OK;
}

igxrt_status igxrt_server_wait(igxrt_server* s, uint64_t ticket, double timeout_s,
                               igxrt_request_stats* stats) {
    if (!s)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end())
        return IGXRT_ERROR_INVALID_ARGUMENT;
    Request* q = it->second.get();
    auto pred = [q]() { return q->done; };
    if (timeout_s < 0)
        s->cv_done.wait(lock, pred);
    else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), pred))
        return IGXRT_ERROR_TIMEOUT;
    if (stats)
        *stats = q->st;
    return (igxrt_status)q->st.status;
}

igxrt_status igxrt_server_get_stats(igxrt_server* s, igxrt_server_stats* out) {
    if (!s || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    std::vector<double> l = s->latencies_ms;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&l](double p) {
            const size_t i = std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5));
            return l[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = l.back();
        double sum = 0;
        for (double x : l)
            sum += x;
        out->mean_ms = sum / l.size();
    }
    return IGXRT_OK;
}

igxrt_status igxrt_server_destroy(igxrt_server* s) {
    if (!s)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable())
        s->worker.join();
    {
        DeviceGuard guard(s->ctx->device);
        for (auto& sl : s->slots) {
            if (sl.stream)
                cudaStreamSynchronize(sl.stream);
            if (sl.event)
                cudaEventDestroy(sl.event);
            if (sl.d_table)
                cudaFree(sl.d_table);
            if (sl.h_table)
                cudaFreeHost(sl.h_table);
            if (sl.stream)
                cudaStreamDestroy(sl.stream);
        }
        if (s->d_arena)
            cudaFree(s->d_arena);
    }
    delete s;
    return IGXRT_OK;
}

}  // extern "C"
