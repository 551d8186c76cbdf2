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
//      the admitted requests with rays not yet launched are coalesced into
//      one batched persistent launch on that stream (uploads, the kernel,
//      downloads, an event), each request with its next slice of at most
//      `slice_rays` rays, up to max_batch_rays per launch.  A large request
//      therefore spreads over several launches, each shared with the requests
//      queued behind it, instead of making them wait for all of its rays;
//   3. completion: finished events account each slice; a request whose
//      slices are all done releases its arena block (so waiting requests can
//      be admitted) and wakes its waiters.
// Requests that arrive while batches run are admitted and launched on the
// next free slot, so their work overlaps the running batches on the device;
// each batch kernel stamps its first start and last exit with %globaltimer,
// which igxrt_server_batch_times reports.  Latency runs from a request's
// arrival: its scheduled time when igxrt_server_replay paces it, else its
// submission.  Every ray's result depends only on its own scene and ray, so
// a request's results are the same alone, sliced, or in any mix.
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
    uint32_t launched_rays = 0;  // rays handed to batches (scheduler thread)
    uint32_t done_rays = 0;      // rays whose batch has completed
    bool done = false;
};

// Rays [first, first + count) of a request, carried by one batch.
struct Slice {
    Request* q;
    uint32_t first, count;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t event = nullptr;
    BatchItemDev* d_table = nullptr;
    BatchItemDev* h_table = nullptr;  // pinned
    uint32_t* queue = nullptr;
    unsigned long long* d_times = nullptr;  // {first CTA start, last warp exit}
    unsigned long long* h_times = nullptr;  // pinned copy, read at completion
    std::vector<Slice> slices;
    uint32_t seq = 0;
    uint64_t rays = 0;
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

    std::deque<Request*> ready;  // admitted, rays left to launch (scheduler thread only)
    uint32_t batch_seq = 0;
    std::vector<igxrt_batch_time> batch_times;  // completed batches (under mu)
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
    void admit();
    bool launch_one();
    bool complete();
    igxrt_status submit(const igxrt_request* req, double arrival, uint64_t* ticket);
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
    s->slices.clear();
    uint64_t rays = 0;
    uint32_t packets = 0;
    bool mixed = false;
    // every request in the ready queue, in order, adds its next slice
    for (auto it = ready.begin(); it != ready.end() && s->slices.size() < opt.max_batch_requests;) {
        Request* q = *it;
        const uint32_t n = std::min(q->r.count - q->launched_rays, opt.slice_rays);
        if (!s->slices.empty() && rays + n > opt.max_batch_rays)
            break;
        const uint32_t first = q->launched_rays;
        const igxrt_scene* sc = scenes[q->r.scene_id];
        char* base = d_arena + q->offset;
        const size_t rb = round256((size_t)q->r.count * sizeof(igxrt_ray));
        const size_t pb = q->r.prev_hit ? round256((size_t)q->r.count * 4) : 0;
        const size_t elem = q->r.mode ? sizeof(uint32_t) : sizeof(igxrt_hit);
        igxrt_ray* d_rays = reinterpret_cast<igxrt_ray*>(base) + first;
        uint32_t* d_prev = q->r.prev_hit ? reinterpret_cast<uint32_t*>(base + rb) + first : nullptr;
        BatchItemDev& d = s->h_table[s->slices.size()];
        batch_item_for(sc, params, d_rays, d_prev, base + rb + pb + (size_t)first * elem, n, q->r.mode, d);
        d.packet_begin = packets;
        packets += (n + params.packet_size - 1) / params.packet_size;
        rays += n;
        mixed |= sc->mixed;
        cudaMemcpyAsync(d_rays, q->r.rays + first, (size_t)n * sizeof(igxrt_ray), cudaMemcpyHostToDevice,
                        s->stream);
        if (q->r.prev_hit)
            cudaMemcpyAsync(d_prev, q->r.prev_hit + first, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream);
        s->slices.push_back({q, first, n});
        q->launched_rays += n;
        if (q->launched_rays == q->r.count)
            it = ready.erase(it);
        else
            ++it;
    }
    const uint32_t n = (uint32_t)s->slices.size();
    const uint32_t seq = ++batch_seq;
    cudaMemcpyAsync(s->d_table, s->h_table, n * sizeof(BatchItemDev), cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(s->d_times, 0xff, sizeof(unsigned long long), s->stream);
    cudaMemsetAsync(s->d_times + 1, 0, sizeof(unsigned long long), s->stream);
    igxrt_status st = launch_batch(ctx, s->d_table, n, packets, rays, params, s->queue, s->stream, mixed,
                                   s->d_times);
    const double t = now();
    for (const Slice& sl : s->slices) {
        Request* q = sl.q;
        const size_t rb = round256((size_t)q->r.count * sizeof(igxrt_ray));
        const size_t pb = q->r.prev_hit ? round256((size_t)q->r.count * 4) : 0;
        const size_t elem = q->r.mode ? sizeof(uint32_t) : sizeof(igxrt_hit);
        cudaMemcpyAsync(static_cast<char*>(q->r.out) + (size_t)sl.first * elem,
                        d_arena + q->offset + rb + pb + (size_t)sl.first * elem, (size_t)sl.count * elem,
                        cudaMemcpyDeviceToHost, s->stream);
        if (sl.first == 0)
            q->st.launched = t;
        q->st.batch = seq;
        if (st != IGXRT_OK)
            q->st.status = st;
    }
    cudaMemcpyAsync(s->h_times, s->d_times, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->stream);
    cudaEventRecord(s->event, s->stream);
    s->seq = seq;
    s->rays = rays;
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
    for (size_t k = 0; k < slots.size(); ++k) {
        Slot& s = slots[k];
        if (!s.busy)
            continue;
        const cudaError_t e = cudaEventQuery(s.event);
        if (e == cudaErrorNotReady)
            continue;
        const double t = now();
        std::lock_guard<std::mutex> lock(mu);
        igxrt_batch_time bt{};
        bt.start_ns = s.h_times[0];
        bt.end_ns = s.h_times[1];
        bt.batch = s.seq;
        bt.stream = (uint32_t)k;
        bt.rays = s.rays;
        batch_times.push_back(bt);
        for (const Slice& sl : s.slices) {
            Request* q = sl.q;
            if (e != cudaSuccess)
                q->st.status = IGXRT_ERROR_CUDA;
            q->done_rays += sl.count;
            if (q->done_rays < q->r.count)
                continue;
            arena->release(q->offset, q->bytes);
            q->st.completed = t;
            q->done = true;
            stats.completed++;
            stats.rays_completed += q->r.count;
            stats.last_complete = t;
            latencies_ms.push_back(1e3 * (t - q->st.arrival));
        }
        s.slices.clear();
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

igxrt_status igxrt_server::submit(const igxrt_request* req, double arrival, uint64_t* ticket) {
    std::unique_ptr<Request> q(new (std::nothrow) Request());
    if (!q)
        return IGXRT_ERROR_OUT_OF_MEMORY;
    q->r = *req;
    const double t = now();
    q->st.submitted = t;
    q->st.arrival = arrival < 0 ? t : arrival;
    std::lock_guard<std::mutex> lock(mu);
    if (req->scene_id >= scenes.size() || req->mode > 1 || (req->count && (!req->rays || !req->out)))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (((uintptr_t)req->rays % 16) || ((uintptr_t)req->prev_hit % 4) || ((uintptr_t)req->out % 4))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    q->bytes = round256((size_t)req->count * sizeof(igxrt_ray)) +
               (req->prev_hit ? round256((size_t)req->count * 4) : 0) +
               round256((size_t)req->count * (req->mode ? sizeof(uint32_t) : sizeof(igxrt_hit)));
    stats.submitted++;
    if (stats.first_submit < 0)
        stats.first_submit = t;
    if (q->bytes > opt.memory_cap_bytes) {
        stats.rejected++;
        return IGXRT_ERROR_ADMISSION;
    }
    q->ticket = next_ticket++;
    *ticket = q->ticket;
    Request* raw = q.get();
    reqs.emplace(q->ticket, std::move(q));
    if (raw->r.count == 0) {
        raw->st.admitted = raw->st.launched = raw->st.completed = t;
        raw->done = true;
        stats.completed++;
        latencies_ms.push_back(1e3 * (t - raw->st.arrival));
        cv_done.notify_all();
        return IGXRT_OK;
    }
    pending.push_back(raw);
    stats.peak_pending = std::max<uint32_t>(stats.peak_pending, (uint32_t)pending.size());
    cv_work.notify_one();
    return IGXRT_OK;
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
        s->opt.max_batch_rays = 1u << 20;
    if (!s->opt.slice_rays)
        s->opt.slice_rays = 256u << 10;
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
        // item table, then the queue word, then the two timestamps, 256 bytes apart
        const size_t tb = round256(s->opt.max_batch_requests * sizeof(BatchItemDev));
        e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaMalloc(&sl.d_table, tb + 512);
        if (e == cudaSuccess)
            e = cudaMallocHost(&sl.h_table, tb + 256);
        if (e != cudaSuccess) {
            igxrt_server_destroy(s.release());
            return cuda_fail(ctx, e, "server stream slots");
        }
        sl.queue = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(sl.d_table) + tb);
        sl.d_times = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(sl.d_table) + tb + 256);
        sl.h_times = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(sl.h_table) + tb);
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
    // the batched kernel traces the tree in the server's layout (mixed
    // scenes run its mixed variant)
    if (!scene->has_layout(s->params.layout))
        return IGXRT_ERROR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(s->mu);
    *scene_id = (uint32_t)s->scenes.size();
    s->scenes.push_back(scene);
    return IGXRT_OK;
}

igxrt_status igxrt_server_submit(igxrt_server* s, const igxrt_request* req, uint64_t* ticket) {
    if (!s || !req || !ticket)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    return s->submit(req, -1.0, ticket);
}

igxrt_status igxrt_server_replay(igxrt_server* s, const igxrt_request* reqs, const double* arrival_s,
                                 uint32_t count, uint64_t* tickets) {
    if (!s || (count && (!reqs || !arrival_s || !tickets)))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    const double start = s->now();
    for (uint32_t i = 0; i < count; ++i) {
        const double due = start + arrival_s[i];
        for (;;) {
            const double d = due - s->now();
            if (d <= 0)
                break;
            if (d > 300e-6)
                std::this_thread::sleep_for(std::chrono::duration<double>(d - 200e-6));
        }
        tickets[i] = 0;
        const igxrt_status st = s->submit(&reqs[i], due, &tickets[i]);
        if (st != IGXRT_OK && st != IGXRT_ERROR_ADMISSION)
            return st;
    }
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

igxrt_status igxrt_server_batch_times(igxrt_server* s, igxrt_batch_time* out, uint32_t max_batches,
                                      uint32_t* count) {
    if (!s || !count || (max_batches && !out))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    const uint32_t n = (uint32_t)std::min<size_t>(max_batches, s->batch_times.size());
    std::copy(s->batch_times.begin(), s->batch_times.begin() + n, out);
    *count = n;
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
