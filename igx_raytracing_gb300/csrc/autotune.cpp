// autotune.cpp — picks the batched kernel's launch parameters by timing them.
//
// Search: coordinate descent from the context's current parameters over
// node layout, packet size, refill threshold, block size, shared stack depth
// and the node phase's early end (two rounds; a change is kept only when it
// is at least 1% faster).
// Each candidate is timed with CUDA events on a private stream over the
// caller's items (median of `reps` repetitions after one warm-up), as one
// batched launch or, with IGXRT_TUNE_PLAIN, as one plain launch per item.
// Results can be cached in a text file, one line per (GPU name, class key):
//     <gpu>|<key>\t<block> <stack> <packet> <layout> <ctas> <refill> <phase_break>\t<ms>
// The default class key buckets the workload by item count, total rays,
// total triangles (powers of two) and the share of any-hit items.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "engine.h"

using namespace igxrt;

namespace {

int log2_bucket(uint64_t x) {
    int b = 0;
    while (x > 1) {
        x >>= 1;
        ++b;
    }
    return b;
}

std::string derive_key(const igxrt_batch_item* items, uint32_t count) {
    uint64_t rays = 0, tris = 0, any = 0;
    for (uint32_t i = 0; i < count; ++i) {
        rays += items[i].count;
        tris += items[i].scene ? items[i].scene->info.triangle_count : 0;
        any += items[i].mode == IGXRT_MODE_ANY ? items[i].count : 0;
    }
    return format("items2^%d rays2^%d tris2^%d any%d%%", log2_bucket(count), log2_bucket(rays),
                  log2_bucket(tris), rays ? (int)(100 * any / rays) : 0);
}

bool cache_lookup(const char* path, const std::string& key, igxrt_launch_params& p, float& ms) {
    std::ifstream f(path);
    if (!f)
        return false;
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        const size_t t1 = line.find('\t');
        if (t1 == std::string::npos || line.compare(0, t1, key) != 0 || t1 != key.size())
            continue;
        const size_t t2 = line.find('\t', t1 + 1);
        std::istringstream in(line.substr(t1 + 1, t2 == std::string::npos ? std::string::npos : t2 - t1 - 1));
        igxrt_launch_params q{};
        if (in >> q.block_size >> q.stack_depth >> q.packet_size >> q.layout >> q.ctas_per_sm >> q.refill_lanes) {
            if (!(in >> q.phase_break))
                q.phase_break = 0;  // an entry written before the field existed: the default
            p = q;
            ms = t2 == std::string::npos ? 0.f : std::strtof(line.c_str() + t2 + 1, nullptr);
            found = true;  // the last entry for a key wins
        }
    }
    return found;
}

void cache_store(const char* path, const std::string& key, const igxrt_launch_params& p, float ms) {
    FILE* f = fopen(path, "a");
    if (!f)
        return;
    fprintf(f, "%s\t%u %u %u %u %u %u %u\t%.4f\n", key.c_str(), p.block_size, p.stack_depth,
            p.packet_size, p.layout, p.ctas_per_sm, p.refill_lanes, p.phase_break, ms);
    fclose(f);
}

struct Timer {
    igxrt_context* ctx;
    const igxrt_batch_item* items;
    uint32_t count;
    uint32_t reps;
    bool plain;
    cudaStream_t stream = nullptr;
    BatchItemDev* d_table = nullptr;
    uint32_t* queue = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;

    igxrt_status init() {
        // item table, then the queue word 256 bytes further on
        const size_t tb = (std::max<size_t>(count, 1) * sizeof(BatchItemDev) + 255) / 256 * 256;
        cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaMalloc(&d_table, tb + 256);
        if (e == cudaSuccess)
            e = cudaEventCreate(&e0);
        if (e == cudaSuccess)
            e = cudaEventCreate(&e1);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "autotune setup");
        queue = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(d_table) + tb);
        return IGXRT_OK;
    }

    ~Timer() {
        if (stream)
            cudaStreamSynchronize(stream);
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
        if (d_table)
            cudaFree(d_table);
        if (stream)
            cudaStreamDestroy(stream);
    }

    // Median launch time in ms, or a negative value if `p` cannot launch.
    float time(const igxrt_launch_params& p) {
        if (plain)
            return time_plain(p);
        std::vector<BatchItemDev> table;
        uint32_t packets = 0;
        uint64_t rays = 0;
        bool mixed = false;
        if (build_batch_table(ctx, items, count, p, table, packets, rays, mixed) != IGXRT_OK)
            return -1.f;
        if (!table.empty() &&
            cudaMemcpyAsync(d_table, table.data(), table.size() * sizeof(BatchItemDev),
                            cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return -1.f;
        std::vector<float> ts;
        for (uint32_t r = 0; r < reps + 1; ++r) {
            cudaEventRecord(e0, stream);
            if (launch_batch(ctx, d_table, count, packets, rays, p, queue, stream, mixed) != IGXRT_OK)
                return -1.f;
            cudaEventRecord(e1, stream);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                return -1.f;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0)
                ts.push_back(ms);
        }
        std::sort(ts.begin(), ts.end());
        return ts[ts.size() / 2];
    }

    // The items as plain launches, one per item in order (IGXRT_TUNE_PLAIN).
    float time_plain(const igxrt_launch_params& p) {
        std::vector<float> ts;
        for (uint32_t r = 0; r < reps + 1; ++r) {
            cudaEventRecord(e0, stream);
            for (uint32_t i = 0; i < count; ++i) {
                const igxrt_batch_item& it = items[i];
                TraceRequest req{it.scene, it.rays, it.prev_hit, it.count, it.mode,
                                 it.mode == IGXRT_MODE_CLOSEST ? static_cast<igxrt_hit*>(it.out) : nullptr,
                                 it.mode == IGXRT_MODE_ANY ? static_cast<uint32_t*>(it.out) : nullptr,
                                 nullptr, nullptr};
                if (launch_trace(ctx, req, p, stream) != IGXRT_OK)
                    return -1.f;
            }
            cudaEventRecord(e1, stream);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                return -1.f;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0)
                ts.push_back(ms);
        }
        std::sort(ts.begin(), ts.end());
        return ts[ts.size() / 2];
    }
};

// Items a plain-launch tuning can time: scenes of this context, arrays the
// kernels can address, known modes.
igxrt_status check_plain_items(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count) {
    for (uint32_t i = 0; i < count; ++i) {
        const igxrt_batch_item& it = items[i];
        igxrt_status st = check_scene(ctx, it.scene);
        if (st != IGXRT_OK)
            return st;
        if (it.mode != IGXRT_MODE_CLOSEST && it.mode != IGXRT_MODE_ANY)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: unknown mode %u", i, it.mode));
        if (it.count && (!it.rays || !it.out))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: rays or out is NULL", i));
        if (!device_accessible(it.rays) || !device_accessible(it.prev_hit) || !device_accessible(it.out))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                        format("item %u: an array is not addressable by the device", i));
    }
    return IGXRT_OK;
}

}  // namespace

extern "C" igxrt_status igxrt_autotune(igxrt_context* ctx, const igxrt_batch_item* items,
                                       uint32_t count, const igxrt_tune_options* opts,
                                       igxrt_launch_params* best, float* best_ms) {
    if (!ctx || !best)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (!count || !items)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "autotune needs at least one item");
    const uint32_t reps = opts && opts->reps ? opts->reps : 3;
    if (opts && (opts->flags & ~IGXRT_TUNE_PLAIN))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown tune flags 0x%x", opts->flags));
    const bool plain = opts && (opts->flags & IGXRT_TUNE_PLAIN);
    if (plain) {
        igxrt_status st = check_plain_items(ctx, items, count);
        if (st != IGXRT_OK)
            return st;
    }
    uint32_t mask = opts && opts->layouts_mask ? opts->layouts_mask : ((1u << IGXRT_LAYOUT_COUNT) - 1);
    for (uint32_t i = 0; i < count; ++i)  // only layouts every scene has
        for (uint32_t l = 0; l < IGXRT_LAYOUT_COUNT; ++l)
            if (items[i].scene && !items[i].scene->has_layout(l))
                mask &= ~(1u << l);
    if (!(mask & ((1u << IGXRT_LAYOUT_COUNT) - 1)))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, "autotune: no node layout common to all scenes");
    const std::string key = ctx->device_name + "|" +
                            ((opts && opts->class_key) ? std::string(opts->class_key) : derive_key(items, count)) +
                            (plain ? "|plain" : "");
    const char* cache = opts ? opts->cache_path : nullptr;
    if (cache && !(opts && opts->force)) {
        igxrt_launch_params p{};
        float ms = 0.f;
        if (cache_lookup(cache, key, p, ms)) {
            igxrt_launch_params r;
            if (resolve_params(ctx, p, r) == IGXRT_OK && (mask >> r.layout) & 1u) {
                *best = r;
                if (best_ms)
                    *best_ms = ms;
                return IGXRT_OK;
            }
        }
    }
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    Timer t{ctx, items, count, reps, plain};
    igxrt_status st = t.init();
    if (st != IGXRT_OK)
        return st;

    igxrt_launch_params cur;
    st = resolve_params(ctx, ctx->params, cur);
    if (st != IGXRT_OK)
        return st;
    if (!((mask >> cur.layout) & 1u))
        for (uint32_t l = 0; l < IGXRT_LAYOUT_COUNT; ++l)
            if ((mask >> l) & 1u) {
                cur.layout = l;
                break;
            }
    float cur_ms = t.time(cur);
    if (cur_ms < 0)
        return fail(ctx, IGXRT_ERROR_CUDA, "autotune: the starting parameters do not launch");

    const std::vector<uint32_t> layouts = {IGXRT_LAYOUT_BVH2, IGXRT_LAYOUT_BVH4, IGXRT_LAYOUT_BVH8};
    const std::vector<uint32_t> packets = {8, 16, 32, 64, 128, 256};
    const std::vector<uint32_t> refills = {1, 2, 4, 8, 16};
    const std::vector<uint32_t> blocks = {64, 128, 256};
    const std::vector<uint32_t> stacks = {8, 16, 32};
    const std::vector<uint32_t> breaks = {1, 2, 3, 32};
    for (int round = 0; round < 2; ++round) {
        bool changed = false;
        for (int dim = 0; dim < 6; ++dim) {
            const std::vector<uint32_t>& vals = dim == 0   ? layouts
                                                : dim == 1 ? packets
                                                : dim == 2 ? refills
                                                : dim == 3 ? blocks
                                                : dim == 4 ? stacks
                                                           : breaks;
            for (uint32_t v : vals) {
                igxrt_launch_params c = cur;
                uint32_t* field = dim == 0 ? &c.layout : dim == 1 ? &c.packet_size
                                  : dim == 2 ? &c.refill_lanes : dim == 3 ? &c.block_size
                                  : dim == 4 ? &c.stack_depth : &c.phase_break;
                if (*field == v)
                    continue;
                if (dim == 0 && !((mask >> v) & 1u))
                    continue;
                *field = v;
                const float ms = t.time(c);
                if (ms > 0 && ms < cur_ms * 0.99f) {
                    cur = c;
                    cur_ms = ms;
                    changed = true;
                }
            }
        }
        if (!changed)
            break;
    }
    *best = cur;
    if (best_ms)
        *best_ms = cur_ms;
    if (cache)
        cache_store(cache, key, cur, cur_ms);
    return IGXRT_OK;
}
