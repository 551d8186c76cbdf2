// batch.cu — one persistent launch over many scenes' ray batches.
//
// The rays of all items form a single space of packets (each item's rays cut
// into packets of `packet` rays; an item's packets are contiguous).  A warp
// claims one packet at a time with an atomicAdd on the batch's queue word,
// finds the packet's item by a binary search over the items' first-packet
// indices, and hands the packet's rays to its idle lanes.  Lanes therefore
// carry their own item (node array, records, output, query mode): a warp can
// finish rays of one scene while starting rays of the next, and the GPU stays
// full across item boundaries instead of draining at the end of each launch.
// Per ray the traversal is the plain kernel's (same visiting order, same
// arithmetic, and the same tail work sharing once the queue is drained), so
// results equal tracing each item alone.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "engine.h"
#include "share.cuh"
#include "traverse.cuh"

namespace igxrt {

static_assert(sizeof(BatchItemDev) == 72, "batch item layout");

struct BatchArgs {
    const BatchItemDev* items;
    uint32_t item_count;
    uint32_t total_packets;
    uint32_t* queue;
    uint32_t* status;
    uint32_t packet;
    uint32_t sh_depth;
    uint32_t refill_lanes;
    uint32_t phase_break;       // node_phase's early end (igxrt_launch_params.phase_break)
    unsigned long long* times;  // optional: {earliest CTA start, latest warp exit}
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A finished ray's record: occluded word (any hit) or hit (closest).  Mixed
// scenes keep a priority code in best.prim (traverse.cuh), decoded here.
template <bool MIXED>
__device__ __forceinline__ void write_result(void* out, uint32_t mode, uint32_t ray, const RayState& r,
                                             const BestHit& best, bool occluded) {
    if (mode) {
        __stcs(static_cast<uint32_t*>(out) + ray, occluded ? 1u : 0u);
    } else {
        const bool hit = MIXED ? (best.t < r.tmax_eff || best.prim < kPrioNone) : best.t < r.tmax_eff;
        const uint32_t prim = MIXED ? id_of_prio(best.prim) : best.prim;
        const float4 h = hit ? make_float4(best.t, best.u, best.v, __uint_as_float(prim))
                             : make_float4(IGXRT_NO_HIT, 0.f, 0.f, __uint_as_float(IGXRT_NO_RAY_HIT));
        __stcs(static_cast<float4*>(out) + ray, h);
    }
}

// A lane's item (scene arrays, output, query mode), which a helper in the
// tail copies from the lane whose ray it helps (share.cuh).
struct BatchLane {
    const float4*& nodes;
    const float4*& prims;
    void*& out;
    uint32_t& mode;
    __device__ __forceinline__ void take(uint32_t src) {
        nodes = reinterpret_cast<const float4*>(__shfl_sync(0xffffffffu, (unsigned long long)nodes, src));
        prims = reinterpret_cast<const float4*>(__shfl_sync(0xffffffffu, (unsigned long long)prims, src));
        out = reinterpret_cast<void*>(__shfl_sync(0xffffffffu, (unsigned long long)out, src));
        mode = __shfl_sync(0xffffffffu, mode, src);
    }
};

// MIXED: items may hold spheres, cubes and planes (typed leaves, planes tested
// when a ray starts, priority-coded best hit); triangle-only items trace the
// same in it.
template <int LAYOUT, bool MIXED>
__global__ void __launch_bounds__(256) batch_kernel(BatchArgs a) {
    if (a.times && threadIdx.x == 0)
        atomicMin(a.times, global_ns());
    extern __shared__ uint32_t smem[];
    TraversalStack st;
    st.sh = reinterpret_cast<uint2*>(smem) + threadIdx.x;
    st.stride = blockDim.x;
    st.sh_depth = a.sh_depth;
    st.sp = 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lower = (1u << lane) - 1u;
    // warp-uniform window: rays [w_base, w_end) of item w_item
    uint32_t w_item = 0, w_base = 0, w_end = 0;
    bool queue_done = false;
    // lane state
    bool alive = false, occluded_at_start = false;
    uint32_t ray = 0, mode = 0;
    const float4* nodes = nullptr;
    const float4* prims = nullptr;
    void* out = nullptr;
    int32_t next = kRefDone;
    RayState r;
    BestHit best;
    uint32_t unused = 0;
    // work sharing once the queue is drained (share.cuh)
    uint32_t link = lane;
    for (;;) {
        if (queue_done && __ballot_sync(0xffffffffu, !alive || (link & (kLinkWait | kLinkMerge))) != 0) {
            BatchLane lane_item{nodes, prims, out, mode};
            share_tail<kSharePerLane>(lane, lower, link, alive, ray, r, best, st, next, lane_item,
                                      [&](bool occ) { write_result<MIXED>(out, mode, ray, r, best, occ); },
                                      MIXED ? kPrioNone : 0u);
        }
        const uint32_t idle = __ballot_sync(0xffffffffu, !alive);
        const uint32_t nidle = __popc(idle);
        if (!queue_done && nidle != 0 && (nidle >= a.refill_lanes || nidle == 32)) {
            const uint32_t rank = __popc(idle & lower);
            uint32_t given = 0;
            while (given < nidle) {
                if (w_base >= w_end) {
                    uint32_t p = 0, item = 0;
                    if (lane == 0) {
                        p = atomicAdd(a.queue, 1u);
                        if (p < a.total_packets) {
                            uint32_t lo = 0, hi = a.item_count;
                            while (hi - lo > 1) {
                                const uint32_t mid = (lo + hi) >> 1;
                                if (__ldg(&a.items[mid].packet_begin) <= p)
                                    lo = mid;
                                else
                                    hi = mid;
                            }
                            item = lo;
                        }
                    }
                    p = __shfl_sync(0xffffffffu, p, 0);
                    item = __shfl_sync(0xffffffffu, item, 0);
                    if (p >= a.total_packets) {
                        queue_done = true;
                        break;
                    }
                    w_item = item;
                    w_base = (p - __ldg(&a.items[item].packet_begin)) * a.packet;
                    w_end = min(w_base + a.packet, __ldg(&a.items[item].count));
                }
                const uint32_t take = min(nidle - given, w_end - w_base);
                if (!alive && rank >= given && rank < given + take) {
                    const BatchItemDev* it = a.items + w_item;
                    ray = w_base + (rank - given);
                    nodes = it->nodes;
                    prims = it->prims;
                    out = it->out;
                    mode = it->mode;
                    const uint32_t* prev = it->prev;
                    r = load_ray(it->rays, ray, prev ? __ldg(prev + ray) : IGXRT_NO_RAY_HIT);
                    best.t = r.tmax_eff;
                    best.u = 0.f;
                    best.v = 0.f;
                    best.prim = MIXED ? kPrioNone : 0u;
                    best.tcull = cull_limit(best.t);
                    next = it->node_count ? 0 : kRefDone;
                    occluded_at_start = false;
                    if (MIXED) {
                        const uint32_t np = it->plane_count;
                        if (np) {
                            occluded_at_start = mode ? test_planes<true>(it->planes, np, it->plane_base, r, best)
                                                     : test_planes<false>(it->planes, np, it->plane_base, r, best);
                            if (occluded_at_start)
                                next = kRefDone;
                        }
                    }
                    st.sp = 0;
                    alive = true;
                }
                given += take;
                w_base += take;
            }
        }
        if (__ballot_sync(0xffffffffu, alive) == 0)
            break;
        const bool working = alive && !(link & (kLinkWait | kLinkMerge));
        const uint32_t wmask = __ballot_sync(0xffffffffu, working);
        // node phase as in the plain kernels, every lane taking part
        // (traverse.cuh: node_phase)
        bool overflow = false;
        node_phase<LAYOUT, false, MIXED>(nodes, working, wmask, a.phase_break, next, r, best, st, overflow, unused);
        if (working) {
            // a plane occluding the ray at its start decides it in this first
            // round only (the lane may next help another ray in the tail)
            bool occluded = occluded_at_start;
            occluded_at_start = false;
            if (next < 0) {
                if (MIXED)
                    occluded = mode ? process_leaf_mixed<true>(prims, next, r, best)
                                    : process_leaf_mixed<false>(prims, next, r, best);
                else
                    occluded = mode ? process_leaf<true, false>(prims, next, r, best, unused)
                                    : process_leaf<false, false>(prims, next, r, best, unused);
                if (!occluded)
                    next = st.pop_live(best.tcull);
            }
            if (overflow)
                atomicOr(a.status, kStatusStackOverflow);
            if (occluded || next == kRefDone) {
                if (queue_done) {
                    // share_tail writes the ray once no helper of it remains
                    link |= ((link & 31u) == lane ? kLinkWait : kLinkMerge) | (occluded ? kLinkOcc : 0u);
                } else {
                    write_result<MIXED>(out, mode, ray, r, best, occluded);
                    alive = false;
                }
            }
        }
    }
    if (a.times && lane == 0)
        atomicMax(a.times + 1, global_ns());
}

using BatchFn = void (*)(BatchArgs);

static BatchFn select_batch_kernel(uint32_t layout, bool mixed) {
    constexpr int B2 = IGXRT_LAYOUT_BVH2, B4 = IGXRT_LAYOUT_BVH4, B8 = IGXRT_LAYOUT_BVH8;
    if (mixed)
        return layout == B8 ? batch_kernel<B8, true> : layout == B4 ? batch_kernel<B4, true> : batch_kernel<B2, true>;
    return layout == B8 ? batch_kernel<B8, false> : layout == B4 ? batch_kernel<B4, false> : batch_kernel<B2, false>;
}

namespace {

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

}  // namespace

void batch_item_for(const igxrt_scene* scene, const igxrt_launch_params& p, const igxrt_ray* rays,
                    const uint32_t* prev, void* out, uint32_t count, uint32_t mode, BatchItemDev& d) {
    d.nodes = reinterpret_cast<const float4*>(scene->nodes[p.layout]);
    d.prims = reinterpret_cast<const float4*>(scene->prims);
    d.rays = rays;
    d.prev = prev;
    d.out = out;
    d.planes = reinterpret_cast<const float4*>(scene->planes);
    d.count = count;
    d.mode = mode;
    d.node_count = scene->node_count[p.layout];
    d.packet_begin = 0;
    d.plane_count = scene->plane_count;
    d.plane_base = scene->plane_base;
}

igxrt_status build_batch_table(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                               const igxrt_launch_params& p, std::vector<BatchItemDev>& table,
                               uint32_t& total_packets, uint64_t& total_rays, bool& mixed) {
    if (count && !items)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "items is NULL");
    table.resize(count);
    uint64_t packets = 0;
    total_rays = 0;
    mixed = false;
    for (uint32_t i = 0; i < count; ++i) {
        const igxrt_batch_item& it = items[i];
        if (!it.scene)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: scene is NULL", i));
        if (it.scene->device != ctx->device)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: scene on another device", i));
        if (!it.scene->has_layout(p.layout))
            return fail(ctx, IGXRT_ERROR_UNSUPPORTED, format("item %u: the scene has no layout %u", i, p.layout));
        if (it.mode > 1)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: unknown mode %u", i, it.mode));
        if (it.count && (!it.rays || !it.out))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: NULL rays or output", i));
        if (!aligned(it.rays, 16) || !aligned(it.out, it.mode ? 4 : 16) || !aligned(it.prev_hit, 4))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: misaligned array", i));
        if (it.count > 0x7fffffffu)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("item %u: too many rays", i));
        if (it.count && (!device_accessible(it.rays) || !device_accessible(it.out) ||
                         !device_accessible(it.prev_hit)))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                        format("item %u: batch arrays must be device memory", i));
        BatchItemDev& d = table[i];
        batch_item_for(it.scene, p, it.rays, it.prev_hit, it.out, it.count, it.mode, d);
        d.packet_begin = (uint32_t)packets;
        mixed |= it.scene->mixed;
        packets += (it.count + p.packet_size - 1) / p.packet_size;
        total_rays += it.count;
        if (packets >= 0x7fffffffu)
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "too many packets in one batch");
    }
    total_packets = (uint32_t)packets;
    return IGXRT_OK;
}

igxrt_status launch_batch(igxrt_context* ctx, const BatchItemDev* d_table, uint32_t count,
                          uint32_t total_packets, uint64_t total_rays, const igxrt_launch_params& p,
                          uint32_t* queue, cudaStream_t stream, bool mixed, unsigned long long* times) {
    if (total_packets == 0)
        return IGXRT_OK;
    BatchFn fn = select_batch_kernel(p.layout, mixed);
    const size_t smem = (size_t)p.stack_depth * p.block_size * kStackEntryBytes;
    int per_sm = 0;
    cudaError_t e = allow_smem((const void*)fn, smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)p.block_size, smem);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "occupancy query");
    if (per_sm < 1)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "launch parameters leave no resident CTA");
    if (p.ctas_per_sm)
        per_sm = std::min(per_sm, (int)p.ctas_per_sm);
    const uint64_t lanes_needed = total_rays;
    const uint64_t ctas_needed = (lanes_needed + p.block_size - 1) / p.block_size;
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, ctas_needed));
    BatchArgs a;
    a.items = d_table;
    a.item_count = count;
    a.total_packets = total_packets;
    a.queue = queue;
    a.status = status_word(ctx);
    a.packet = p.packet_size;
    a.sh_depth = p.stack_depth;
    a.refill_lanes = p.refill_lanes;
    a.phase_break = p.phase_break;
    a.times = times;
    e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch queue reset");
    fn<<<grid, p.block_size, smem, stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch kernel launch");
    return IGXRT_OK;
}

// Batch tables for igxrt_trace_batch: a ring of slots in one allocation; a
// slot is reused only after the launch that read it has completed.
igxrt_status batch_slot(igxrt_context* ctx, uint32_t count, BatchItemDev** slot, cudaEvent_t** done) {
    if (count > kBatchSlotItems)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("%u items exceed %u per igxrt_trace_batch call (use igxrt_batch_create)",
                           count, kBatchSlotItems));
    if (!ctx->d_batch) {
        const size_t bytes = (size_t)kBatchSlots * kBatchSlotItems * sizeof(BatchItemDev);
        cudaError_t e = cudaMalloc(&ctx->d_batch, bytes);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "batch table allocation");
        for (uint32_t i = 0; i < kBatchSlots; ++i) {
            e = cudaEventCreateWithFlags(&ctx->batch_events[i], cudaEventDisableTiming);
            if (e != cudaSuccess)
                return cuda_fail(ctx, e, "batch event");
        }
    }
    const uint32_t s = ctx->next_batch_slot;
    ctx->next_batch_slot = (s + 1) % kBatchSlots;
    cudaError_t e = cudaEventSynchronize(ctx->batch_events[s]);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch slot reuse");
    *slot = reinterpret_cast<BatchItemDev*>(ctx->d_batch) + (size_t)s * kBatchSlotItems;
    *done = &ctx->batch_events[s];
    return IGXRT_OK;
}

}  // namespace igxrt

using namespace igxrt;

struct igxrt_batch {
    igxrt_context* ctx = nullptr;
    void* d_mem = nullptr;  // item table + queue word
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t total_rays = 0;
};

extern "C" {

igxrt_status igxrt_trace_batch(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                               void* stream_ptr) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_launch_params p;
    igxrt_status st = resolve_params(ctx, ctx->params, p);
    if (st != IGXRT_OK)
        return st;
    std::vector<BatchItemDev> table;
    uint32_t packets = 0;
    uint64_t rays = 0;
    bool mixed = false;
    st = build_batch_table(ctx, items, count, p, table, packets, rays, mixed);
    if (st != IGXRT_OK || packets == 0)
        return st;
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    BatchItemDev* d_table = nullptr;
    cudaEvent_t* done = nullptr;
    st = batch_slot(ctx, count, &d_table, &done);
    if (st != IGXRT_OK)
        return st;
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    cudaError_t e = cudaMemcpyAsync(d_table, table.data(), table.size() * sizeof(BatchItemDev),
                                    cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch table upload");
    uint32_t* queue = take_queue_slot(ctx);
    st = launch_batch(ctx, d_table, count, packets, rays, p, queue, stream, mixed);
    if (st != IGXRT_OK)
        return st;
    // the ring's slots are zero between launches (trace launches skip the
    // reset and rely on it)
    e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), stream);
    if (e == cudaSuccess)
        e = cudaEventRecord(*done, stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch slot event");
    return IGXRT_OK;
}

igxrt_status igxrt_batch_create(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                                const igxrt_launch_params* params, igxrt_batch** out) {
    if (!ctx || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_launch_params p;
    igxrt_status st = resolve_params(ctx, params ? *params : ctx->params, p);
    if (st != IGXRT_OK)
        return st;
    std::vector<BatchItemDev> table;
    uint32_t packets = 0;
    uint64_t rays = 0;
    bool mixed = false;
    st = build_batch_table(ctx, items, count, p, table, packets, rays, mixed);
    if (st != IGXRT_OK)
        return st;
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    igxrt_batch* b = new (std::nothrow) igxrt_batch();
    if (!b)
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "batch object");
    b->ctx = ctx;
    b->total_rays = rays;
    const size_t tb = (table.size() * sizeof(BatchItemDev) + 255) / 256 * 256;
    cudaError_t e = cudaMalloc(&b->d_mem, tb + 256);
    if (e == cudaSuccess && !table.empty())
        e = cudaMemcpy(b->d_mem, table.data(), table.size() * sizeof(BatchItemDev), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (b->d_mem)
            cudaFree(b->d_mem);
        delete b;
        return cuda_fail(ctx, e, "batch table");
    }
    uint32_t* queue = reinterpret_cast<uint32_t*>(static_cast<char*>(b->d_mem) + tb);
    cudaStream_t cap = nullptr;
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        st = launch_batch(ctx, static_cast<const BatchItemDev*>(b->d_mem), count, packets, rays, p,
                          queue, cap, mixed);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
        b->graph = g;
        if (st == IGXRT_OK && e2 != cudaSuccess)
            st = cuda_fail(ctx, e2, "batch graph capture");
        if (st == IGXRT_OK && b->graph) {
            e = cudaGraphInstantiate(&b->exec, b->graph, 0);
            if (e != cudaSuccess)
                st = cuda_fail(ctx, e, "batch graph instantiate");
        }
    } else {
        st = cuda_fail(ctx, e, "batch capture stream");
    }
    if (cap)
        cudaStreamDestroy(cap);
    if (st != IGXRT_OK) {
        igxrt_batch_destroy(b);
        return st;
    }
    *out = b;
    return IGXRT_OK;
}

igxrt_status igxrt_batch_launch(igxrt_batch* b, void* stream) {
    if (!b)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (!b->exec)
        return IGXRT_OK;  // an empty batch captured nothing
    DeviceGuard guard(b->ctx->device);
    const cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(b->ctx, e, "batch graph launch");
    return IGXRT_OK;
}

igxrt_status igxrt_batch_destroy(igxrt_batch* b) {
    if (!b)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    {
        DeviceGuard guard(b->ctx->device);
        cudaDeviceSynchronize();
        if (b->exec)
            cudaGraphExecDestroy(b->exec);
        if (b->graph)
            cudaGraphDestroy(b->graph);
        if (b->d_mem)
            cudaFree(b->d_mem);
    }
    delete b;
    return IGXRT_OK;
}

}  // extern "C"
