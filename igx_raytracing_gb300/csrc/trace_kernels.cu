// trace_kernels.cu — the plain traversal kernels and their launcher.
//
// One persistent kernel per (node layout, query mode, instrumentation):
// CTAs stay resident, each warp repeatedly takes a packet of `packet` rays
// from a global atomic work queue and its lanes trace them, so uneven ray
// costs (a miss of the root box vs. a deep closest hit) balance across the
// GPU without a tail of idle SMs.  Node and primitive records are read with
// 128-bit read-only loads; hit records are written with streaming stores so
// they do not displace BVH lines from L2.
#include <algorithm>

#include "engine.h"
#include "gbuffer.cuh"
#include "share.cuh"
#include "traverse.cuh"

namespace igxrt {

static_assert(kStackCapacityDevice == kStackCapacity, "stack capacity mismatch");
static_assert(sizeof(igxrt_bvh2_node) == 64, "BVH2 node must be 64 bytes");
static_assert(sizeof(igxrt_bvh4_node) == 128, "BVH4 node must be 128 bytes");
static_assert(sizeof(igxrt_prim_record) == 48, "primitive record must be 48 bytes");
static_assert(sizeof(igxrt_ray) == 32, "ray must be 32 bytes");
static_assert(sizeof(igxrt_hit) == 16, "hit must be 16 bytes");

struct KernelArgs {
    const float4* nodes;
    const float4* prims;
    uint32_t node_count;
    const igxrt_ray* rays;
    const uint32_t* prev;
    uint32_t count;
    const uint32_t* count_dev;  // non-null: the ray count is this device word (at most `count`)
    igxrt_hit* hits;
    uint32_t* occluded;
    uint32_t* node_fetches;
    uint32_t* prim_fetches;
    uint32_t* queue;
    uint32_t* status;
    uint32_t packet;
    uint32_t sh_depth;
    uint32_t refill_lanes;
    uint32_t phase_break;  // node_phase's early end (igxrt_launch_params.phase_break)
    const float4* planes;  // mixed scenes: planes outside the tree
    uint32_t plane_count;
    uint32_t plane_base;   // object id of the first plane
    // non-null: the queue slot's exit counter; the last warp to leave zeroes
    // it and the queue word, so the slot needs no reset before its next launch
    uint32_t* exit_count;
    uint32_t independent;  // IGXRT_TRACE_INDEPENDENT: no wait for the kernel before
    CameraSource camera;   // CAMERA kernels: the rays' camera
};

template <bool ANY, bool COUNT, bool MIXED>
__device__ __forceinline__ void finish_ray(const KernelArgs& a, uint32_t i, const RayState& r,
                                           const BestHit& best, bool occluded, uint32_t nf,
                                           uint32_t pf) {
    if (ANY) {
        __stcs(a.occluded + i, occluded ? 1u : 0u);
    } else {
        const bool hit = MIXED ? (best.t < r.tmax_eff || best.prim < kPrioNone) : best.t < r.tmax_eff;
        const uint32_t prim = MIXED ? id_of_prio(best.prim) : best.prim;
        const float4 h = hit ? make_float4(best.t, best.u, best.v, __uint_as_float(prim))
                             : make_float4(IGXRT_NO_HIT, 0.f, 0.f, __uint_as_float(IGXRT_NO_RAY_HIT));
        __stcs(reinterpret_cast<float4*>(a.hits) + i, h);
    }
    if (COUNT) {
        a.node_fetches[i] = nf;
        a.prim_fetches[i] = pf;
    }
}

// Register budget per instantiation: what each reached before the tail
// sharing was added, so the sharing (run once a warp's queue is drained)
// leaves every kernel's occupancy where it was.
constexpr int trace_kernel_regs(int layout, bool any, bool mixed) {
    return layout == IGXRT_LAYOUT_BVH2   ? (mixed && !any ? 64 : 56)
           : layout == IGXRT_LAYOUT_BVH4 ? (mixed && !any ? 72 : 64)
                                         : (any && !mixed ? 64 : 80);
}

// Persistent traversal.  Every lane owns one ray at a time; a warp alternates
// a node phase (each lane descends until it reaches a leaf or finishes, or
// until few lanes still descend: node_phase) and a leaf phase (each lane at
// a leaf tests it), so lanes at the same kind of work execute together.  Between phases, once `refill_lanes` lanes are idle the
// warp hands them new rays: one atomicAdd on the global queue claims a
// packet of `packet` ray indices for the warp, and idle lanes take the next
// indices in lane order (ballot + popc).  Until the warp finds the queue
// drained, and always in the instrumented (COUNT) kernels, each ray's
// sequence of node and leaf visits is exactly the host traversal's
// (oracle/trace_oracle.c); after that share_tail splits rays across lanes,
// which visits the same subtrees in another order with the same result.
// MIXED: scenes with spheres, cubes and planes (typed leaves, planes tested
// when a ray starts, priority-coded best hit).  CAMERA: ray i is made in the
// kernel, the camera's primary ray of pixel i in row-major order
// (igxrt_trace_gbuffer; closest hit on triangles).
template <int LAYOUT, bool ANY, bool COUNT, bool MIXED, bool CAMERA = false>
__global__ void __maxnreg__(trace_kernel_regs(LAYOUT, ANY, MIXED)) trace_kernel(KernelArgs a) {
    static_assert(!CAMERA || (!ANY && !COUNT && !MIXED), "camera rays: closest hit on triangles");
    // Launched with programmatic stream serialization: unless the caller
    // stated independence, wait until the kernel queued before this one has
    // finished and its writes are visible (a no-op after any other work)
    if (!a.independent)
        asm volatile("griddepcontrol.wait;" ::: "memory");
    extern __shared__ uint32_t smem[];
    TraversalStack st;
    st.sh = reinterpret_cast<uint2*>(smem) + threadIdx.x;
    st.stride = blockDim.x;
    st.sh_depth = a.sh_depth;
    st.sp = 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lower = (1u << lane) - 1u;
    uint32_t pk_base = 0, pk_end = 0;  // warp-uniform window of claimed rays
    bool queue_done = false;           // warp-uniform
    bool alive = false, occluded_at_start = false;
    uint32_t ray = 0, nf = 0, pf = 0;
    int32_t next = kRefDone;
    const uint32_t count = a.count_dev ? min(*a.count_dev, a.count) : a.count;
    RayState r;
    BestHit best;
    // work sharing in the tail (share_tail); the instrumented kernels keep
    // the single-lane order their fetch counts describe
    constexpr bool STEAL = !COUNT;
    uint32_t link = lane;
    for (;;) {
        if (STEAL && queue_done &&
            __ballot_sync(0xffffffffu, !alive || (link & (kLinkWait | kLinkMerge))) != 0) {
            NoLaneExtra none;
            share_tail<ANY ? kShareAny : kShareClosest>(
                lane, lower, link, alive, ray, r, best, st, next, none,
                [&](bool occ) { finish_ray<ANY, false, MIXED>(a, ray, r, best, occ, 0, 0); },
                MIXED ? kPrioNone : 0u);
        }
        const uint32_t idle = __ballot_sync(0xffffffffu, !alive);
        const uint32_t nidle = __popc(idle);
        if (!queue_done && nidle != 0 && (nidle >= a.refill_lanes || nidle == 32)) {
            const uint32_t rank = __popc(idle & lower);
            uint32_t given = 0;
            while (given < nidle) {
                if (pk_base >= pk_end) {
                    uint32_t b = 0;
                    if (lane == 0)
                        b = atomicAdd(a.queue, a.packet);
                    b = __shfl_sync(0xffffffffu, b, 0);
                    if (b >= count) {
                        queue_done = true;
                        // every ray is claimed: the next kernel on the stream
                        // may start on the SMs this launch's tail leaves idle
                        asm volatile("griddepcontrol.launch_dependents;");
                        break;
                    }
                    pk_base = b;
                    pk_end = min(b + a.packet, count);
                }
                const uint32_t take = min(nidle - given, pk_end - pk_base);
                if (!alive && rank >= given && rank < given + take) {
                    ray = pk_base + (rank - given);
                    if (CAMERA) {
                        const uint32_t y = ray / a.camera.cam.width, x = ray - y * a.camera.cam.width;
                        r = camera_ray_state(a.camera.cam,
                                             camera_dir(a.camera.cam, a.camera.inv_w, a.camera.inv_h, x, y));
                    } else {
                        r = load_ray(a.rays, ray, a.prev ? __ldg(a.prev + ray) : IGXRT_NO_RAY_HIT);
                    }
                    best.t = r.tmax_eff;
                    best.u = 0.f;
                    best.v = 0.f;
                    // "prim < best.prim" cannot hold before a first hit
                    best.prim = MIXED ? kPrioNone : 0u;
                    best.tcull = cull_limit(best.t);
                    next = a.node_count ? 0 : kRefDone;
                    occluded_at_start = false;
                    if (MIXED && a.plane_count) {
                        occluded_at_start = test_planes<ANY>(a.planes, a.plane_count, a.plane_base, r, best);
                        if (occluded_at_start)
                            next = kRefDone;
                    }
                    st.sp = 0;
                    nf = 0;
                    pf = 0;
                    alive = true;
                }
                given += take;
                pk_base += take;
            }
        }
        if (__ballot_sync(0xffffffffu, alive) == 0)
            break;  // only reachable once the queue is drained
        const bool working = alive && !(STEAL && (link & (kLinkWait | kLinkMerge)));
        const uint32_t wmask = __ballot_sync(0xffffffffu, working);
        // node phase: every lane of the warp takes part, the working lanes
        // descend (traverse.cuh: node_phase, which may end it early)
        bool overflow = false;
        node_phase<LAYOUT, COUNT, MIXED>(a.nodes, working, wmask, a.phase_break, next, r, best, st, overflow, nf);
        if (working) {
            // a plane occluding the ray when it started decides it in this
            // first round; the flag must not outlive the ray (the lane may
            // next help another ray's traversal in the tail)
            bool occluded = occluded_at_start;
            occluded_at_start = false;
            // leaf phase
            if (next < 0) {
                occluded = MIXED ? process_leaf_mixed<ANY, COUNT>(a.prims, next, r, best, &pf)
                                 : process_leaf<ANY, COUNT>(a.prims, next, r, best, pf);
                if (!occluded)
                    next = st.pop_live(best.tcull);
            }
            if (overflow)
                atomicOr(a.status, kStatusStackOverflow);
            if (occluded || next == kRefDone) {
                if (STEAL && queue_done) {
                    // share_tail writes the ray once no helper of it remains
                    link |= ((link & 31u) == lane ? kLinkWait : kLinkMerge) | (occluded ? kLinkOcc : 0u);
                } else {
                    finish_ray<ANY, COUNT, MIXED>(a, ray, r, best, occluded, nf, pf);
                    alive = false;
                }
            }
        }
    }
    if (a.exit_count && lane == 0) {
        // every warp's queue claims come before its exit count
        __threadfence();
        const uint32_t warps = gridDim.x * (blockDim.x >> 5);
        if (atomicAdd(a.exit_count, 1u) == warps - 1u) {
            *a.queue = 0u;
            *a.exit_count = 0u;
        }
    }
}

using KernelFn = void (*)(KernelArgs);

// Every variant has an instrumented twin (COUNT) that also writes per-ray
// fetch counts; for triangle-only scenes they equal the host traversal's.
static KernelFn select_kernel(uint32_t layout, bool any, bool count, bool mixed) {
    constexpr int B2 = IGXRT_LAYOUT_BVH2, B4 = IGXRT_LAYOUT_BVH4, B8 = IGXRT_LAYOUT_BVH8;
    if (mixed) {
        if (count) {  // instrumented mixed kernels: no host traversal to compare with
            if (layout == B8)
                return any ? trace_kernel<B8, true, true, true> : trace_kernel<B8, false, true, true>;
            if (layout == B4)
                return any ? trace_kernel<B4, true, true, true> : trace_kernel<B4, false, true, true>;
            return any ? trace_kernel<B2, true, true, true> : trace_kernel<B2, false, true, true>;
        }
        if (layout == B8)
            return any ? trace_kernel<B8, true, false, true> : trace_kernel<B8, false, false, true>;
        if (layout == B4)
            return any ? trace_kernel<B4, true, false, true> : trace_kernel<B4, false, false, true>;
        return any ? trace_kernel<B2, true, false, true> : trace_kernel<B2, false, false, true>;
    }
    if (layout == B8) {
        if (count)
            return any ? trace_kernel<B8, true, true, false> : trace_kernel<B8, false, true, false>;
        return any ? trace_kernel<B8, true, false, false> : trace_kernel<B8, false, false, false>;
    }
    if (layout == B4) {
        if (count)
            return any ? trace_kernel<B4, true, true, false> : trace_kernel<B4, false, true, false>;
        return any ? trace_kernel<B4, true, false, false> : trace_kernel<B4, false, false, false>;
    }
    if (count)
        return any ? trace_kernel<B2, true, true, false> : trace_kernel<B2, false, true, false>;
    return any ? trace_kernel<B2, true, false, false> : trace_kernel<B2, false, false, false>;
}

static KernelFn select_camera_kernel(uint32_t layout) {
    constexpr int B2 = IGXRT_LAYOUT_BVH2, B4 = IGXRT_LAYOUT_BVH4, B8 = IGXRT_LAYOUT_BVH8;
    return layout == B8   ? trace_kernel<B8, false, false, false, true>
           : layout == B4 ? trace_kernel<B4, false, false, false, true>
                          : trace_kernel<B2, false, false, false, true>;
}

namespace {

// The launch shape and arguments every traversal launch shares: the kernel
// for the scene and query, its shared stack, a persistent grid of at most the
// resident CTAs (fewer when the rays need fewer warps), and the scene, ray
// and output pointers.  The caller adds the work-queue, error and exit words.
struct TraceLaunch {
    KernelFn fn = nullptr;
    size_t smem = 0;
    uint32_t grid = 0;
    KernelArgs a{};
};

igxrt_status prepare_trace(igxrt_context* ctx, const TraceRequest& req, const igxrt_launch_params& p,
                           TraceLaunch& l) {
    const igxrt_scene* s = req.scene;
    if (req.camera && (s->mixed || req.mode != 0 || req.node_fetches))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, "camera rays are traced for closest hits on triangles");
    l.fn = req.camera ? select_camera_kernel(p.layout)
                      : select_kernel(p.layout, req.mode == 1, req.node_fetches != nullptr, s->mixed);
    l.smem = (size_t)p.stack_depth * p.block_size * kStackEntryBytes;
    int per_sm = 0;
    cudaError_t e = allow_smem((const void*)l.fn, l.smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, l.fn, (int)p.block_size, l.smem);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "occupancy query");
    if (per_sm < 1)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "launch parameters leave no resident CTA");
    if (p.ctas_per_sm)
        per_sm = std::min(per_sm, (int)p.ctas_per_sm);
    const uint64_t warps_needed = ((uint64_t)req.count + p.packet_size - 1) / p.packet_size;
    const uint64_t ctas_needed = (warps_needed + p.block_size / 32 - 1) / (p.block_size / 32);
    l.grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, ctas_needed));

    KernelArgs& a = l.a;
    a.nodes = reinterpret_cast<const float4*>(s->nodes[p.layout]);
    a.prims = reinterpret_cast<const float4*>(s->prims);
    a.node_count = s->node_count[p.layout];
    a.rays = req.rays;
    a.prev = req.prev;
    a.count = req.count;
    a.count_dev = req.count_dev;
    a.hits = req.hits;
    a.occluded = req.occluded;
    a.node_fetches = req.node_fetches;
    a.prim_fetches = req.prim_fetches;
    a.packet = p.packet_size;
    a.sh_depth = p.stack_depth;
    a.refill_lanes = p.refill_lanes;
    a.phase_break = p.phase_break;
    a.planes = reinterpret_cast<const float4*>(s->planes);
    a.plane_count = s->plane_count;
    a.plane_base = s->plane_base;
    a.queue = nullptr;
    a.status = nullptr;
    a.exit_count = nullptr;
    a.independent = 0u;
    if (req.camera)
        a.camera = *req.camera;
    return IGXRT_OK;
}

}  // namespace

igxrt_status launch_trace(igxrt_context* ctx, const TraceRequest& req,
                          const igxrt_launch_params& p, cudaStream_t stream) {
    if (req.count == 0)
        return IGXRT_OK;
    TraceLaunch l;
    igxrt_status st = prepare_trace(ctx, req, p, l);
    if (st != IGXRT_OK)
        return st;
    l.a.queue = take_queue_slot(ctx);
    l.a.status = status_word(ctx);
    // the slot's words are zero (zeroed at context creation, and by the last
    // warp of the slot's previous launch), so no reset sits between this
    // launch and the kernel before it
    l.a.exit_count = exit_word(l.a.queue);
    l.a.independent = req.independent ? 1u : 0u;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(l.grid);
    cfg.blockDim = dim3(p.block_size);
    cfg.dynamicSmemBytes = l.smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, l.fn, l.a);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "trace kernel launch");
    return IGXRT_OK;
}

igxrt_status launch_trace_words(igxrt_context* ctx, const TraceRequest& req,
                                const igxrt_launch_params& p, cudaStream_t stream,
                                uint32_t* queue, uint32_t* status) {
    if (req.count == 0)
        return IGXRT_OK;
    TraceLaunch l;
    igxrt_status st = prepare_trace(ctx, req, p, l);
    if (st != IGXRT_OK)
        return st;
    l.a.queue = queue;
    l.a.status = status;  // the caller resets both words; no exit counter
    l.fn<<<l.grid, p.block_size, l.smem, stream>>>(l.a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "trace kernel launch");
    return IGXRT_OK;
}

}  // namespace igxrt
