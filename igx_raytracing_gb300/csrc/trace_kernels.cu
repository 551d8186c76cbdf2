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
    const float4* planes;  // mixed scenes: planes outside the tree
    uint32_t plane_count;
    uint32_t plane_base;   // object id of the first plane
    // non-null: the queue slot's exit counter; the last warp to leave zeroes
    // it and the queue word, so the slot needs no reset before its next launch
    uint32_t* exit_count;
    uint32_t independent;  // IGXRT_TRACE_INDEPENDENT: no wait for the kernel before
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

// ---- work sharing once the queue is drained --------------------------------
//
// After a warp finds the queue empty its lanes finish the rays they hold, and
// the warp runs until its slowest ray is done while finished lanes idle.
// From then on an idle lane takes the bottom entry (the oldest, largest
// pending subtree) of a busy lane's stack and traverses it for the same ray,
// as a helper of the lane that owns the ray.  A helper keeps its own best hit
// and stack; when its subtrees are done it hands the best hit to the owner,
// and the owner writes the ray's result once its own traversal is over and no
// helper of its ray remains.  The result equals the single-lane traversal's:
// the closest hit is the smallest (t, prim) among the accepted triangles, and
// every box pruned by a cull limit (the owner's, which a helper adopts) holds
// no triangle that beats the hit behind that limit; an any-hit result is the
// OR over the same triangles.  `link` holds the owner lane (bits 0-4; the
// lane itself for its own ray) and the flags below.
constexpr uint32_t kLinkWait = 1u << 8;   // owner: traversal over, helpers pending
constexpr uint32_t kLinkMerge = 1u << 9;  // helper: subtrees done, best hit to hand over
constexpr uint32_t kLinkOcc = 1u << 10;   // any-hit: an occluder was found

template <bool ANY>
__device__ __forceinline__ void share_tail(const KernelArgs& a, uint32_t lane, uint32_t lower,
                                           uint32_t& link, bool& alive, uint32_t& ray, RayState& r,
                                           BestHit& best, TraversalStack& st, int32_t& next) {
    constexpr uint32_t FULL = 0xffffffffu;
    // 1. finished helpers hand their best hit (or occluder) to the owner
    uint32_t m = __ballot_sync(FULL, alive && (link & kLinkMerge));
    while (m) {
        const int h = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t hl = __shfl_sync(FULL, link, h);
        const uint32_t o = hl & 31u;
        if (ANY) {
            if (lane == o)
                link |= hl & kLinkOcc;
        } else {
            // (t, prim) decide; u and v follow one at a time (few live registers)
            const float ht = __shfl_sync(FULL, best.t, h);
            const uint32_t hp = __shfl_sync(FULL, best.prim, h);
            const bool take = lane == o && (ht < best.t || (ht == best.t && hp < best.prim));
            if (take) {
                best.t = ht;
                best.prim = hp;
                best.tcull = cull_limit(ht);
            }
            const float hu = __shfl_sync(FULL, best.u, h);
            if (take)
                best.u = hu;
            const float hv = __shfl_sync(FULL, best.v, h);
            if (take)
                best.v = hv;
        }
    }
    if (alive && (link & kLinkMerge)) {
        alive = false;
        link = lane;
    }
    // 2. any-hit: the helpers of an occluded ray stop
    if (ANY) {
        const uint32_t ol = __shfl_sync(FULL, link, link & 31u);
        if (alive && (link & 31u) != lane && (ol & kLinkOcc)) {
            alive = false;
            link = lane;
        }
    }
    // 3. an owner whose ray is decided and has no helper left writes it
    const uint32_t grp = __match_any_sync(FULL, alive ? (link & 31u) : 32u + lane);
    if (alive && (link & 31u) == lane && (link & (kLinkWait | kLinkOcc)) && grp == (1u << lane)) {
        finish_ray<ANY, false, false>(a, ray, r, best, (link & kLinkOcc) != 0, 0, 0);
        alive = false;
        link = lane;
    }
    // helpers prune with their owner's cull limit when it is tighter
    if (!ANY) {
        const float otc = __shfl_sync(FULL, best.tcull, link & 31u);
        if (alive && (link & 31u) != lane && otc < best.tcull)
            best.tcull = otc;
    }
    // 4. idle lanes take the bottom entries of busy lanes' stacks: the idle
    //    lanes are dealt round-robin over the busy ones, the j-th thief of a
    //    victim taking its entry j (entries in shared memory only)
    const uint32_t idle = __ballot_sync(FULL, !alive);
    const uint32_t can = __ballot_sync(FULL, alive && !(link & (kLinkWait | kLinkMerge)) && st.sp > 0);
    const uint32_t nt = __popc(idle), nv = __popc(can);
    if (nt == 0 || nv == 0)
        return;
    const uint32_t ri = __popc(idle & lower), rv = __popc(can & lower);
    uint32_t src = lane, j = 0;
    if (!alive) {
        uint32_t mm = can;
        for (uint32_t k = ri % nv; k > 0; --k)
            mm &= mm - 1;
        src = __ffs(mm) - 1;
        j = ri / nv;
    }
    const uint32_t vsp = __shfl_sync(FULL, st.sp, src);
    const uint32_t vray = __shfl_sync(FULL, ray, src), vlink = __shfl_sync(FULL, link, src);
    const float vtc = __shfl_sync(FULL, best.tcull, src);
    // the victim's ray, read in place: a lane that is no thief reads its own
    r.ox = __shfl_sync(FULL, r.ox, src);
    r.oy = __shfl_sync(FULL, r.oy, src);
    r.oz = __shfl_sync(FULL, r.oz, src);
    r.dx = __shfl_sync(FULL, r.dx, src);
    r.dy = __shfl_sync(FULL, r.dy, src);
    r.dz = __shfl_sync(FULL, r.dz, src);
    r.ix = __shfl_sync(FULL, r.ix, src);
    r.iy = __shfl_sync(FULL, r.iy, src);
    r.iz = __shfl_sync(FULL, r.iz, src);
    r.oix = __shfl_sync(FULL, r.oix, src);
    r.oiy = __shfl_sync(FULL, r.oiy, src);
    r.oiz = __shfl_sync(FULL, r.oiz, src);
    r.tmin = __shfl_sync(FULL, r.tmin, src);
    r.tmin_box = __shfl_sync(FULL, r.tmin_box, src);
    r.tmax_eff = __shfl_sync(FULL, r.tmax_eff, src);
    r.prev = __shfl_sync(FULL, r.prev, src);
    const bool thief = !alive && j < min(vsp, st.sh_depth);
    uint2 e = make_uint2(0u, 0u);
    if (thief)
        e = (st.sh + ((int)src - (int)lane))[j * st.stride];  // entry j of the victim's column
    __syncwarp();
    if ((can >> lane) & 1u) {
        // the thieves dealt to this lane took its entries 0 .. g-1
        const uint32_t dealt = rv < nt ? (nt - 1 - rv) / nv + 1 : 0u;
        const uint32_t g = min(dealt, min(st.sp, st.sh_depth));
        if (g)
            st.drop_bottom(g);
    }
    __syncwarp();
    if (thief && __uint_as_float(e.y) <= vtc) {
        ray = vray;
        link = vlink & 31u;
        best.t = r.tmax_eff;
        best.u = 0.f;
        best.v = 0.f;
        best.prim = 0u;
        best.tcull = vtc;
        next = (int32_t)e.x;
        st.sp = 0;
        alive = true;
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
// a node phase (each lane descends until it reaches a leaf or finishes) and a
// leaf phase (each lane tests one leaf), so lanes at the same kind of work
// execute together.  Between phases, once `refill_lanes` lanes are idle the
// warp hands them new rays: one atomicAdd on the global queue claims a
// packet of `packet` ray indices for the warp, and idle lanes take the next
// indices in lane order (ballot + popc).  Until the warp finds the queue
// drained, and always in the instrumented (COUNT) kernels, each ray's
// sequence of node and leaf visits is exactly the host traversal's
// (oracle/trace_oracle.c); after that share_tail splits rays across lanes,
// which visits the same subtrees in another order with the same result.
// MIXED: scenes with spheres, cubes and planes (typed leaves, planes tested
// when a ray starts, priority-coded best hit).
template <int LAYOUT, bool ANY, bool COUNT, bool MIXED>
__global__ void __maxnreg__(trace_kernel_regs(LAYOUT, ANY, MIXED)) trace_kernel(KernelArgs a) {
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
    constexpr bool STEAL = !COUNT && !MIXED;
    uint32_t link = lane;
    for (;;) {
        if (STEAL && queue_done &&
            __ballot_sync(0xffffffffu, !alive || (link & (kLinkWait | kLinkMerge))) != 0)
            share_tail<ANY>(a, lane, lower, link, alive, ray, r, best, st, next);
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
                    r = load_ray(a.rays, ray, a.prev ? __ldg(a.prev + ray) : IGXRT_NO_RAY_HIT);
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
        if (alive && !(STEAL && (link & (kLinkWait | kLinkMerge)))) {
            bool overflow = false;
            // node phase
            while (next >= 0 && next != kRefDone)
                next = visit_node<LAYOUT, COUNT, MIXED>(a.nodes, next, r, best, st, overflow, nf);
            bool occluded = occluded_at_start;
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

igxrt_status launch_trace(igxrt_context* ctx, const TraceRequest& req,
                          const igxrt_launch_params& p, cudaStream_t stream) {
    if (req.count == 0)
        return IGXRT_OK;
    const igxrt_scene* s = req.scene;
    const bool count = req.node_fetches != nullptr;
    KernelFn fn = select_kernel(p.layout, req.mode == 1, count, s->mixed);
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
    const uint64_t warps_needed = ((uint64_t)req.count + p.packet_size - 1) / p.packet_size;
    const uint64_t ctas_needed = (warps_needed + p.block_size / 32 - 1) / (p.block_size / 32);
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, ctas_needed));

    KernelArgs a;
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
    a.queue = take_queue_slot(ctx);
    a.status = status_word(ctx);
    a.packet = p.packet_size;
    a.sh_depth = p.stack_depth;
    a.refill_lanes = p.refill_lanes;
    a.planes = reinterpret_cast<const float4*>(s->planes);
    a.plane_count = s->plane_count;
    a.plane_base = s->plane_base;
    // the slot's words are zero (zeroed at context creation, and by the last
    // warp of the slot's previous launch), so no reset sits between this
    // launch and the kernel before it
    a.exit_count = exit_word(a.queue);
    a.independent = req.independent ? 1u : 0u;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(p.block_size);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, fn, a);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "trace kernel launch");
    return IGXRT_OK;
}

igxrt_status launch_trace_words(igxrt_context* ctx, const TraceRequest& req,
                                const igxrt_launch_params& p, cudaStream_t stream,
                                uint32_t* queue, uint32_t* status) {
    if (req.count == 0)
        return IGXRT_OK;
    const igxrt_scene* s = req.scene;
    KernelFn fn = select_kernel(p.layout, req.mode == 1, req.node_fetches != nullptr, s->mixed);
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
    const uint64_t warps_needed = ((uint64_t)req.count + p.packet_size - 1) / p.packet_size;
    const uint64_t ctas_needed = (warps_needed + p.block_size / 32 - 1) / (p.block_size / 32);
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, ctas_needed));
    KernelArgs a;
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
    a.queue = queue;
    a.status = status;
    a.exit_count = nullptr;  // the caller resets its words
    a.independent = 0u;
    a.packet = p.packet_size;
    a.sh_depth = p.stack_depth;
    a.refill_lanes = p.refill_lanes;
    a.planes = reinterpret_cast<const float4*>(s->planes);
    a.plane_count = s->plane_count;
    a.plane_base = s->plane_base;
    fn<<<grid, p.block_size, smem, stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "trace kernel launch");
    return IGXRT_OK;
}

}  // namespace igxrt
