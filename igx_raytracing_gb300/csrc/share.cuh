// share.cuh — work sharing among a warp's lanes once the work queue is drained.
#pragma once

#include "traverse.cuh"

namespace igxrt {

// ---- work sharing once the queue is drained --------------------------------
//
// After a warp finds the queue empty its lanes finish the rays they hold, and
// the warp runs until its slowest ray is done while finished lanes idle.
// From then on idle lanes take the bottom entries (the oldest, largest
// pending subtrees) of busy lanes' stacks and traverse them for the same
// rays, as helpers of the lanes that own the rays.  A helper keeps its own best hit
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

// Query modes of share_tail: every lane the same (closest or any hit), or
// either per lane (the batch kernel: the merge then handles both).
constexpr int kShareClosest = 0, kShareAny = 1, kSharePerLane = 2;

// No per-lane state beyond the ray (the plain trace kernels).
struct NoLaneExtra {
    __device__ __forceinline__ void take(uint32_t) {}
};

// One round of tail work sharing, run by the whole warp between traversal
// phases.  `extra` holds lane state a helper must copy from its victim
// (take(src) reads it from lane src; lanes that take nothing read their
// own); `finish(occluded)` writes the lane's ray; `no_hit` is the value of
// BestHit.prim before a first hit (0, or the priority code of mixed
// scenes, whose merges then compare (t, priority) like their leaves do).
template <int MODE, class Extra, class Finish>
__device__ __forceinline__ void share_tail(uint32_t lane, uint32_t lower, uint32_t& link, bool& alive,
                                           uint32_t& ray, RayState& r, BestHit& best, TraversalStack& st,
                                           int32_t& next, Extra& extra, Finish finish, uint32_t no_hit = 0u) {
    constexpr bool CLOSEST = MODE != kShareAny;  // per-lane mode merges both ways
    constexpr uint32_t FULL = 0xffffffffu;
    // 1. finished helpers hand their best hit (or occluder) to the owner
    uint32_t m = __ballot_sync(FULL, alive && (link & kLinkMerge));
    while (m) {
        const int h = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t hl = __shfl_sync(FULL, link, h);
        const uint32_t o = hl & 31u;
        if (MODE != kShareClosest && lane == o)
            link |= hl & kLinkOcc;
        if (CLOSEST) {
            // (t, prim) decide; u and v follow one at a time (few live
            // registers); an any-hit ray's best hit never moves, so the merge
            // leaves it as it is
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
    if (MODE != kShareClosest) {
        const uint32_t ol = __shfl_sync(FULL, link, link & 31u);
        if (alive && (link & 31u) != lane && (ol & kLinkOcc)) {
            alive = false;
            link = lane;
        }
    }
    // 3. an owner whose ray is decided and has no helper left writes it
    const uint32_t grp = __match_any_sync(FULL, alive ? (link & 31u) : 32u + lane);
    if (alive && (link & 31u) == lane && (link & (kLinkWait | kLinkOcc)) && grp == (1u << lane)) {
        finish((link & kLinkOcc) != 0);
        alive = false;
        link = lane;
    }
    // helpers prune with their owner's cull limit when it is tighter
    if (CLOSEST) {
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
    extra.take(src);
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
        best.prim = no_hit;
        best.tcull = vtc;
        next = (int32_t)e.x;
        st.sp = 0;
        alive = true;
    }
}

}  // namespace igxrt
