// traverse.cuh — device-side ray/box and ray/triangle tests and the BVH
// traversal loops shared by the plain, batched and instrumented kernels.
//
// Arithmetic contract (identical to the host oracle in oracle/trace_oracle.c):
//   * the triangle test is rayIntersectTri (res/shaders/primitive.glsl:239-284)
//     in binary32 with every multiply and add rounded separately
//     (__fmul_rn / __fadd_rn / __fsub_rn never fuse), dot products summed left
//     to right, cross products in GLSL component order, f = 1/a correctly
//     rounded (__frcp_rn), denormals kept (the library is built without
//     -ftz);
//   * the slab test uses explicit fmaf on both sides so the host and the GPU
//     cull the same boxes and visit nodes in the same order;
//   * a hit (t, prim) replaces the best one when t < best.t, or t == best.t
//     and prim < best.prim: the linear loop's "first index reaching the
//     smallest t" (trace.glsl:25-27 with the strict t >= hit.hitT rejection at
//     primitive.glsl:276), independent of visiting order.
#pragma once

#include <cstdint>

#include "igxrt.h"
#include "internal.h"

namespace igxrt {

constexpr uint32_t kStatusStackOverflow = 1u;
// Traversal stack entries per ray (shared part + local spill).
constexpr uint32_t kStackCapacityDevice = 128;

struct RayState {
    float ox, oy, oz;
    float dx, dy, dz;
    float ix, iy, iz;     // 1/d with |d| < 2^-80 raised to 2^-80
    float oix, oiy, oiz;  // o * (1/d)
    float tmin, tmin_box, tmax_eff;
    uint32_t prev;
};

struct BestHit {
    float t, u, v;
    uint32_t prim;
    float tcull;
};

__device__ __forceinline__ float safe_dir(float d) {
    return fabsf(d) < 0x1p-80f ? copysignf(0x1p-80f, d) : d;
}

// Upper bound used to cull boxes: best t widened upward by 2^-10 of its
// magnitude (t can be negative with a negative tmin or an enclosing cube),
// kept finite so the {+inf} box of an absent child is never entered.
__device__ __forceinline__ float cull_limit(float t) {
    return fminf(__fmaf_rn(fabsf(t), 0x1p-10f, t), 3.4028235e38f);
}

__device__ __forceinline__ RayState load_ray(const igxrt_ray* __restrict__ rays, uint32_t i,
                                             uint32_t prev) {
    const float4* p = reinterpret_cast<const float4*>(rays) + 2 * (size_t)i;
    const float4 a = __ldg(p), b = __ldg(p + 1);
    RayState r;
    r.ox = a.x;
    r.oy = a.y;
    r.oz = a.z;
    r.dx = b.x;
    r.dy = b.y;
    r.dz = b.z;
    r.ix = __frcp_rn(safe_dir(b.x));
    r.iy = __frcp_rn(safe_dir(b.y));
    r.iz = __frcp_rn(safe_dir(b.z));
    r.oix = __fmul_rn(a.x, r.ix);
    r.oiy = __fmul_rn(a.y, r.iy);
    r.oiz = __fmul_rn(a.z, r.iz);
    r.tmin = a.w;
    r.tmin_box = (a.w > -INFINITY) ? __fmaf_rn(-fabsf(a.w), 0x1p-10f, a.w) : -INFINITY;
    r.tmax_eff = b.w < IGXRT_NO_HIT ? b.w : IGXRT_NO_HIT;
    r.prev = prev;
    return r;
}

__device__ __forceinline__ bool box_hit(const RayState& r, float lox, float hix, float loy,
                                        float hiy, float loz, float hiz, float tcull, float& tn) {
    const float t0x = __fmaf_rn(lox, r.ix, -r.oix), t1x = __fmaf_rn(hix, r.ix, -r.oix);
    const float t0y = __fmaf_rn(loy, r.iy, -r.oiy), t1y = __fmaf_rn(hiy, r.iy, -r.oiy);
    const float t0z = __fmaf_rn(loz, r.iz, -r.oiz), t1z = __fmaf_rn(hiz, r.iz, -r.oiz);
    const float tnear =
        fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), r.tmin_box));
    const float tfar = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tcull));
    tn = tnear;
    return tnear <= tfar;
}

// Slab test of mixed scenes: the entry distance is not clamped to tmin, so a
// box around the origin keeps its negative entry distance (a cube around the
// origin is hit there, and a negative best t must not cull it); boxes wholly
// behind tmin are still culled.
__device__ __forceinline__ bool box_hit_mixed(const RayState& r, float lox, float hix, float loy,
                                              float hiy, float loz, float hiz, float tcull, float& tn) {
    const float t0x = __fmaf_rn(lox, r.ix, -r.oix), t1x = __fmaf_rn(hix, r.ix, -r.oix);
    const float t0y = __fmaf_rn(loy, r.iy, -r.oiy), t1y = __fmaf_rn(hiy, r.iy, -r.oiy);
    const float t0z = __fmaf_rn(loz, r.iz, -r.oiz), t1z = __fmaf_rn(hiz, r.iz, -r.oiz);
    const float tnear = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    const float tslab = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    tn = tnear;
    return tslab >= r.tmin_box && tnear <= fminf(tslab, tcull);
}

// rayIntersectTri's arithmetic on a primitive record {p0,prim}{e1,end}{e2,pad}.
// Returns false when the u/v tests reject; otherwise t, u, v are the
// reference's values (t may still be rejected by the caller).
__device__ __forceinline__ bool tri_test(const RayState& r, const float4& v0, const float4& v1,
                                         const float4& v2, float& t, float& u, float& v) {
    // h = cross(dir, e2)
    const float hx = __fsub_rn(__fmul_rn(r.dy, v2.z), __fmul_rn(v2.y, r.dz));
    const float hy = __fsub_rn(__fmul_rn(r.dz, v2.x), __fmul_rn(v2.z, r.dx));
    const float hz = __fsub_rn(__fmul_rn(r.dx, v2.y), __fmul_rn(v2.x, r.dy));
    // a = dot(e1, h); s = pos - p0; dsh = dot(s, h)
    const float a = __fadd_rn(__fadd_rn(__fmul_rn(v1.x, hx), __fmul_rn(v1.y, hy)), __fmul_rn(v1.z, hz));
    const float sx = __fsub_rn(r.ox, v0.x), sy = __fsub_rn(r.oy, v0.y), sz = __fsub_rn(r.oz, v0.z);
    const float dsh = __fadd_rn(__fadd_rn(__fmul_rn(sx, hx), __fmul_rn(sy, hy)), __fmul_rn(sz, hz));
    // u = f * dsh with f = 1/a rounded has the sign of a * dsh; it is < 0
    // (rejected below) whenever the signs differ, dsh != 0, a is finite and
    // |dsh| >= 2^-100 |a|, since then |u| >= 2^-100 (1 - 2^-24) cannot round
    // to zero (for a = 0, f is infinite and u = -inf).  Deciding that case
    // before the correctly rounded reciprocal changes no result.
    if (((__float_as_uint(a) ^ __float_as_uint(dsh)) & 0x80000000u) && dsh != 0.f &&
        fabsf(a) <= 3.4028235e38f && __fmul_rn(fabsf(dsh), 0x1p100f) >= fabsf(a))
        return false;
    // f = 1 / a; u = f * dot(s, h)
    const float f = __frcp_rn(a);
    u = __fmul_rn(f, dsh);
    if (u < 0.f || u > 1.f)
        return false;
    // q = cross(s, e1); v = f * dot(dir, q)
    const float qx = __fsub_rn(__fmul_rn(sy, v1.z), __fmul_rn(v1.y, sz));
    const float qy = __fsub_rn(__fmul_rn(sz, v1.x), __fmul_rn(v1.z, sx));
    const float qz = __fsub_rn(__fmul_rn(sx, v1.y), __fmul_rn(v1.x, sy));
    v = __fmul_rn(f, __fadd_rn(__fadd_rn(__fmul_rn(r.dx, qx), __fmul_rn(r.dy, qy)), __fmul_rn(r.dz, qz)));
    if (v < 0.f || __fadd_rn(u, v) > 1.f)
        return false;
    // t = f * dot(e2, q)
    t = __fmul_rn(f, __fadd_rn(__fadd_rn(__fmul_rn(v2.x, qx), __fmul_rn(v2.y, qy)), __fmul_rn(v2.z, qz)));
    return true;
}

constexpr int32_t kRefDone = 0x7fffffff;  // "stack empty": the traversal is over

// Traversal stack of {child reference, entry distance of its box when it was
// pushed}: the first `sh_depth` entries live in shared memory (strided by
// the block size so a warp's accesses stay conflict-free), the rest in a
// per-thread local array.  pop_live drops entries whose distance is beyond
// the current cull limit without fetching them (their box test would fail
// now), exactly as the host traversal does.
struct TraversalStack {
    uint2* sh;  // this thread's column of the block's shared stack
    uint32_t stride;
    uint32_t sh_depth;
    uint32_t sp;
    uint2 spill[kStackCapacityDevice];

    __device__ __forceinline__ void push(int32_t ref, float tnear) {
        const uint2 e = make_uint2((uint32_t)ref, __float_as_uint(tnear));
        if (sp < sh_depth)
            sh[sp * stride] = e;
        else
            spill[sp - sh_depth] = e;
        ++sp;
    }
    __device__ __forceinline__ uint2 at(uint32_t k) const { return k < sh_depth ? sh[k * stride] : spill[k - sh_depth]; }
    __device__ __forceinline__ void set(uint32_t k, uint2 e) {
        if (k < sh_depth)
            sh[k * stride] = e;
        else
            spill[k - sh_depth] = e;
    }
    // Removes the g bottom entries; the rest move down g places.
    __device__ void drop_bottom(uint32_t g) {
        for (uint32_t k = g; k < sp; ++k)
            set(k - g, at(k));
        sp -= g;
    }
    __device__ __forceinline__ int32_t pop_live(float tcull) {
        while (sp) {
            --sp;
            const uint2 e = sp < sh_depth ? sh[sp * stride] : spill[sp - sh_depth];
            if (__uint_as_float(e.y) <= tcull)
                return (int32_t)e.x;
        }
        return kRefDone;
    }
};

// Bytes of shared memory per stack entry and thread.
constexpr uint32_t kStackEntryBytes = 8;

// Closest-hit / any-hit leaf processing.  Returns true when an any-hit query
// is decided (occluder found).
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool process_leaf(const float4* __restrict__ prims, int32_t ref,
                                             const RayState& r, BestHit& best, uint32_t& pf) {
    uint32_t i = (uint32_t)~ref;
    for (;;) {
        const float4* p = prims + 3 * (size_t)i;
        const float4 v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2);
        if (COUNT)
            ++pf;
        float t, u, v;
        if (tri_test(r, v0, v1, v2, t, u, v)) {
            const uint32_t prim = __float_as_uint(v0.w);
            if (!(t <= r.tmin) && prim != r.prev) {
                if (ANY) {
                    if (t < r.tmax_eff)
                        return true;
                } else if (t < best.t || (t == best.t && prim < best.prim)) {
                    best.t = t;
                    best.u = u;
                    best.v = v;
                    best.prim = prim;
                    best.tcull = cull_limit(t);
                }
            }
        }
        if (__float_as_uint(v1.w))
            break;
        ++i;
    }
    return false;
}

template <int LAYOUT, bool COUNT, bool MIXED>
__device__ __forceinline__ int32_t visit_node(const float4* __restrict__ nodes, int32_t node,
                                              const RayState& r, const BestHit& best,
                                              TraversalStack& st, bool& overflow, uint32_t& nf);

// The node phase of the persistent kernels, called by all 32 lanes of the
// warp together (every ballot names the whole warp); the lanes with
// `working` set (their set is `wmask`) each descend through interior nodes
// until they hold a leaf or their traversal is over, the others only take
// part in the ballots.  A working lane that got there first waits for the
// others (the leaf phase that follows tests the lanes' leaves together), and
// most waiting happens behind a few lanes with long descents; so once
// `phase_break` times the lanes still descending is at most the number of
// working lanes waiting (at a leaf, or done), the phase ends and the
// descending lanes resume in the warp's next round, after the leaves.  The
// order in which each ray visits its nodes and records is the same for every
// phase_break; phase_break 32 never ends the phase early.
template <int LAYOUT, bool COUNT, bool MIXED>
__device__ __forceinline__ void node_phase(const float4* __restrict__ nodes, bool working, uint32_t wmask,
                                           uint32_t phase_break, int32_t& next, const RayState& r,
                                           const BestHit& best, TraversalStack& st, bool& overflow,
                                           uint32_t& nf) {
    for (;;) {
        const bool down = working && next >= 0 && next != kRefDone;
        const uint32_t dm = __ballot_sync(0xffffffffu, down);
        if (dm == 0)
            break;
        if ((uint32_t)__popc(dm) * phase_break <= (uint32_t)__popc(wmask & ~dm))
            break;
        if (down)
            next = visit_node<LAYOUT, COUNT, MIXED>(nodes, next, r, best, st, overflow, nf);
    }
}

// 256-bit read-only load (sm_100+): eight floats from a 32-byte aligned address.
__device__ __forceinline__ void ldg256(const void* p, float4& lo, float4& hi) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w)
        : "l"(p));
}

struct SlotKey {
    float tn;
    int32_t child;
    uint32_t slot;
};

__device__ __forceinline__ void order2(SlotKey& a, SlotKey& b) {
    const bool swap = b.tn < a.tn || (b.tn == a.tn && b.slot < a.slot);
    if (swap) {
        const SlotKey t = a;
        a = b;
        b = t;
    }
}

template <bool MIXED>
__device__ __forceinline__ bool box_test(const RayState& r, float lox, float hix, float loy,
                                         float hiy, float loz, float hiz, float tcull, float& tn) {
    return MIXED ? box_hit_mixed(r, lox, hix, loy, hiy, loz, hiz, tcull, tn)
                 : box_hit(r, lox, hix, loy, hiy, loz, hiz, tcull, tn);
}

// BVH8 slot order: the entry distance as an order-preserving word whose low
// 3 bits are replaced by the slot, so keys are distinct and sort by
// (distance, slot).  A pushed entry keeps the distance of the key with those
// bits cleared, never larger than the box's own (the host traversal does the
// same).
__device__ __forceinline__ uint32_t slot_key(float t, uint32_t slot) {
    const uint32_t u = __float_as_uint(t);
    return (((u & 0x80000000u) ? ~u : (u | 0x80000000u)) & ~7u) | slot;
}

__device__ __forceinline__ float key_distance(uint32_t k) {
    k &= ~7u;
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ void sort2(uint32_t& a, uint32_t& b) {
    const uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

// Byte `i` of a little-endian word pair as an exact float: the byte placed
// in the mantissa of 2^23 (one byte permute), minus 2^23.
__device__ __forceinline__ float byte_float(float w0, float w1, int i) {
    const uint32_t w = __float_as_uint(i < 4 ? w0 : w1);
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)(i & 3))),
                     8388608.0f);
}

// A ray-space step that is a finite normal float (its product with a byte
// and the sum with the offset then round like the world-space test).
__device__ __forceinline__ bool ray_space_ok(float m) {
    const float a = fabsf(m);
    return a >= 1.17549435e-38f && a <= 3.4028235e38f;
}

// box_hit / box_hit_mixed with each axis' entry and exit distances given
// (near and far planes already told apart by the direction's sign).
template <bool MIXED>
__device__ __forceinline__ bool slab_test(const RayState& r, float tnx, float tfx, float tny, float tfy,
                                          float tnz, float tfz, float tcull, float& tn) {
    if (MIXED) {
        const float tnear = fmaxf(fmaxf(tnx, tny), tnz);
        const float tslab = fminf(fminf(tfx, tfy), tfz);
        tn = tnear;
        return tslab >= r.tmin_box && tnear <= fminf(tslab, tcull);
    }
    const float tnear = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin_box));
    const float tfar = fminf(fminf(tfx, tfy), fminf(tfz, tcull));
    tn = tnear;
    return tnear <= tfar;
}

__device__ __forceinline__ int32_t pick8(const float4& c0, const float4& c1, uint32_t slot) {
    const float4& c = (slot & 4u) ? c1 : c0;
    const float v = (slot & 2u) ? ((slot & 1u) ? c.w : c.z) : ((slot & 1u) ? c.y : c.x);
    return __float_as_int(v);
}

// One interior-node visit in the kernels' order: test the children, descend
// into the nearer hit child and push the other.  Returns the next reference
// (a node, a leaf, or kRefDone), or sets `overflow`.
template <int LAYOUT, bool COUNT, bool MIXED = false>
__device__ __forceinline__ int32_t visit_node(const float4* __restrict__ nodes, int32_t node,
                                              const RayState& r, const BestHit& best,
                                              TraversalStack& st, bool& overflow, uint32_t& nf) {
    if (COUNT)
        ++nf;
    if (LAYOUT == IGXRT_LAYOUT_BVH8) {
        // 96-byte node: {origin, exp bytes + valid}{lo_x, hi_x} {lo_y, hi_y, lo_z, hi_z} {child[8]}
        const float4* n = nodes + 6 * (size_t)node;
        float4 hdr, qx, qy, qz, c0, c1;
        ldg256(n, hdr, qx);
        ldg256(n + 2, qy, qz);
        ldg256(n + 4, c0, c1);
        const uint32_t meta = __float_as_uint(hdr.w);
        // 2^exp as a float (exp in [-126, 127], checked by the validator)
        const float sx = __int_as_float(((int)(int8_t)(meta & 0xffu) + 127) << 23);
        const float sy = __int_as_float(((int)(int8_t)((meta >> 8) & 0xffu) + 127) << 23);
        const float sz = __int_as_float(((int)(int8_t)((meta >> 16) & 0xffu) + 127) << 23);
        const uint32_t valid = meta >> 24;
        uint32_t k[8];
        uint32_t m = 0;
        // Ray space: a plane q steps from the origin lies at
        // t = fmaf(q, 2^exp * (1/d), fmaf(origin, 1/d, -o/d)), one product
        // scaled by a power of two (exact while it stays a normal float) and
        // two roundings, like box_hit's fmaf(plane, 1/d, -o/d).  With a
        // positive step the lo byte is the near plane, else the hi byte.
        const float mx = __fmul_rn(sx, r.ix), my = __fmul_rn(sy, r.iy), mz = __fmul_rn(sz, r.iz);
        const float bx = __fmaf_rn(hdr.x, r.ix, -r.oix), by = __fmaf_rn(hdr.y, r.iy, -r.oiy),
                    bz = __fmaf_rn(hdr.z, r.iz, -r.oiz);
        const bool fast = ray_space_ok(mx) && ray_space_ok(my) && ray_space_ok(mz) &&
                          fabsf(bx) <= 3.4028235e38f && fabsf(by) <= 3.4028235e38f &&
                          fabsf(bz) <= 3.4028235e38f;
        if (fast) {
            const bool px = mx > 0.f, py = my > 0.f, pz = mz > 0.f;
            const float nx0 = px ? qx.x : qx.z, nx1 = px ? qx.y : qx.w, fx0 = px ? qx.z : qx.x,
                        fx1 = px ? qx.w : qx.y;
            const float ny0 = py ? qy.x : qy.z, ny1 = py ? qy.y : qy.w, fy0 = py ? qy.z : qy.x,
                        fy1 = py ? qy.w : qy.y;
            const float nz0 = pz ? qz.x : qz.z, nz1 = pz ? qz.y : qz.w, fz0 = pz ? qz.z : qz.x,
                        fz1 = pz ? qz.w : qz.y;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const float tnx = __fmaf_rn(byte_float(nx0, nx1, c), mx, bx);
                const float tfx = __fmaf_rn(byte_float(fx0, fx1, c), mx, bx);
                const float tny = __fmaf_rn(byte_float(ny0, ny1, c), my, by);
                const float tfy = __fmaf_rn(byte_float(fy0, fy1, c), my, by);
                const float tnz = __fmaf_rn(byte_float(nz0, nz1, c), mz, bz);
                const float tfz = __fmaf_rn(byte_float(fz0, fz1, c), mz, bz);
                float tn;
                const bool h = slab_test<MIXED>(r, tnx, tfx, tny, tfy, tnz, tfz, best.tcull, tn) &&
                               ((valid >> c) & 1u);
                k[c] = h ? slot_key(tn, (uint32_t)c) : 0xffffffffu;
                m += h ? 1u : 0u;
            }
        } else {
            // a step out of the normal range: decode the planes in world space
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const float lox = __fmaf_rn(byte_float(qx.x, qx.y, c), sx, hdr.x);
                const float hix = __fmaf_rn(byte_float(qx.z, qx.w, c), sx, hdr.x);
                const float loy = __fmaf_rn(byte_float(qy.x, qy.y, c), sy, hdr.y);
                const float hiy = __fmaf_rn(byte_float(qy.z, qy.w, c), sy, hdr.y);
                const float loz = __fmaf_rn(byte_float(qz.x, qz.y, c), sz, hdr.z);
                const float hiz = __fmaf_rn(byte_float(qz.z, qz.w, c), sz, hdr.z);
                float tn;
                const bool h = box_test<MIXED>(r, lox, hix, loy, hiy, loz, hiz, best.tcull, tn) &&
                               ((valid >> c) & 1u);
                k[c] = h ? slot_key(tn, (uint32_t)c) : 0xffffffffu;
                m += h ? 1u : 0u;
            }
        }
        if (m == 0)
            return st.pop_live(best.tcull);
        // ascending keys: the optimal 19-comparator network for 8 inputs
        sort2(k[0], k[2]); sort2(k[1], k[3]); sort2(k[4], k[6]); sort2(k[5], k[7]);
        sort2(k[0], k[4]); sort2(k[1], k[5]); sort2(k[2], k[6]); sort2(k[3], k[7]);
        sort2(k[0], k[1]); sort2(k[2], k[3]); sort2(k[4], k[5]); sort2(k[6], k[7]);
        sort2(k[2], k[4]); sort2(k[3], k[5]);
        sort2(k[1], k[4]); sort2(k[3], k[6]);
        sort2(k[1], k[2]); sort2(k[3], k[4]); sort2(k[5], k[6]);
        if (st.sp + m - 1 > kStackCapacityDevice) {
            overflow = true;
            return kRefDone;
        }
#pragma unroll
        for (int j = 7; j >= 1; --j)
            if ((uint32_t)j < m)
                st.push(pick8(c0, c1, k[j] & 7u), key_distance(k[j]));
        return pick8(c0, c1, k[0] & 7u);
    } else if (LAYOUT == IGXRT_LAYOUT_BVH4) {
        const float4* n = nodes + 8 * (size_t)node;
        float4 lx, hx, ly, hy, lz, hz, c, unused;
        ldg256(n, lx, hx);
        ldg256(n + 2, ly, hy);
        ldg256(n + 4, lz, hz);
        ldg256(n + 6, c, unused);
        const int4 ch = make_int4(__float_as_int(c.x), __float_as_int(c.y), __float_as_int(c.z),
                                  __float_as_int(c.w));
        float tn;
        uint32_t h, m = 0;
        h = box_test<MIXED>(r,lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, best.tcull, tn);
        m += h;
        SlotKey k0 = {h ? tn : INFINITY, ch.x, 0u};
        h = box_test<MIXED>(r,lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, best.tcull, tn);
        m += h;
        SlotKey k1 = {h ? tn : INFINITY, ch.y, 1u};
        h = box_test<MIXED>(r,lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, best.tcull, tn);
        m += h;
        SlotKey k2 = {h ? tn : INFINITY, ch.z, 2u};
        h = box_test<MIXED>(r,lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, best.tcull, tn);
        m += h;
        SlotKey k3 = {h ? tn : INFINITY, ch.w, 3u};
        if (m == 0)
            return st.pop_live(best.tcull);
        // (tnear, slot) ascending; missed slots carry +inf and sort last (a
        // hit's tnear is at most the finite cull limit)
        order2(k0, k1);
        order2(k2, k3);
        order2(k0, k2);
        order2(k1, k3);
        order2(k1, k2);
        if (st.sp + m - 1 > kStackCapacityDevice) {
            overflow = true;
            return kRefDone;
        }
        if (m > 3)
            st.push(k3.child, k3.tn);
        if (m > 2)
            st.push(k2.child, k2.tn);
        if (m > 1)
            st.push(k1.child, k1.tn);
        return k0.child;
    } else {
        const float4* n = nodes + 4 * (size_t)node;
        float4 xy0, xy1, z01, c;
        ldg256(n, xy0, xy1);
        ldg256(n + 2, z01, c);
        const int32_t c0 = __float_as_int(c.x), c1 = __float_as_int(c.y);
        float tn0, tn1;
        const bool h0 = box_test<MIXED>(r,xy0.x, xy0.y, xy0.z, xy0.w, z01.x, z01.y, best.tcull, tn0);
        const bool h1 = box_test<MIXED>(r,xy1.x, xy1.y, xy1.z, xy1.w, z01.z, z01.w, best.tcull, tn1);
        if (h0 && h1) {
            const bool first1 = tn1 < tn0;
            if (st.sp >= kStackCapacityDevice) {
                overflow = true;
                return kRefDone;
            }
            st.push(first1 ? c0 : c1, first1 ? tn0 : tn1);
            return first1 ? c1 : c0;
        }
        if (h0)
            return c0;
        if (h1)
            return c1;
        return st.pop_live(best.tcull);
    }
}

// ---- mixed scenes: spheres, cubes, planes ---------------------------------
//
// In mixed scenes BestHit.prim holds a priority instead of the object id:
// at equal t a lower priority wins.  Cubes accept ties (the cube test rejects
// only tmin > hit.hitT, primitive.glsl:302) so among the linear loop's
// candidates at the smallest t the last cube wins, and without a cube the
// first other object wins: cube id i -> 0x7fffffff - i, other id i ->
// 0x80000000 + i, and the "no hit yet" state is 0x80000000 (a non-cube needs
// t < tmax, a cube t <= tmax).
constexpr uint32_t kPrioNone = 0x80000000u;
__device__ __forceinline__ uint32_t prio_other(uint32_t id) { return 0x80000000u + id; }
__device__ __forceinline__ uint32_t prio_cube(uint32_t id) { return 0x7fffffffu - id; }
__device__ __forceinline__ uint32_t id_of_prio(uint32_t p) {
    return p >= 0x80000000u ? p - 0x80000000u : 0x7fffffffu - p;
}
__device__ __forceinline__ bool better(float t, uint32_t p, const BestHit& b) {
    return t < b.t || (t == b.t && p < b.prim);
}

// GLSL min / max as the specification defines them (NaN handling included).
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// rayIntersectSphere (primitive.glsl:173-210): hitT and the in-sphere test.
__device__ __forceinline__ bool sphere_hit(const RayState& r, float cx, float cy, float cz, float rad,
                                           float& hitT) {
    const float dx = __fsub_rn(cx, r.ox), dy = __fsub_rn(cy, r.oy), dz = __fsub_rn(cz, r.oz);
    const float t = dot3f(dx, dy, dz, r.dx, r.dy, r.dz);
    const float qx = __fsub_rn(dx, __fmul_rn(t, r.dx)), qy = __fsub_rn(dy, __fmul_rn(t, r.dy)),
                qz = __fsub_rn(dz, __fmul_rn(t, r.dz));
    const float Q2 = dot3f(qx, qy, qz, qx, qy, qz);
    const float R2 = __fmul_rn(rad, rad);
    hitT = __fsub_rn(t, __fsqrt_rn(__fsub_rn(R2, Q2)));
    return !(Q2 > R2);
}

// The sphere's uv (primitive.glsl:189-204).  asin and atan give the
// correctly rounded binary32 value: evaluated in binary64 (CUDA's asin /
// atan, a few binary64 ulp) and rounded once, which lands on the correctly
// rounded float unless the binary64 value falls within its error of a
// binary32 rounding midpoint.  The oracle evaluates them the same way, so u
// and v, which cancel towards 0 near the poles and the seam (lat * 1/pi +
// 0.5), come out bit for bit instead of many float ulp apart.
__device__ __forceinline__ void sphere_uv(const RayState& r, float cx, float cy, float cz, float hitT,
                                          float& u, float& v) {
    const float ox = __fadd_rn(__fmul_rn(hitT, r.dx), r.ox), oy = __fadd_rn(__fmul_rn(hitT, r.dy), r.oy),
                oz = __fadd_rn(__fmul_rn(hitT, r.dz), r.oz);
    const float nx = __fsub_rn(cx, ox), ny = __fsub_rn(cy, oy), nz = __fsub_rn(cz, oz);
    const float len = __fsqrt_rn(dot3f(nx, ny, nz, nx, ny, nz));
    const float ux = __fdiv_rn(nx, len), uy = __fdiv_rn(ny, len), uz = __fdiv_rn(nz, len);
    const float lat = __double2float_rn(asin((double)uz));
    float lon = __double2float_rn(atan((double)__fdiv_rn(uy, ux)));
    if (lon != lon)
        lon = 0.f;
    const float k = (float)(0.636619746685 * 0.5);
    u = __fadd_rn(__fmul_rn(lat, k), 0.5f);
    v = __fadd_rn(__fmul_rn(lon, k), 0.5f);
}

// rayIntersectCube (primitive.glsl:286-333) with the ray's raw 1/dir.
// Returns whether [tmin, tmax] is a valid interval reaching tmin_ray.
__device__ __forceinline__ bool cube_hit(const RayState& r, const float4& s, const float4& e, float& tmin,
                                         float& u, float& v) {
    const float rx = __frcp_rn(r.dx), ry = __frcp_rn(r.dy), rz = __frcp_rn(r.dz);
    const float sx = __fmul_rn(__fsub_rn(s.x, r.ox), rx), sy = __fmul_rn(__fsub_rn(s.y, r.oy), ry),
                sz = __fmul_rn(__fsub_rn(s.z, r.oz), rz);
    const float ex = __fmul_rn(__fsub_rn(e.x, r.ox), rx), ey = __fmul_rn(__fsub_rn(e.y, r.oy), ry),
                ez = __fmul_rn(__fsub_rn(e.z, r.oz), rz);
    const float mix = gmin(sx, ex), miy = gmin(sy, ey), miz = gmin(sz, ez);
    const float max_ = gmax(sx, ex), may = gmax(sy, ey), maz = gmax(sz, ez);
    tmin = gmax(gmax(mix, miy), miz);
    const float tmax = gmin(gmin(max_, may), maz);
    if (tmax < r.tmin || tmin > tmax)
        return false;
    // pos = (dir * tmin + pos) - start; pos /= end
    const float px = __fdiv_rn(__fsub_rn(__fadd_rn(__fmul_rn(r.dx, tmin), r.ox), s.x), e.x);
    const float py = __fdiv_rn(__fsub_rn(__fadd_rn(__fmul_rn(r.dy, tmin), r.oy), s.y), e.y);
    const float pz = __fdiv_rn(__fsub_rn(__fadd_rn(__fmul_rn(r.dz, tmin), r.oz), s.z), e.z);
    if (tmin == mix) {
        u = py;
        v = pz;
    } else if (tmin == miy) {
        u = px;
        v = pz;
    } else {
        u = px;
        v = py;
    }
    return true;
}

// rayIntersectPlane (primitive.glsl:212-237): hitT, and the uv on request.
__device__ __forceinline__ float plane_hit(const RayState& r, const float4& pl) {
    const float len = __fsqrt_rn(dot3f(pl.x, pl.y, pl.z, pl.x, pl.y, pl.z));
    const float nx = -__fdiv_rn(pl.x, len), ny = -__fdiv_rn(pl.y, len), nz = -__fdiv_rn(pl.z, len);
    const float dif = dot3f(r.dx, r.dy, r.dz, nx, ny, nz);
    return __fdiv_rn(-__fadd_rn(dot3f(r.ox, r.oy, r.oz, nx, ny, nz), pl.w), dif);
}

__device__ __forceinline__ void plane_uv(const RayState& r, const float4& pl, float hitT, float& u,
                                         float& v) {
    const float ox = __fadd_rn(__fmul_rn(hitT, r.dx), r.ox), oy = __fadd_rn(__fmul_rn(hitT, r.dy), r.oy),
                oz = __fadd_rn(__fmul_rn(hitT, r.dz), r.oz);
    // planeX = cross(n, (0,0,1)), planeZ = cross(n, (1,0,0)) in GLSL component order
    const float xx = __fsub_rn(__fmul_rn(pl.y, 1.0f), __fmul_rn(0.0f, pl.z));
    const float xy = __fsub_rn(__fmul_rn(pl.z, 0.0f), __fmul_rn(1.0f, pl.x));
    const float xz = __fsub_rn(__fmul_rn(pl.x, 0.0f), __fmul_rn(0.0f, pl.y));
    const float zx = __fsub_rn(__fmul_rn(pl.y, 0.0f), __fmul_rn(0.0f, pl.z));
    const float zy = __fsub_rn(__fmul_rn(pl.z, 1.0f), __fmul_rn(0.0f, pl.x));
    const float zz = __fsub_rn(__fmul_rn(pl.x, 0.0f), __fmul_rn(1.0f, pl.y));
    u = dot3f(ox, oy, oz, xx, xy, xz);
    v = dot3f(ox, oy, oz, zx, zy, zz);
}

// Leaf of a mixed scene.  Returns true when an any-hit query is decided.
// best_rec (optional): the record index of the best hit so far, for callers
// that need the hit object's record afterwards (the G-buffer's normals).
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ bool process_leaf_mixed(const float4* __restrict__ prims, int32_t ref,
                                                   const RayState& r, BestHit& best, uint32_t* pf = nullptr,
                                                   uint32_t* best_rec = nullptr) {
    uint32_t i = (uint32_t)~ref;
    for (;;) {
        const float4* p = prims + 3 * (size_t)i;
        const float4 v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2);
        if (COUNT)
            ++*pf;
        const uint32_t type = __float_as_uint(v2.w), id = __float_as_uint(v0.w);
        if (id != r.prev) {
            if (type == kPrimTriangle) {
                float t, u, v;
                if (tri_test(r, v0, v1, v2, t, u, v) && !(t <= r.tmin)) {
                    if (ANY) {
                        if (t < r.tmax_eff)
                            return true;
                    } else if (better(t, prio_other(id), best)) {
                        best.t = t;
                        best.u = u;
                        best.v = v;
                        best.prim = prio_other(id);
                        best.tcull = cull_limit(t);
                        if (best_rec)
                            *best_rec = i;
                    }
                }
            } else if (type == kPrimSphere) {
                float t;
                if (sphere_hit(r, v0.x, v0.y, v0.z, v1.x, t) && t >= r.tmin) {
                    if (ANY) {
                        if (t < r.tmax_eff)
                            return true;
                    } else if (better(t, prio_other(id), best)) {
                        sphere_uv(r, v0.x, v0.y, v0.z, t, best.u, best.v);
                        best.t = t;
                        best.prim = prio_other(id);
                        best.tcull = cull_limit(t);
                        if (best_rec)
                            *best_rec = i;
                    }
                }
            } else {
                float t, u, v;
                if (cube_hit(r, v0, v1, t, u, v)) {
                    if (ANY) {
                        if (t < r.tmax_eff)
                            return true;
                    } else if (better(t, prio_cube(id), best)) {
                        best.t = t;
                        best.u = u;
                        best.v = v;
                        best.prim = prio_cube(id);
                        best.tcull = cull_limit(t);
                        if (best_rec)
                            *best_rec = i;
                    }
                }
            }
        }
        if (__float_as_uint(v1.w))
            break;
        ++i;
    }
    return false;
}

// Planes of a mixed scene (outside the tree): every ray tests all of them.
// best_rec (optional) receives kRecPlane | j when plane j becomes the best hit.
constexpr uint32_t kRecPlane = 0x80000000u;

template <bool ANY>
__device__ __forceinline__ bool test_planes(const float4* __restrict__ planes, uint32_t count,
                                            uint32_t base, const RayState& r, BestHit& best,
                                            uint32_t* best_rec = nullptr) {
    for (uint32_t j = 0; j < count; ++j) {
        const uint32_t id = base + j;
        if (id == r.prev)
            continue;
        const float4 pl = __ldg(planes + j);
        const float t = plane_hit(r, pl);
        if (!(t >= r.tmin))
            continue;
        if (ANY) {
            if (t < r.tmax_eff)
                return true;
        } else if (better(t, prio_other(id), best)) {
            plane_uv(r, pl, t, best.u, best.v);
            best.t = t;
            best.prim = prio_other(id);
            best.tcull = cull_limit(t);
            if (best_rec)
                *best_rec = kRecPlane | j;
        }
    }
    return false;
}

// Rounds of trace_warp after which a warp gives up and reports
// kStatusRoundLimit (each round advances at least one lane by a node or a
// leaf, so a correct traversal stays far below this).
constexpr uint32_t kStatusRoundLimit = 2u;
constexpr uint32_t kTraceWarpRounds = 1u << 22;

// Closest hit of one ray per lane, called by all 32 lanes of the warp
// together with the same scene; the lanes with `active` set trace their rays
// (each lane's whole traversal, no refill) in the persistent kernels' order:
// the node phase (node_phase, with its early end) and the leaf phase
// alternate until every lane's traversal is over.  Each round's working
// lanes are those still tracing, so a finished lane never counts as waiting
// (the early end would otherwise keep ending the phase before the lanes
// still descending move).  MIXED: planes are tested first, best.prim ends as
// a priority code (id_of_prio gives the object) and best_rec as the best
// hit's record index, or kRecPlane | plane index.  Returns kStatusRoundLimit
// if the warp gave up, else 0.
template <int LAYOUT, bool MIXED>
__device__ __forceinline__ uint32_t trace_warp(const float4* __restrict__ nodes, const float4* __restrict__ prims,
                                               uint32_t node_count, const float4* __restrict__ planes,
                                               uint32_t plane_count, uint32_t plane_base, bool active,
                                               uint32_t phase_break, const RayState& r, BestHit& best,
                                               TraversalStack& st, bool& overflow, uint32_t& best_rec) {
    best.t = r.tmax_eff;
    best.u = 0.f;
    best.v = 0.f;
    best.prim = MIXED ? kPrioNone : 0u;
    best.tcull = cull_limit(best.t);
    best_rec = 0xffffffffu;
    if (MIXED && plane_count && active)
        test_planes<false>(planes, plane_count, plane_base, r, best, &best_rec);
    if (!node_count)
        return 0u;
    st.sp = 0;
    uint32_t unused = 0;
    int32_t next = active ? 0 : kRefDone;
    for (uint32_t round = 0;; ++round) {
        const bool tracing = next != kRefDone;
        const uint32_t live = __ballot_sync(0xffffffffu, tracing);
        if (live == 0)
            return 0u;
        if (round == kTraceWarpRounds)
            return kStatusRoundLimit;
        node_phase<LAYOUT, false, MIXED>(nodes, tracing, live, phase_break, next, r, best, st, overflow, unused);
        if (next < 0) {
            if (MIXED)
                process_leaf_mixed<false>(prims, next, r, best, nullptr, &best_rec);
            else
                process_leaf<false, false>(prims, next, r, best, unused);
            next = st.pop_live(best.tcull);
        }
    }
}

}  // namespace igxrt
