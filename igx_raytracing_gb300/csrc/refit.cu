// refit.cu — GPU refit of a resident scene for moving geometry.
//
// The reference re-uploads its moving spheres every frame and traces them with
// a linear loop (test/scene/niels_scene.cpp:61-70, res/shaders/trace.glsl:22-46);
// over a BVH, moved geometry needs the node boxes to follow.  Four passes on
// the caller's stream:
//   1. scan: bounds of every object, max |coordinate| (which sets the padding)
//      and the scene box, reduced per block, then one atomicMax per block and
//      state word; a non-finite coordinate records the object and turns the
//      later passes into no-ops, so a rejected refit leaves the scene as it was;
//   2. records: primitive records (triangle p0/e1/e2, sphere centre/radius, cube
//      corners) and the scene's triangle and plane copies are rewritten, and
//      every record's object box is stored in leaf order beside its leaf_end
//      flag (the scene's refit scratch);
//   3. nodes: a thread per node writes the node's leaf slots (from the stored
//      boxes: one contiguous read per record, shared by the BVH2 and BVH4
//      trees) and arrives at the node; each interior child's climber arrives
//      there too.  The last of the node's arrivals (an atomic counter per
//      node) writes its interior slots from the children's union boxes, stores
//      the node's own union box for its parent and climbs on; the others exit.
//      A climber so waits on two round trips per level (the arrival, then the
//      node's slots and its children's unions), and nothing waits on another
//      thread: a thread either continues or exits;
//   4. BVH8: every compressed node re-quantized from the BVH2 boxes its slots
//      were built from (eight lanes per node).
// Boxes follow the host builder exactly (same min/max argument order, padded by
// max(2^-18 * max|coordinate|, 1e-30)), so the GPU refit equals igxrt_bvh_refit
// bit for bit.
#include <cuda_runtime.h>

#include <algorithm>

#include "geometry.cuh"

namespace igxrt {

void node_parents(const igxrt_bvh& bvh, std::vector<uint32_t>& p2, std::vector<uint32_t>& p4) {
    p2.assign(bvh.nodes2.size(), kNoParent);
    p4.assign(bvh.nodes4.size(), kNoParent);
    for (size_t i = 0; i < bvh.nodes2.size(); ++i) {
        const igxrt_bvh2_node& n = bvh.nodes2[i];
        const bool used[2] = {true, !(n.c1_x[0] == INFINITY && n.c1_x[1] == INFINITY)};
        for (int c = 0; c < 2; ++c)
            if (used[c] && n.child[c] >= 0)
                p2[n.child[c]] = (uint32_t)i;
    }
    for (size_t i = 0; i < bvh.nodes4.size(); ++i) {
        const igxrt_bvh4_node& n = bvh.nodes4[i];
        for (int c = 0; c < 4; ++c)
            if (!(n.lo_x[c] == INFINITY && n.hi_x[c] == INFINITY) && n.child[c] >= 0)
                p4[n.child[c]] = (uint32_t)i;
    }
}

igxrt_status stage_scene_desc(igxrt_context* ctx, const igxrt_scene_desc* desc, uint32_t flags,
                              cudaStream_t s, SceneObjects& o) {
    if ((desc->triangle_count && !desc->triangles) || (desc->sphere_count && !desc->spheres) ||
        (desc->cube_count && !desc->cubes) || (desc->plane_count && !desc->planes))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "a primitive buffer with a non-zero count is NULL");
    const uint64_t total = (uint64_t)desc->triangle_count + desc->sphere_count + desc->cube_count;
    if (total + desc->plane_count >= 0x7fffffffu)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "too many primitives");
    o = SceneObjects{};
    o.nt = desc->triangle_count;
    o.ns = desc->sphere_count;
    o.nc = desc->cube_count;
    o.np = desc->plane_count;
    if (!(flags & IGXRT_TRACE_HOST_MEMORY)) {
        if (!device_accessible(desc->triangles) || !device_accessible(desc->spheres) ||
            !device_accessible(desc->cubes) || !device_accessible(desc->planes))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                        "a primitive buffer is not device memory (pass IGXRT_TRACE_HOST_MEMORY)");
        o.tris = desc->triangles;
        o.spheres = desc->spheres;
        o.cubes = desc->cubes;
        o.planes = desc->planes;
        return IGXRT_OK;
    }
    const size_t bt = sizeof(igxrt_triangle) * o.nt, bs = 16 * (size_t)o.ns,
                 bc = sizeof(igxrt_cube) * o.nc, bp = 16 * (size_t)o.np;
    const size_t os = round_up(bt, 256), oc = round_up(os + bs, 256), op = round_up(oc + bc, 256),
                 all = std::max<size_t>(op + bp, 256);
    igxrt_status st = grow_stage(ctx, all);
    if (st != IGXRT_OK)
        return st;
    char* base = static_cast<char*>(ctx->d_stage);
    o.tris = reinterpret_cast<const igxrt_triangle*>(base);
    o.spheres = reinterpret_cast<const float*>(base + os);
    o.cubes = reinterpret_cast<const igxrt_cube*>(base + oc);
    o.planes = reinterpret_cast<const float*>(base + op);
    cudaError_t e = cudaSuccess;
    if (bt)
        e = cudaMemcpyAsync(base, desc->triangles, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && bs)
        e = cudaMemcpyAsync(base + os, desc->spheres, bs, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && bc)
        e = cudaMemcpyAsync(base + oc, desc->cubes, bc, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && bp)
        e = cudaMemcpyAsync(base + op, desc->planes, bp, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "scene upload");
    return IGXRT_OK;
}

std::string non_finite_message(uint32_t bad_word, uint32_t objects) {
    const uint32_t id = ~bad_word;
    return id < objects ? format("primitive %u has a non-finite coordinate", id)
                        : format("plane %u has a non-finite coefficient", id - objects);
}

}  // namespace igxrt

using namespace igxrt;

namespace {

struct RefitArgs {
    SceneObjects obj;          // the new primitive buffers
    igxrt_prim_record* prims;  // the scene's copies
    igxrt_triangle* scene_tris;
    float* scene_planes;
    void* nodes2;
    void* nodes4;
    const uint32_t* parents2;
    const uint32_t* parents4;
    uint32_t n2, n4;
    uint32_t* state;  // kRefitStateWords, then arrival counters (n2, then n4)
    igxrt_bvh8_node* nodes8;
    const uint32_t* src8;
    uint32_t n8;
    float4* boxes;   // per record, in leaf order: {lo, leaf_end}, {hi, 0}
    float4* unions;  // per node of BVH2, then of BVH4: {lo, 0}, {hi, 0}
};

static_assert(kRefitStateWords == 8, "refit state words");

// Pass 1: maxabs, scene box and the non-finite check.
__global__ void __launch_bounds__(kScanBlock) refit_scan_kernel(RefitArgs a) {
    scan_objects<false>(a.obj, a.state);
}

// Pass 2: primitive records and the scene's triangle and plane copies.  The
// scene's buffers are 256-byte aligned; 16-byte loads and stores are used
// wherever the caller's buffer is 16-byte aligned too.
__global__ void refit_records_kernel(RefitArgs a) {
    if (a.state[kWordBad])
        return;
    const SceneObjects& o = a.obj;
    const uint32_t n = o.count();
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    const bool tris16 = (reinterpret_cast<uintptr_t>(o.tris) & 15u) == 0;
    float4* rec = reinterpret_cast<float4*>(a.prims);
    for (uint32_t i = first; i < n; i += stride) {
        float4 r0 = rec[3 * (size_t)i], r1 = rec[3 * (size_t)i + 1], r2 = rec[3 * (size_t)i + 2];
        const uint32_t id = __float_as_uint(r0.w);
        if (id < o.nt && tris16) {
            const float4* t = reinterpret_cast<const float4*>(o.tris + id);
            const float4 q0 = __ldg(t), q1 = __ldg(t + 1), q2 = __ldg(t + 2);
            r0 = make_float4(q0.x, q0.y, q0.z, r0.w);
            r1 = make_float4(__fsub_rn(q1.x, q0.x), __fsub_rn(q1.y, q0.y), __fsub_rn(q1.z, q0.z), r1.w);
            r2 = make_float4(__fsub_rn(q2.x, q0.x), __fsub_rn(q2.y, q0.y), __fsub_rn(q2.z, q0.z), r2.w);
        } else {
            igxrt_prim_record r;
            memcpy(&r, &r0, 16);
            memcpy(reinterpret_cast<char*>(&r) + 16, &r1, 16);
            memcpy(reinterpret_cast<char*>(&r) + 32, &r2, 16);
            fill_record(o, id, r);
            memcpy(&r0, &r, 16);
            memcpy(&r1, reinterpret_cast<const char*>(&r) + 16, 16);
            memcpy(&r2, reinterpret_cast<const char*>(&r) + 32, 16);
        }
        rec[3 * (size_t)i] = r0;
        rec[3 * (size_t)i + 1] = r1;
        rec[3 * (size_t)i + 2] = r2;
        const Box ob = object_box<false>(o, id);
        a.boxes[2 * (size_t)i] = make_float4(ob.lo[0], ob.lo[1], ob.lo[2], r1.w);  // r1.w: leaf_end
        a.boxes[2 * (size_t)i + 1] = make_float4(ob.hi[0], ob.hi[1], ob.hi[2], 0.f);
    }
    if (tris16) {
        const float4* src = reinterpret_cast<const float4*>(o.tris);
        float4* dst = reinterpret_cast<float4*>(a.scene_tris);
        for (size_t i = first; i < 3 * (size_t)o.nt; i += stride)
            dst[i] = __ldg(src + i);
    } else {
        for (uint32_t i = first; i < o.nt; i += stride)
            a.scene_tris[i] = o.tris[i];
    }
    for (uint32_t i = first; i < 4 * o.np; i += stride)
        a.scene_planes[i] = o.planes[i];
}

// Padded box of the leaf whose records start at ~ref: the union, in record
// order, of the object boxes the record pass stored.
__device__ Box leaf_box(const RefitArgs& a, int32_t ref, float pad) {
    Box b;
    b.reset();
    for (uint32_t i = (uint32_t)~ref;; ++i) {
        const float4 l = __ldg(a.boxes + 2 * (size_t)i), h = __ldg(a.boxes + 2 * (size_t)i + 1);
        Box ob;
        ob.lo[0] = l.x, ob.lo[1] = l.y, ob.lo[2] = l.z;
        ob.hi[0] = h.x, ob.hi[1] = h.y, ob.hi[2] = h.z;
        b.grow(ob);
        if (__float_as_uint(l.w))
            break;
    }
    b.pad(pad);
    return b;
}

// Pass 3 for one tree.  The thread of `node` writes the node's leaf slots,
// then every thread arrives at its node: a node takes one arrival from its
// own thread and one from the climber of each interior child, and the last
// one (the counter's acquire-release add makes every earlier arrival's
// writes visible to it) finishes the node: its interior slots from the
// children's stored unions, the node's own union (slots folded in slot
// order, as the host refit folds a child node's slots) stored for the
// parent, and on to the parent.  The slots and refs it reads are loaded
// after its arrival; the refs alone, which a refit never changes, are read
// before it.
template <int LAYOUT>
__device__ void refit_climb(const RefitArgs& a, uint32_t node, float pad) {
    using Ops = NodeOps<LAYOUT>;
    using Node = typename Ops::Node;
    Node* nodes = static_cast<Node*>(LAYOUT == IGXRT_LAYOUT_BVH2 ? a.nodes2 : a.nodes4);
    const uint32_t* parents = LAYOUT == IGXRT_LAYOUT_BVH2 ? a.parents2 : a.parents4;
    const uint32_t base = LAYOUT == IGXRT_LAYOUT_BVH2 ? 0u : a.n2;
    uint32_t* arrive = a.state + kRefitStateWords + base;
    float4* unions = a.unions + 2 * (size_t)base;
    float f[Ops::kFloats];
    Ops::load(nodes + node, f);
    for (int c = 0; c < Ops::kSlots; ++c) {
        if (Ops::empty(f, c) || Ops::child(f, c) >= 0)
            continue;
        Ops::put(nodes + node, c, leaf_box(a, Ops::child(f, c), pad));
    }
    for (;;) {
        int need = 1;
        for (int c = 0; c < Ops::kSlots; ++c)
            need += (!Ops::empty(f, c) && Ops::child(f, c) >= 0) ? 1 : 0;
        const uint32_t p = parents[node];
        if (arrive_at(arrive + node) + 1u != (uint32_t)need)
            return;  // another arrival at this node is still to come
        Ops::load(nodes + node, f);
        Box u;
        u.reset();
        for (int c = 0; c < Ops::kSlots; ++c) {
            if (Ops::empty(f, c))
                continue;
            const int32_t ref = Ops::child(f, c);
            Box b;
            if (ref >= 0) {
                const float4 l = __ldcg(unions + 2 * (size_t)ref), h = __ldcg(unions + 2 * (size_t)ref + 1);
                b.lo[0] = l.x, b.lo[1] = l.y, b.lo[2] = l.z;
                b.hi[0] = h.x, b.hi[1] = h.y, b.hi[2] = h.z;
                Ops::put(nodes + node, c, b);
            } else {
                Ops::get(f, c, b);
            }
            u.grow(b);
        }
        if (p == kNoParent)
            return;
        __stcg(unions + 2 * (size_t)node, make_float4(u.lo[0], u.lo[1], u.lo[2], 0.f));
        __stcg(unions + 2 * (size_t)node + 1, make_float4(u.hi[0], u.hi[1], u.hi[2], 0.f));
        node = p;
        Ops::load(nodes + node, f);  // refs only: its slots are read again after the arrival
    }
}

// Pass 3: one thread per node of BVH2, then of BVH4.
__global__ void refit_nodes_kernel(RefitArgs a) {
    if (a.state[kWordBad])
        return;
    const float pad = box_pad(a.state);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n2)
        refit_climb<IGXRT_LAYOUT_BVH2>(a, i, pad);
    else if (i < a.n2 + a.n4)
        refit_climb<IGXRT_LAYOUT_BVH4>(a, i - a.n2, pad);
}

// Pass 4: every BVH8 node re-quantized from the refit BVH2 boxes of its
// slots, eight lanes per node, one per slot.  The node's bounds are reduced
// across the eight lanes with the lower slot as the first operand of every
// comparison, which picks the same element as the host's slot-order loop in
// bvh8_quantize_node (ties, signed zeros included); three lanes find the
// axes' exponents with the same bvh8_exponent, each lane quantizes its own
// slot with the same bvh8_quantize, and the bytes are
// packed into words with shuffles and stored as four 16-byte words.
__global__ void __launch_bounds__(128) refit_bvh8_kernel(RefitArgs a) {
    if (a.state[kWordBad])
        return;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t node = t >> 3;
    const uint32_t slot = (uint32_t)(t & 7u);
    const bool live = node < a.n8;  // the same for the eight lanes of a node
    const uint32_t src = live ? a.src8[8 * node + slot] : kNoSource;
    const bool used = src != kNoSource;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (used) {
        const float4* q = reinterpret_cast<const float4*>(static_cast<const igxrt_bvh2_node*>(a.nodes2) +
                                                          (src >> 1));
        const uint32_t s = src & 1u;
        const float4 xy = q[s];  // c{s}_x, c{s}_y
        const float2 z = reinterpret_cast<const float2*>(q + 2)[s];  // c{s}_z
        lo[0] = xy.x, hi[0] = xy.y, lo[1] = xy.z, hi[1] = xy.w, lo[2] = z.x, hi[2] = z.y;
    }
    float nlo[3], nhi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nlo[k] = lo[k];
        nhi[k] = hi[k];
    }
#pragma unroll
    for (int d = 1; d < 8; d <<= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float olo = __shfl_down_sync(0xffffffffu, nlo[k], d, 8);
            const float ohi = __shfl_down_sync(0xffffffffu, nhi[k], d, 8);
            nlo[k] = olo < nlo[k] ? olo : nlo[k];
            nhi[k] = nhi[k] < ohi ? ohi : nhi[k];
        }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nlo[k] = __shfl_sync(0xffffffffu, nlo[k], 0, 8);
        nhi[k] = __shfl_sync(0xffffffffu, nhi[k], 0, 8);
    }
    // lanes 0, 1 and 2 of the node find the exponent of axis x, y and z
    const float alo = slot == 0 ? nlo[0] : (slot == 1 ? nlo[1] : nlo[2]);
    const float ahi = slot == 0 ? nhi[0] : (slot == 1 ? nhi[1] : nhi[2]);
    const int my_e = live && slot < 3 ? bvh8_exponent(alo, ahi) : 0;
    uint32_t word[6];  // lo_x, hi_x, lo_y, hi_y, lo_z, hi_z: this lane's byte in place
    int e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e[k] = __shfl_sync(0xffffffffu, my_e, k, 8);
        uint8_t ql = 0, qh = 0;
        if (used)
            bvh8_quantize(nlo[k], e[k], lo[k], hi[k], ql, qh);
        word[2 * k] = (uint32_t)ql << (8 * (slot & 3u));
        word[2 * k + 1] = (uint32_t)qh << (8 * (slot & 3u));
    }
    uint32_t half[2][6];  // [slots 0-3 | slots 4-7][array]
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        uint32_t w = word[k];
        w |= __shfl_xor_sync(0xffffffffu, w, 1, 8);
        w |= __shfl_xor_sync(0xffffffffu, w, 2, 8);
        const uint32_t other = __shfl_xor_sync(0xffffffffu, w, 4, 8);
        half[0][k] = slot < 4 ? w : other;
        half[1][k] = slot < 4 ? other : w;
    }
    if (!live || slot > 3)
        return;
    uint4* out = reinterpret_cast<uint4*>(a.nodes8 + node);
    uint4 v;
    if (slot == 0) {
        const uint32_t valid = out[0].w & 0xff000000u;  // kept; the exponents are rewritten
        v = make_uint4(__float_as_uint(nlo[0]), __float_as_uint(nlo[1]), __float_as_uint(nlo[2]),
                       (uint32_t)(uint8_t)e[0] | (uint32_t)(uint8_t)e[1] << 8 | (uint32_t)(uint8_t)e[2] << 16 |
                           valid);
    } else {
        const int k = 2 * (int)(slot - 1);  // slot 1: lo_x, hi_x; 2: lo_y, hi_y; 3: lo_z, hi_z
        v = make_uint4(half[0][k], half[1][k], half[0][k + 1], half[1][k + 1]);
    }
    out[slot] = v;
}

}  // namespace

extern "C" {

igxrt_status igxrt_scene_refit(igxrt_context* ctx, igxrt_scene* scene, const igxrt_scene_desc* desc,
                               uint32_t flags, void* stream) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (!desc)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "desc is NULL");
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    if (flags & ~IGXRT_TRACE_HOST_MEMORY)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown flags 0x%x", flags));
    const igxrt_bvh_info& info = scene->info;
    if (desc->triangle_count != info.triangle_count || desc->sphere_count != info.sphere_count ||
        desc->cube_count != info.cube_count || desc->plane_count != info.plane_count)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("refit needs the primitive counts of the scene (%u/%u/%u/%u triangles/"
                           "spheres/cubes/planes)", info.triangle_count, info.sphere_count,
                           info.cube_count, info.plane_count));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    RefitArgs a{};
    if ((st = stage_scene_desc(ctx, desc, flags, s, a.obj)) != IGXRT_OK)
        return st;
    a.prims = const_cast<igxrt_prim_record*>(scene->prims);
    a.scene_tris = const_cast<igxrt_triangle*>(scene->tris);
    a.scene_planes = const_cast<float*>(scene->planes);
    a.nodes2 = const_cast<void*>(scene->nodes[IGXRT_LAYOUT_BVH2]);
    a.nodes4 = const_cast<void*>(scene->nodes[IGXRT_LAYOUT_BVH4]);
    a.parents2 = scene->parents[IGXRT_LAYOUT_BVH2];
    a.parents4 = scene->parents[IGXRT_LAYOUT_BVH4];
    a.n2 = scene->node_count[IGXRT_LAYOUT_BVH2];
    a.n4 = scene->node_count[IGXRT_LAYOUT_BVH4];
    a.state = scene->refit_words;
    a.nodes8 = static_cast<igxrt_bvh8_node*>(const_cast<void*>(scene->nodes[IGXRT_LAYOUT_BVH8]));
    a.src8 = scene->src8;
    a.n8 = scene->node_count[IGXRT_LAYOUT_BVH8];

    const uint32_t n = a.obj.count();
    if (n && !scene->refit_boxes) {  // once per scene, at its first refit
        const cudaError_t e = cudaMalloc(&scene->refit_boxes, 2 * sizeof(float4) * (size_t)n);
        if (e != cudaSuccess) {
            scene->refit_boxes = nullptr;
            return cuda_fail(ctx, e, "refit scratch allocation");
        }
    }
    a.boxes = scene->refit_boxes;
    if (a.n2 + a.n4 && !scene->refit_unions) {
        const cudaError_t e = cudaMalloc(&scene->refit_unions, 2 * sizeof(float4) * ((size_t)a.n2 + a.n4));
        if (e != cudaSuccess) {
            scene->refit_unions = nullptr;
            return cuda_fail(ctx, e, "refit scratch allocation");
        }
    }
    a.unions = scene->refit_unions;
    const size_t words = kRefitStateWords + (size_t)a.n2 + a.n4;
    cudaError_t e = cudaMemsetAsync(a.state, 0, words * sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit state reset");
    const uint32_t span = std::max({n, 4 * a.obj.np, 1u});
    const uint32_t grid = std::min<uint32_t>((span + kScanBlock - 1) / kScanBlock,
                                             (uint32_t)std::max(ctx->sm_count, 1) * 4);
    refit_scan_kernel<<<grid, kScanBlock, 0, s>>>(a);
    refit_records_kernel<<<grid, kScanBlock, 0, s>>>(a);
    const uint32_t nodes = a.n2 + a.n4;
    if (nodes)
        refit_nodes_kernel<<<(nodes + 127) / 128, 128, 0, s>>>(a);
    if (a.n8)
        refit_bvh8_kernel<<<(uint32_t)((8 * (uint64_t)a.n8 + 127) / 128), 128, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit launch");
    uint32_t w[kRefitStateWords];
    e = cudaMemcpyAsync(w, a.state, sizeof(w), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit");
    if (w[kWordBad])
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, non_finite_message(w[kWordBad], n));
    float maxabs;
    memcpy(&maxabs, &w[kWordMaxAbs], 4);
    scene->info.pad_abs = std::max(maxabs * 0x1p-18f, 1e-30f);
    for (int k = 0; k < 3; ++k) {
        scene->info.bounds[k] = n ? key_to_float(~w[kWordLo + k]) : 0.f;
        scene->info.bounds[3 + k] = n ? key_to_float(w[kWordHi + k]) : 0.f;
    }
    return IGXRT_OK;
}

igxrt_status igxrt_scene_read_bvh(igxrt_context* ctx, const igxrt_scene* scene, uint32_t layout,
                                  void* nodes, uint64_t node_count, igxrt_prim_record* prims,
                                  uint64_t prim_count) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    if (layout >= IGXRT_LAYOUT_COUNT)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown layout %u", layout));
    const uint64_t records =
        (uint64_t)scene->info.triangle_count + scene->info.sphere_count + scene->info.cube_count;
    if (nodes && node_count != scene->node_count[layout])
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("node_count %llu, the scene has %u", (unsigned long long)node_count,
                           scene->node_count[layout]));
    if (prims && prim_count != records)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("prim_count %llu, the scene has %llu", (unsigned long long)prim_count,
                           (unsigned long long)records));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaError_t e = cudaDeviceSynchronize();
    const size_t node_bytes = layout == IGXRT_LAYOUT_BVH2   ? sizeof(igxrt_bvh2_node)
                              : layout == IGXRT_LAYOUT_BVH4 ? sizeof(igxrt_bvh4_node)
                                                            : sizeof(igxrt_bvh8_node);
    if (e == cudaSuccess && nodes && node_count)
        e = cudaMemcpy(nodes, scene->nodes[layout], node_bytes * node_count, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && prims && prim_count)
        e = cudaMemcpy(prims, scene->prims, sizeof(igxrt_prim_record) * prim_count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "scene read-back");
    return IGXRT_OK;
}

}  // extern "C"
