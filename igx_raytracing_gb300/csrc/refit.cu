// refit.cu — GPU refit of a resident scene for moving geometry.
//
// The reference re-uploads its moving spheres every frame and traces them with
// a linear loop (test/scene/niels_scene.cpp:61-70, res/shaders/trace.glsl:22-46);
// over a BVH, moved geometry needs the node boxes to follow.  Three passes on
// the caller's stream:
//   1. scan: bounds of every object, max |coordinate| (which sets the padding)
//      and the scene box, reduced per block, then one atomicMax per block and
//      state word; a non-finite coordinate records the object and turns the
//      later passes into no-ops, so a rejected refit leaves the scene as it was;
//   2. records: primitive records (triangle p0/e1/e2, sphere centre/radius, cube
//      corners) and the scene's triangle and plane copies are rewritten;
//   3. nodes: a thread per node whose children are all leaves writes that
//      node's slot boxes, then climbs through the parent links.  At each parent
//      an atomic arrival counter lets only the thread of the last interior child
//      go on, so every node is written once, after all of its children.  Nothing
//      waits on another thread: a thread either continues or exits.
// Boxes follow the host builder exactly (same min/max argument order, padded by
// max(2^-18 * max|coordinate|, 1e-30)), so the GPU refit equals igxrt_bvh_refit
// bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "engine.h"

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

}  // namespace igxrt

using namespace igxrt;

namespace {

// State words (all reduced with atomicMax, zeroed before the refit):
//   0      max |coordinate| as float bits (non-negative floats order as words)
//   1..3   ~order_key(scene lo) per axis
//   4..6   order_key(scene hi) per axis
//   7      ~(first object with a non-finite value), 0 when none
constexpr int kWordMaxAbs = 0, kWordLo = 1, kWordHi = 4, kWordBad = 7;
constexpr int kScanBlock = 256;

struct RefitArgs {
    const igxrt_triangle* tris;  // the new primitive buffers
    const float* spheres;
    const igxrt_cube* cubes;
    const float* planes;
    uint32_t nt, ns, nc, np;
    igxrt_prim_record* prims;  // the scene's copies
    igxrt_triangle* scene_tris;
    float* scene_planes;
    uint32_t n_records;
    void* nodes2;
    void* nodes4;
    const uint32_t* parents2;
    const uint32_t* parents4;
    uint32_t n2, n4;
    uint32_t* state;  // kRefitStateWords, then arrival counters (n2, then n4)
};

// std::min / std::max of the host builder, argument order included.
__device__ __forceinline__ float host_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float host_max(float a, float b) { return (a < b) ? b : a; }

__device__ __forceinline__ uint32_t order_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Box {
    float lo[3], hi[3];
    __device__ void reset() {
        for (int k = 0; k < 3; ++k) {
            lo[k] = INFINITY;
            hi[k] = -INFINITY;
        }
    }
    __device__ void grow_point(const float* p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = host_min(lo[k], p[k]);
            hi[k] = host_max(hi[k], p[k]);
        }
    }
    __device__ void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = host_min(lo[k], b.lo[k]);
            hi[k] = host_max(hi[k], b.hi[k]);
        }
    }
};

// Object bounds by the builder's rule over the points it bounds: triangle
// vertices; sphere centre -/+ |radius|; cube start and end corners.  With
// CHECK, `finite` and `maxabs` cover the same points.
template <bool CHECK>
__device__ Box object_box(const RefitArgs& a, uint32_t id, bool* finite = nullptr, float* maxabs = nullptr) {
    float v[3][3];
    int nv;
    if (id < a.nt) {
        const igxrt_triangle& t = a.tris[id];
        for (int k = 0; k < 3; ++k) {
            v[0][k] = t.p0[k];
            v[1][k] = t.p1[k];
            v[2][k] = t.p2[k];
        }
        nv = 3;
    } else if (id < a.nt + a.ns) {
        const float* s = a.spheres + 4 * (size_t)(id - a.nt);
        const float r = fabsf(s[3]);
        for (int k = 0; k < 3; ++k) {
            v[0][k] = __fsub_rn(s[k], r);
            v[1][k] = __fadd_rn(s[k], r);
        }
        nv = 2;
    } else {
        const igxrt_cube& c = a.cubes[id - a.nt - a.ns];
        v[0][0] = c.xy0[0];
        v[0][1] = c.xy0[1];
        v[0][2] = c.z0_x1[0];
        v[1][0] = c.z0_x1[1];
        v[1][1] = c.yz1[0];
        v[1][2] = c.yz1[1];
        nv = 2;
    }
    Box b;
    b.reset();
    for (int j = 0; j < nv; ++j) {
        if (CHECK) {
            for (int k = 0; k < 3; ++k) {
                *finite = *finite && isfinite(v[j][k]);
                *maxabs = fmaxf(*maxabs, fabsf(v[j][k]));
            }
        }
        b.grow_point(v[j]);
    }
    return b;
}

// Pass 1: maxabs, scene box and the non-finite check (grid-stride, then one
// reduction per block).
__global__ void __launch_bounds__(kScanBlock) refit_scan_kernel(RefitArgs a) {
    uint32_t w[kRefitStateWords] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t n = a.nt + a.ns + a.nc;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += stride) {
        bool finite = true;
        float m = 0.f;
        const Box b = object_box<true>(a, id, &finite, &m);
        if (!finite) {
            w[kWordBad] = max(w[kWordBad], ~id);
            continue;
        }
        w[kWordMaxAbs] = max(w[kWordMaxAbs], __float_as_uint(m));
        for (int k = 0; k < 3; ++k) {
            w[kWordLo + k] = max(w[kWordLo + k], ~order_key(b.lo[k]));
            w[kWordHi + k] = max(w[kWordHi + k], order_key(b.hi[k]));
        }
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * a.np; i += stride)
        if (!isfinite(a.planes[i]))
            w[kWordBad] = max(w[kWordBad], ~(n + i / 4));
    __shared__ uint32_t red[kScanBlock / 32][kRefitStateWords];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int k = 0; k < (int)kRefitStateWords; ++k) {
        const uint32_t v = __reduce_max_sync(0xffffffffu, w[k]);
        if (lane == 0)
            red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kRefitStateWords) {
        uint32_t v = 0;
        for (int i = 0; i < kScanBlock / 32; ++i)
            v = max(v, red[i][threadIdx.x]);
        if (v)
            atomicMax(a.state + threadIdx.x, v);
    }
}

// Pass 2: primitive records and the scene's triangle and plane copies.
__global__ void refit_records_kernel(RefitArgs a) {
    if (a.state[kWordBad])
        return;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t span = max(max(a.n_records, a.nt), 4 * a.np);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < span; i += stride) {
        if (i < a.n_records) {
            igxrt_prim_record r = a.prims[i];
            const uint32_t id = r.prim;
            if (id < a.nt) {
                const igxrt_triangle& t = a.tris[id];
                for (int k = 0; k < 3; ++k) {
                    r.p0[k] = t.p0[k];
                    r.e1[k] = __fsub_rn(t.p1[k], t.p0[k]);
                    r.e2[k] = __fsub_rn(t.p2[k], t.p0[k]);
                }
            } else if (id < a.nt + a.ns) {
                const float* s = a.spheres + 4 * (size_t)(id - a.nt);
                for (int k = 0; k < 3; ++k)
                    r.p0[k] = s[k];
                r.e1[0] = s[3];
            } else {
                const igxrt_cube& c = a.cubes[id - a.nt - a.ns];
                r.p0[0] = c.xy0[0];
                r.p0[1] = c.xy0[1];
                r.p0[2] = c.z0_x1[0];
                r.e1[0] = c.z0_x1[1];
                r.e1[1] = c.yz1[0];
                r.e1[2] = c.yz1[1];
            }
            a.prims[i] = r;
        }
        if (i < a.nt)
            a.scene_tris[i] = a.tris[i];
        if (i < 4 * a.np)
            a.scene_planes[i] = a.planes[i];
    }
}

__device__ Box leaf_box(const RefitArgs& a, int32_t ref, float pad) {
    Box b;
    b.reset();
    for (uint32_t i = (uint32_t)~ref;; ++i) {
        b.grow(object_box<false>(a, a.prims[i].prim));
        if (a.prims[i].leaf_end)
            break;
    }
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = __fsub_rn(b.lo[k], pad);
        b.hi[k] = __fadd_rn(b.hi[k], pad);
    }
    return b;
}

// Node access per layout: slot boxes, child refs and empty slots.  Reads of
// child nodes go through L2 (ld.global.cg): another SM may have written them.
template <int LAYOUT>
struct NodeOps;

template <>
struct NodeOps<IGXRT_LAYOUT_BVH2> {
    static constexpr int kSlots = 2;
    using Node = igxrt_bvh2_node;
    __device__ static void load(const Node* p, float (&f)[16]) {
        const float4* q = reinterpret_cast<const float4*>(p);
        for (int i = 0; i < 4; ++i) {
            const float4 v = __ldcg(q + i);
            f[4 * i] = v.x;
            f[4 * i + 1] = v.y;
            f[4 * i + 2] = v.z;
            f[4 * i + 3] = v.w;
        }
    }
    // slot c: x at 4c, y at 4c + 2, z at 8 + 2c (lo, hi pairs)
    __device__ static bool empty(const float (&f)[16], int c) {
        return f[4 * c] == INFINITY && f[4 * c + 1] == INFINITY;
    }
    __device__ static int32_t child(const float (&f)[16], int c) { return __float_as_int(f[12 + c]); }
    __device__ static void get(const float (&f)[16], int c, Box& b) {
        b.lo[0] = f[4 * c];
        b.hi[0] = f[4 * c + 1];
        b.lo[1] = f[4 * c + 2];
        b.hi[1] = f[4 * c + 3];
        b.lo[2] = f[8 + 2 * c];
        b.hi[2] = f[8 + 2 * c + 1];
    }
    __device__ static void put(Node* p, int c, const Box& b) {
        float* x = c ? p->c1_x : p->c0_x;
        float* y = c ? p->c1_y : p->c0_y;
        float* z = c ? p->c1_z : p->c0_z;
        x[0] = b.lo[0];
        x[1] = b.hi[0];
        y[0] = b.lo[1];
        y[1] = b.hi[1];
        z[0] = b.lo[2];
        z[1] = b.hi[2];
    }
};

template <>
struct NodeOps<IGXRT_LAYOUT_BVH4> {
    static constexpr int kSlots = 4;
    using Node = igxrt_bvh4_node;
    __device__ static void load(const Node* p, float (&f)[32]) {
        const float4* q = reinterpret_cast<const float4*>(p);
        for (int i = 0; i < 8; ++i) {
            const float4 v = __ldcg(q + i);
            f[4 * i] = v.x;
            f[4 * i + 1] = v.y;
            f[4 * i + 2] = v.z;
            f[4 * i + 3] = v.w;
        }
    }
    // lo_x 0..3, hi_x 4..7, lo_y 8..11, hi_y 12..15, lo_z 16..19, hi_z 20..23
    __device__ static bool empty(const float (&f)[32], int c) {
        return f[c] == INFINITY && f[4 + c] == INFINITY;
    }
    __device__ static int32_t child(const float (&f)[32], int c) { return __float_as_int(f[24 + c]); }
    __device__ static void get(const float (&f)[32], int c, Box& b) {
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = f[8 * k + c];
            b.hi[k] = f[8 * k + 4 + c];
        }
    }
    __device__ static void put(Node* p, int c, const Box& b) {
        p->lo_x[c] = b.lo[0];
        p->hi_x[c] = b.hi[0];
        p->lo_y[c] = b.lo[1];
        p->hi_y[c] = b.hi[1];
        p->lo_z[c] = b.lo[2];
        p->hi_z[c] = b.hi[2];
    }
};

template <int LAYOUT>
__device__ int interior_children(const typename NodeOps<LAYOUT>::Node* node) {
    using Ops = NodeOps<LAYOUT>;
    float f[Ops::kSlots * 8];
    Ops::load(node, f);
    int k = 0;
    for (int c = 0; c < Ops::kSlots; ++c)
        k += (!Ops::empty(f, c) && Ops::child(f, c) >= 0) ? 1 : 0;
    return k;
}

// Writes every non-empty slot of `node`: a leaf slot from its objects, an
// interior slot as the union of the child node's (already written) slots.
template <int LAYOUT>
__device__ void refit_node(const RefitArgs& a, typename NodeOps<LAYOUT>::Node* nodes, uint32_t node,
                           float pad) {
    using Ops = NodeOps<LAYOUT>;
    float f[Ops::kSlots * 8];
    Ops::load(nodes + node, f);
    for (int c = 0; c < Ops::kSlots; ++c) {
        if (Ops::empty(f, c))
            continue;
        const int32_t ref = Ops::child(f, c);
        Box b;
        if (ref < 0) {
            b = leaf_box(a, ref, pad);
        } else {
            float g[Ops::kSlots * 8];
            Ops::load(nodes + ref, g);
            b.reset();
            for (int s = 0; s < Ops::kSlots; ++s) {
                if (Ops::empty(g, s))
                    continue;
                Box gb;
                Ops::get(g, s, gb);
                b.grow(gb);
            }
        }
        Ops::put(nodes + node, c, b);
    }
}

template <int LAYOUT>
__device__ void refit_climb(const RefitArgs& a, uint32_t node, float pad) {
    using Node = typename NodeOps<LAYOUT>::Node;
    Node* nodes = static_cast<Node*>(LAYOUT == IGXRT_LAYOUT_BVH2 ? a.nodes2 : a.nodes4);
    const uint32_t* parents = LAYOUT == IGXRT_LAYOUT_BVH2 ? a.parents2 : a.parents4;
    uint32_t* arrive = a.state + kRefitStateWords + (LAYOUT == IGXRT_LAYOUT_BVH2 ? 0 : a.n2);
    if (interior_children<LAYOUT>(nodes + node) != 0)
        return;  // some child's thread reaches this node
    for (;;) {
        refit_node<LAYOUT>(a, nodes, node, pad);
        const uint32_t p = parents[node];
        if (p == kNoParent)
            return;
        __threadfence();  // this node's boxes before the arrival
        const uint32_t need = (uint32_t)interior_children<LAYOUT>(nodes + p);
        if (atomicAdd(arrive + p, 1u) + 1u != need)
            return;  // a sibling's thread is still below; it will come up
        __threadfence();  // the siblings' boxes after their arrivals
        node = p;
    }
}

// Pass 3: one thread per node of BVH2, then of BVH4.
__global__ void refit_nodes_kernel(RefitArgs a) {
    if (a.state[kWordBad])
        return;
    const float maxabs = __uint_as_float(a.state[kWordMaxAbs]);
    const float pad = fmaxf(__fmul_rn(maxabs, 0x1p-18f), 1e-30f);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n2)
        refit_climb<IGXRT_LAYOUT_BVH2>(a, i, pad);
    else if (i < a.n2 + a.n4)
        refit_climb<IGXRT_LAYOUT_BVH4>(a, i - a.n2, pad);
}

float key_to_float(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

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
    if ((desc->triangle_count && !desc->triangles) || (desc->sphere_count && !desc->spheres) ||
        (desc->cube_count && !desc->cubes) || (desc->plane_count && !desc->planes))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "a primitive buffer with a non-zero count is NULL");
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    RefitArgs a{};
    a.nt = desc->triangle_count;
    a.ns = desc->sphere_count;
    a.nc = desc->cube_count;
    a.np = desc->plane_count;
    const size_t bt = sizeof(igxrt_triangle) * a.nt, bs = 16 * (size_t)a.ns,
                 bc = sizeof(igxrt_cube) * a.nc, bp = 16 * (size_t)a.np;
    cudaError_t e = cudaSuccess;
    if (flags & IGXRT_TRACE_HOST_MEMORY) {
        const size_t ot = 0, os = round_up(ot + bt, 256), oc = round_up(os + bs, 256),
                     op = round_up(oc + bc, 256), total = std::max<size_t>(op + bp, 256);
        if ((st = grow_stage(ctx, total)) != IGXRT_OK)
            return st;
        char* base = static_cast<char*>(ctx->d_stage);
        a.tris = reinterpret_cast<const igxrt_triangle*>(base + ot);
        a.spheres = reinterpret_cast<const float*>(base + os);
        a.cubes = reinterpret_cast<const igxrt_cube*>(base + oc);
        a.planes = reinterpret_cast<const float*>(base + op);
        if (bt)
            e = cudaMemcpyAsync(base + ot, desc->triangles, bt, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && bs)
            e = cudaMemcpyAsync(base + os, desc->spheres, bs, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && bc)
            e = cudaMemcpyAsync(base + oc, desc->cubes, bc, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && bp)
            e = cudaMemcpyAsync(base + op, desc->planes, bp, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "refit upload");
    } else {
        if (!device_accessible(desc->triangles) || !device_accessible(desc->spheres) ||
            !device_accessible(desc->cubes) || !device_accessible(desc->planes))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                        "a primitive buffer is not device memory (pass IGXRT_TRACE_HOST_MEMORY)");
        a.tris = desc->triangles;
        a.spheres = desc->spheres;
        a.cubes = desc->cubes;
        a.planes = desc->planes;
    }
    a.prims = const_cast<igxrt_prim_record*>(scene->prims);
    a.scene_tris = const_cast<igxrt_triangle*>(scene->tris);
    a.scene_planes = const_cast<float*>(scene->planes);
    a.n_records = a.nt + a.ns + a.nc;
    a.nodes2 = const_cast<void*>(scene->nodes[IGXRT_LAYOUT_BVH2]);
    a.nodes4 = const_cast<void*>(scene->nodes[IGXRT_LAYOUT_BVH4]);
    a.parents2 = scene->parents[IGXRT_LAYOUT_BVH2];
    a.parents4 = scene->parents[IGXRT_LAYOUT_BVH4];
    a.n2 = scene->node_count[IGXRT_LAYOUT_BVH2];
    a.n4 = scene->node_count[IGXRT_LAYOUT_BVH4];
    a.state = scene->refit_words;

    const size_t words = kRefitStateWords + (size_t)a.n2 + a.n4;
    e = cudaMemsetAsync(a.state, 0, words * sizeof(uint32_t), s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit state reset");
    const uint32_t span = std::max({a.n_records, 4 * a.np, 1u});
    const uint32_t grid = std::min<uint32_t>((span + kScanBlock - 1) / kScanBlock,
                                             (uint32_t)std::max(ctx->sm_count, 1) * 4);
    refit_scan_kernel<<<grid, kScanBlock, 0, s>>>(a);
    refit_records_kernel<<<grid, kScanBlock, 0, s>>>(a);
    const uint32_t nodes = a.n2 + a.n4;
    if (nodes)
        refit_nodes_kernel<<<(nodes + 127) / 128, 128, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit launch");
    uint32_t w[kRefitStateWords];
    e = cudaMemcpyAsync(w, a.state, sizeof(w), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "refit");
    if (w[kWordBad]) {
        const uint32_t id = ~w[kWordBad];
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    id < a.n_records ? format("primitive %u has a non-finite coordinate", id)
                                     : format("plane %u has a non-finite coefficient", id - a.n_records));
    }
    float maxabs;
    memcpy(&maxabs, &w[kWordMaxAbs], 4);
    scene->info.pad_abs = std::max(maxabs * 0x1p-18f, 1e-30f);
    for (int k = 0; k < 3; ++k) {
        scene->info.bounds[k] = a.n_records ? key_to_float(~w[kWordLo + k]) : 0.f;
        scene->info.bounds[3 + k] = a.n_records ? key_to_float(w[kWordHi + k]) : 0.f;
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
    const size_t node_bytes = layout == IGXRT_LAYOUT_BVH2 ? sizeof(igxrt_bvh2_node) : sizeof(igxrt_bvh4_node);
    if (e == cudaSuccess && nodes && node_count)
        e = cudaMemcpy(nodes, scene->nodes[layout], node_bytes * node_count, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && prims && prim_count)
        e = cudaMemcpy(prims, scene->prims, sizeof(igxrt_prim_record) * prim_count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "scene read-back");
    return IGXRT_OK;
}

}  // extern "C"
