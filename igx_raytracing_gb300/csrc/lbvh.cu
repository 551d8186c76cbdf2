// lbvh.cu — BVH build on the GPU for geometry that changes every frame.
//
// The reference uploads its scene every frame (test/scene/niels_scene.cpp:
// 61-70) and traces it with a linear loop; the host SAH builder takes about a
// second per million triangles, so a per-frame scene needs a device build.
// This is a linear BVH (Morton order + radix tree, after Karras 2012, "Maximizing
// parallelism in the construction of BVHs, octrees, and k-d trees"), emitted in
// the same node formats, records and padding rule as the host builder so that
// the traversal kernels, the refit and the read-back work on it unchanged:
//   1. scan: object bounds, max |coordinate|, scene and centroid boxes, the
//      non-finite check (shared with the refit);
//   2. keys: 30-bit Morton code of the centroid in the centroid box, above the
//      object id (so keys are unique), sorted with CUB's radix sort;
//   3. radix tree: one thread per internal node finds its range and split
//      from the common-prefix lengths of neighbouring keys;
//   4. boxes: one thread per object climbs from its leaf; at each node the
//      first arriving child's thread stops and the second computes the union
//      (nothing waits);
//   5. leaves: a subtree of at most `max_leaf_size` objects becomes one leaf
//      (its objects are contiguous in key order, so records stay in leaf
//      order); the remaining internal nodes are compacted by a prefix sum and
//      written as BVH2 nodes with padded boxes;
//   6. BVH4: collapsed top down one level per launch, opening the child of
//      largest area until four slots are used (the host rule);
//   7. stack bounds and depth: bottom-up climbs like the refit's.
// The scene is then allocated exactly and the arrays are copied into it.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <vector>

#include "geometry.cuh"

using namespace igxrt;

namespace {

// State words after the scan's (which use 0..13).
constexpr int kWordNodes2 = 16, kWordNodes4 = 17, kWordLeaves = 18, kWordStack2 = 19, kWordStack4 = 20,
              kWordDepth = 21, kWordMalformed = 22;
constexpr int kWordSah = 32;       // double (words 32, 33)
constexpr int kWordLevels = 64;    // frontier sizes of the BVH4 levels
constexpr int kMaxLevels = 64;     // > key bits: no path is longer
constexpr int kStateWords = kWordLevels + kMaxLevels + 1;
constexpr uint32_t kDefaultLeaf = 4;

struct BuildArgs {
    SceneObjects obj;
    uint32_t n;       // objects in the tree
    uint32_t leaf;    // largest subtree emitted as one leaf
    uint32_t idbits;  // low key bits holding the object id
    uint32_t* state;
    const uint64_t* keys;  // sorted
    int32_t* kchild;       // 2 per internal node: >= 0 internal, < 0 ~key position
    uint2* krange;         // first, last key position
    uint32_t* kparent;     // per internal node
    uint32_t* lparent;     // per key position
    float* kbox;           // 6 per internal node: lo xyz, hi xyz (unpadded)
    uint32_t* arrive;      // per internal node (reused by the climbs)
    uint32_t* live;        // per internal node: 1 if it becomes a BVH2 node
    uint32_t* map;         // exclusive prefix sum of `live`
    igxrt_bvh2_node* nodes2;
    igxrt_bvh4_node* nodes4;
    uint32_t* parents2;
    uint32_t* parents4;
    igxrt_prim_record* prims;
    uint2* frontier[2];    // (BVH2 node, BVH4 node) pairs of one level
    uint32_t* stack_v;     // climb values per node: stack bound
    uint32_t* depth_v;     //                         depth
};

__device__ __forceinline__ float key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ uint32_t object_of(const BuildArgs& a, uint32_t pos) {
    return (uint32_t)(a.keys[pos] & ((1ull << a.idbits) - 1));
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void __launch_bounds__(kScanBlock) build_scan_kernel(BuildArgs a) {
    scan_objects<true>(a.obj, a.state);
}

// Every key is written, also when the scan found a non-finite value (the
// build is rejected afterwards): the object id in the low bits keeps the keys
// distinct, which is all the radix tree needs to be well formed.
__global__ void morton_kernel(BuildArgs a, uint64_t* keys) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.n)
        return;
    const Box b = object_box<false>(a.obj, id);
    uint32_t code = 0;
    for (int k = 0; k < 3; ++k) {
        const float lo = key_float(~a.state[kWordCenLo + k]);
        const float hi = key_float(a.state[kWordCenHi + k]);
        const float c = __fmul_rn(__fadd_rn(b.lo[k], b.hi[k]), 0.5f);
        const float ext = hi - lo;
        float u = ext > 0.f ? (c - lo) / ext : 0.f;
        u = fminf(fmaxf(u, 0.f), 1.f);  // a NaN becomes 0
        const uint32_t q = min((uint32_t)(u * 1024.f), 1023u);
        code |= spread10(q) << (2 - k);
    }
    keys[id] = ((uint64_t)code << a.idbits) | id;
}

__device__ __forceinline__ int prefix(const uint64_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n)
        return -1;
    return __clzll(keys[i] ^ keys[j]);
}

// Radix tree over the sorted keys (Karras 2012, section 4).
__global__ void radix_tree_kernel(BuildArgs a) {
    const int64_t n = a.n;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    const uint64_t* k = a.keys;
    const int d = prefix(k, n, i, i + 1) - prefix(k, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = prefix(k, n, i, i - d);
    int64_t lmax = 2;
    while (prefix(k, n, i, i + lmax * d) > dmin)
        lmax <<= 1;
    int64_t l = 0;
    for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix(k, n, i, i + (l + t) * d) > dmin)
            l += t;
    const int64_t j = i + l * d;
    const int dnode = prefix(k, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (prefix(k, n, i, i + (s + t) * d) > dnode)
            s += t;
    } while (t > 1);
    const int64_t g = i + s * d + min(d, 0);
    const int64_t first = min(i, j), last = max(i, j);
    const int32_t left = first == g ? ~(int32_t)g : (int32_t)g;
    const int32_t right = last == g + 1 ? ~(int32_t)(g + 1) : (int32_t)(g + 1);
    a.kchild[2 * i] = left;
    a.kchild[2 * i + 1] = right;
    a.krange[i] = make_uint2((uint32_t)first, (uint32_t)last);
    if (left >= 0)
        a.kparent[left] = (uint32_t)i;
    else
        a.lparent[~left] = (uint32_t)i;
    if (right >= 0)
        a.kparent[right] = (uint32_t)i;
    else
        a.lparent[~right] = (uint32_t)i;
    if (i == 0)
        a.kparent[0] = kNoParent;
}

__device__ Box child_box(const BuildArgs& a, int32_t ref) {
    Box b;
    if (ref < 0)
        return object_box<false>(a.obj, object_of(a, (uint32_t)~ref));
    const float2* p = reinterpret_cast<const float2*>(a.kbox + 6 * (size_t)ref);
    const float2 x = __ldcg(p), y = __ldcg(p + 1), z = __ldcg(p + 2);
    b.lo[0] = x.x;
    b.lo[1] = x.y;
    b.lo[2] = y.x;
    b.hi[0] = y.y;
    b.hi[1] = z.x;
    b.hi[2] = z.y;
    return b;
}

// Bottom-up boxes: the second child to arrive at a node computes its box.
__global__ void radix_boxes_kernel(BuildArgs a) {
    const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= a.n)
        return;
    uint32_t p = a.lparent[leaf];
    for (int steps = 0; p != kNoParent; ++steps) {
        if (steps >= kMaxLevels) {  // deeper than the key bits allow: malformed
            atomicOr(a.state + kWordMalformed, 1u);
            return;
        }
        if (arrive_at(a.arrive + p) == 0)
            return;  // the sibling's thread computes this node
        Box b = child_box(a, a.kchild[2 * p]);
        b.grow(child_box(a, a.kchild[2 * p + 1]));
        float* o = a.kbox + 6 * (size_t)p;
        o[0] = b.lo[0];
        o[1] = b.lo[1];
        o[2] = b.lo[2];
        o[3] = b.hi[0];
        o[4] = b.hi[1];
        o[5] = b.hi[2];
        p = a.kparent[p];
    }
}

__device__ __forceinline__ uint32_t range_count(const BuildArgs& a, uint32_t node) {
    const uint2 r = a.krange[node];
    return r.y - r.x + 1;
}

__global__ void live_kernel(BuildArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n - 1)
        a.live[i] = range_count(a, i) > a.leaf ? 1u : 0u;
}

// Records in key order (leaf_end is set when the leaves are emitted).
__global__ void build_records_kernel(BuildArgs a) {
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= a.n)
        return;
    const uint32_t id = object_of(a, pos);
    igxrt_prim_record r{};
    fill_record(a.obj, id, r);
    r.prim = id;
    r.leaf_end = 0;
    r.pad = id < a.obj.nt ? kPrimTriangle : (id < a.obj.nt + a.obj.ns ? kPrimSphere : kPrimCube);
    a.prims[pos] = r;
}

__device__ __forceinline__ void put_slot2(igxrt_bvh2_node& o, int c, const Box& b, int32_t ref) {
    NodeOps<IGXRT_LAYOUT_BVH2>::put(&o, c, b);
    o.child[c] = ref;
}

// BVH2 nodes from the live internal nodes.  Sums the SAH cost (areas relative
// to the root box; node cost 1, object cost 1, as the host builder's default).
__global__ void emit2_kernel(BuildArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double sah = 0.0;
    uint32_t leaves = 0;
    if (i < a.n - 1 && a.live[i]) {
        const float pad = box_pad(a.state);
        const float root_area = child_box(a, 0).half_area();
        const float inv_root = root_area > 0.f ? 1.f / root_area : 0.f;
        const uint32_t node = a.map[i];
        igxrt_bvh2_node o{};
        sah += root_area > 0.f ? (double)child_box(a, (int32_t)i).half_area() * inv_root : 1.0;
        for (int c = 0; c < 2; ++c) {
            const int32_t ref = a.kchild[2 * i + c];
            Box b = child_box(a, ref);
            const float rel = root_area > 0.f ? b.half_area() * inv_root : 1.f;
            b.pad(pad);
            if (ref >= 0 && a.live[ref]) {
                const uint32_t child = a.map[ref];
                put_slot2(o, c, b, (int32_t)child);
                a.parents2[child] = node;
            } else {
                const uint2 r = ref >= 0 ? a.krange[ref] : make_uint2(~ref, ~ref);
                put_slot2(o, c, b, ~(int32_t)r.x);
                a.prims[r.y].leaf_end = 1;
                sah += (double)rel * (r.y - r.x + 1);
                ++leaves;
            }
        }
        a.nodes2[node] = o;
        if (i == 0) {
            a.parents2[0] = kNoParent;
            a.state[kWordNodes2] = a.map[a.n - 2] + a.live[a.n - 2];
        }
    }
    // one atomic per warp
    leaves = __reduce_add_sync(0xffffffffu, leaves);
    for (int off = 16; off > 0; off >>= 1)
        sah += __shfl_down_sync(0xffffffffu, sah, off);
    if ((threadIdx.x & 31) == 0 && leaves) {
        atomicAdd(a.state + kWordLeaves, leaves);
        atomicAdd(reinterpret_cast<double*>(a.state + kWordSah), sah);
    }
}

// Scenes of at most `leaf` objects: one root node with the whole scene in
// slot 0 (the host builder's layout for a one-leaf tree).
__global__ void emit_single_leaf_kernel(BuildArgs a) {
    const float pad = box_pad(a.state);
    Box b = a.n == 1 ? child_box(a, ~0) : child_box(a, 0);
    b.pad(pad);
    igxrt_bvh2_node o{};
    put_slot2(o, 0, b, ~0);
    Box e;
    for (int k = 0; k < 3; ++k)
        e.lo[k] = e.hi[k] = INFINITY;
    put_slot2(o, 1, e, 0);
    a.nodes2[0] = o;
    a.parents2[0] = kNoParent;
    igxrt_bvh4_node q{};
    for (int c = 0; c < 4; ++c) {
        NodeOps<IGXRT_LAYOUT_BVH4>::put(&q, c, c == 0 ? b : e);
        q.child[c] = c == 0 ? ~0 : 0;
    }
    a.nodes4[0] = q;
    a.parents4[0] = kNoParent;
    a.prims[a.n - 1].leaf_end = 1;
    a.state[kWordNodes2] = 1;
    a.state[kWordNodes4] = 1;
    a.state[kWordLeaves] = 1;
    *reinterpret_cast<double*>(a.state + kWordSah) = (double)a.n;
}

__global__ void bvh4_root_kernel(BuildArgs a) {
    a.frontier[0][0] = make_uint2(0, 0);
    a.state[kWordLevels] = 1;
    a.state[kWordNodes4] = 1;
    a.parents4[0] = kNoParent;
}

// One BVH4 level: each frontier BVH2 node becomes a BVH4 node whose slots are
// its descendants, opened largest-area-first until four slots are used.  The
// levels are chained by programmatic dependent launch: the next level's blocks
// are scheduled as soon as this one starts, and its griddepcontrol.wait
// returns once this grid has finished and its writes are visible, so the
// (mostly empty) deep levels cost no launch gap.
__global__ void emit4_level_kernel(BuildArgs a, int level) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const uint32_t count = a.state[kWordLevels + level];
    const uint2* in = a.frontier[level & 1];
    uint2* out = a.frontier[(level + 1) & 1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const uint2 job = in[t];
        Box box[4];
        int32_t ref[4];
        float area[4];
        int used = 0;
        using Ops2 = NodeOps<IGXRT_LAYOUT_BVH2>;
        float f[Ops2::kFloats];
        Ops2::load(a.nodes2 + job.x, f);
        for (int c = 0; c < 2; ++c) {
            if (Ops2::empty(f, c))
                continue;
            Ops2::get(f, c, box[used]);
            ref[used] = Ops2::child(f, c);
            area[used] = box[used].half_area();
            ++used;
        }
        while (used < 4) {
            int pick = -1;
            float best = -1.f;
            for (int s = 0; s < used; ++s)
                if (ref[s] >= 0 && area[s] > best) {
                    best = area[s];
                    pick = s;
                }
            if (pick < 0)
                break;
            Ops2::load(a.nodes2 + ref[pick], f);
            for (int s = used; s > pick + 1; --s) {  // make room after `pick`
                box[s] = box[s - 1];
                ref[s] = ref[s - 1];
                area[s] = area[s - 1];
            }
            for (int c = 0; c < 2; ++c) {
                Ops2::get(f, c, box[pick + c]);
                ref[pick + c] = Ops2::child(f, c);
                area[pick + c] = box[pick + c].half_area();
            }
            ++used;
        }
        igxrt_bvh4_node o{};
        for (int s = 0; s < 4; ++s) {
            if (s < used) {
                NodeOps<IGXRT_LAYOUT_BVH4>::put(&o, s, box[s]);
                if (ref[s] >= 0) {
                    const uint32_t child = atomicAdd(a.state + kWordNodes4, 1u);
                    a.parents4[child] = job.y;
                    out[atomicAdd(a.state + kWordLevels + level + 1, 1u)] = make_uint2((uint32_t)ref[s], child);
                    o.child[s] = (int32_t)child;
                } else {
                    o.child[s] = ref[s];
                }
            } else {
                Box e;
                for (int k = 0; k < 3; ++k)
                    e.lo[k] = e.hi[k] = INFINITY;
                NodeOps<IGXRT_LAYOUT_BVH4>::put(&o, s, e);
                o.child[s] = 0;
            }
        }
        a.nodes4[job.y] = o;
    }
}

// Exact traversal-stack bound (a node pushes its entered slots minus one) and
// depth, bottom-up through the parent links like the refit.
template <int LAYOUT>
__global__ void stack_bound_kernel(BuildArgs a, uint32_t count) {
    using Ops = NodeOps<LAYOUT>;
    using Node = typename Ops::Node;
    const Node* nodes = LAYOUT == IGXRT_LAYOUT_BVH2 ? (const Node*)a.nodes2 : (const Node*)a.nodes4;
    const uint32_t* parents = LAYOUT == IGXRT_LAYOUT_BVH2 ? a.parents2 : a.parents4;
    uint32_t node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= count || interior_children<LAYOUT>(nodes + node) != 0)
        return;
    for (int steps = 0;; ++steps) {
        if (steps > kMaxLevels) {
            atomicOr(a.state + kWordMalformed, 2u);
            return;
        }
        float f[Ops::kFloats];
        Ops::load(nodes + node, f);
        uint32_t deepest = 0, depth = 0;
        int used = 0;
        for (int c = 0; c < Ops::kSlots; ++c) {
            if (Ops::empty(f, c))
                continue;
            ++used;
            const int32_t ch = Ops::child(f, c);
            if (ch >= 0) {
                deepest = max(deepest, __ldcg(a.stack_v + ch));
                depth = max(depth, __ldcg(a.depth_v + ch));
            }
        }
        a.stack_v[node] = deepest + (used ? used - 1 : 0);
        a.depth_v[node] = depth + 1;
        const uint32_t p = parents[node];
        if (p == kNoParent) {
            a.state[LAYOUT == IGXRT_LAYOUT_BVH2 ? kWordStack2 : kWordStack4] = a.stack_v[node];
            if (LAYOUT == IGXRT_LAYOUT_BVH2)
                a.state[kWordDepth] = a.depth_v[node];
            return;
        }
        const uint32_t need = (uint32_t)interior_children<LAYOUT>(nodes + p);
        if (arrive_at(a.arrive + p) + 1u != need)
            return;
        node = p;
    }
}

struct Scratch {
    void* mem = nullptr;
    ~Scratch() {
        if (mem)
            cudaFree(mem);
    }
};

}  // namespace

extern "C" {

igxrt_status igxrt_scene_create_gpu(igxrt_context* ctx, const igxrt_scene_desc* desc,
                                    const igxrt_build_options* opts, uint32_t flags, void* stream,
                                    igxrt_scene** out) {
    if (!ctx || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!desc)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "desc is NULL");
    if (flags & ~IGXRT_TRACE_HOST_MEMORY)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown flags 0x%x", flags));
    const uint32_t leaf = (opts && opts->max_leaf_size) ? opts->max_leaf_size : kDefaultLeaf;
    if (leaf > 16)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("max_leaf_size %u outside 1..16", leaf));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    BuildArgs a{};
    igxrt_status st = stage_scene_desc(ctx, desc, flags, s, a.obj);
    if (st != IGXRT_OK)
        return st;
    const uint32_t n = a.obj.count();
    a.n = n;
    a.leaf = leaf;
    a.idbits = 1;
    while (a.idbits < 31 && (1u << a.idbits) < n)
        ++a.idbits;
    const size_t ni = std::max<size_t>(n, 2) - 1;  // internal nodes (at least one slot)
    const size_t nl = std::max<size_t>(n, 1);

    // CUB scratch sizes
    size_t sort_bytes = 0, scan_bytes = 0;
    cub::DoubleBuffer<uint64_t> keys_db(nullptr, nullptr);
    cudaError_t e = cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, keys_db, (int)nl, 0,
                                                    30 + (int)a.idbits, s);
    if (e == cudaSuccess)
        e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                          (int)ni, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "build scratch sizes");

    // one scratch allocation, 256-byte aligned parts
    std::vector<size_t> sizes = {
        kStateWords * 4, 2 * nl * 8, 2 * ni * 4, ni * 8, ni * 4, nl * 4, 6 * ni * 4, ni * 4, ni * 4,
        ni * 4, ni * sizeof(igxrt_bvh2_node), ni * sizeof(igxrt_bvh4_node), ni * 4, ni * 4,
        nl * sizeof(igxrt_prim_record), 2 * ni * 8, ni * 4, ni * 4, std::max(sort_bytes, scan_bytes)};
    std::vector<size_t> offs(sizes.size());
    size_t total = 0;
    for (size_t k = 0; k < sizes.size(); ++k) {
        offs[k] = total;
        total += round_up(std::max<size_t>(sizes[k], 1), 256);
    }
    Scratch scratch;
    e = cudaMalloc(&scratch.mem, total);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "build scratch");
    char* base = static_cast<char*>(scratch.mem);
    int part = 0;
    auto next = [&](auto* ptr) { return reinterpret_cast<decltype(ptr)>(base + offs[part++]); };
    a.state = next((uint32_t*)nullptr);
    uint64_t* keys0 = next((uint64_t*)nullptr);
    uint64_t* keys1 = keys0 + nl;
    a.kchild = next((int32_t*)nullptr);
    a.krange = next((uint2*)nullptr);
    a.kparent = next((uint32_t*)nullptr);
    a.lparent = next((uint32_t*)nullptr);
    a.kbox = next((float*)nullptr);
    a.arrive = next((uint32_t*)nullptr);
    a.live = next((uint32_t*)nullptr);
    a.map = next((uint32_t*)nullptr);
    a.nodes2 = next((igxrt_bvh2_node*)nullptr);
    a.nodes4 = next((igxrt_bvh4_node*)nullptr);
    a.parents2 = next((uint32_t*)nullptr);
    a.parents4 = next((uint32_t*)nullptr);
    a.prims = next((igxrt_prim_record*)nullptr);
    a.frontier[0] = next((uint2*)nullptr);
    a.frontier[1] = a.frontier[0] + ni;
    a.stack_v = next((uint32_t*)nullptr);
    a.depth_v = next((uint32_t*)nullptr);
    void* cub_temp = base + offs[part++];

    const uint32_t threads = 256;
    auto blocks = [threads](size_t count) { return (uint32_t)std::max<size_t>((count + threads - 1) / threads, 1); };
    e = cudaMemsetAsync(a.state, 0, kStateWords * 4, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(a.arrive, 0, ni * 4, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "build state reset");
    const uint32_t scan_grid = std::min<uint32_t>(blocks(std::max<size_t>({(size_t)n, 4 * (size_t)a.obj.np, 1})),
                                                  (uint32_t)std::max(ctx->sm_count, 1) * 4);
    build_scan_kernel<<<scan_grid, kScanBlock, 0, s>>>(a);
    if (n) {
        morton_kernel<<<blocks(n), threads, 0, s>>>(a, keys0);
        keys_db = cub::DoubleBuffer<uint64_t>(keys0, keys1);
        e = cub::DeviceRadixSort::SortKeys(cub_temp, sort_bytes, keys_db, (int)n, 0, 30 + (int)a.idbits, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "key sort");
        a.keys = keys_db.Current();
        build_records_kernel<<<blocks(n), threads, 0, s>>>(a);
    }
    if (n > 1) {
        radix_tree_kernel<<<blocks(n - 1), threads, 0, s>>>(a);
        radix_boxes_kernel<<<blocks(n), threads, 0, s>>>(a);
    }
    const bool single = n >= 1 && n <= leaf;
    if (single) {
        emit_single_leaf_kernel<<<1, 1, 0, s>>>(a);
    } else if (n > 1) {
        live_kernel<<<blocks(n - 1), threads, 0, s>>>(a);
        e = cub::DeviceScan::ExclusiveSum(cub_temp, scan_bytes, a.live, a.map, (int)(n - 1), s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "node compaction");
        emit2_kernel<<<blocks(n - 1), threads, 0, s>>>(a);
        bvh4_root_kernel<<<1, 1, 0, s>>>(a);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((uint32_t)std::max(ctx->sm_count, 1) * 4);
        cfg.blockDim = dim3(threads);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        for (int level = 0; level < kMaxLevels && e == cudaSuccess; ++level)
            e = cudaLaunchKernelEx(&cfg, emit4_level_kernel, a, level);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "BVH4 level launch");
    }
    e = cudaGetLastError();
    uint32_t w[kStateWords];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w, a.state, sizeof(w), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "GPU build");
    if (w[kWordBad])
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, non_finite_message(w[kWordBad], n));
    if (w[kWordMalformed])
        return fail(ctx, IGXRT_ERROR_INVALID_BVH, "GPU build: malformed radix tree");
    const uint32_t n2 = n ? w[kWordNodes2] : 0, n4 = n ? w[kWordNodes4] : 0;
    if (w[kWordLevels + kMaxLevels] != 0)
        return fail(ctx, IGXRT_ERROR_INVALID_BVH, "GPU build: BVH4 deeper than the level limit");
    if (n2 > ni || n4 > ni)
        return fail(ctx, IGXRT_ERROR_INVALID_BVH, "GPU build: node count out of range");

    // stack bounds and depth
    if (n) {
        e = cudaMemsetAsync(a.arrive, 0, ni * 4, s);
        if (e == cudaSuccess)
            stack_bound_kernel<IGXRT_LAYOUT_BVH2><<<blocks(n2), threads, 0, s>>>(a, n2);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(a.arrive, 0, ni * 4, s);
        if (e == cudaSuccess)
            stack_bound_kernel<IGXRT_LAYOUT_BVH4><<<blocks(n4), threads, 0, s>>>(a, n4);
        if (e == cudaSuccess)
            e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(w, a.state, sizeof(w), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "GPU build stack bounds");
        if (w[kWordMalformed])
            return fail(ctx, IGXRT_ERROR_INVALID_BVH, "GPU build: malformed tree");
    }

    igxrt_bvh_info info{};
    info.triangle_count = a.obj.nt;
    info.sphere_count = a.obj.ns;
    info.cube_count = a.obj.nc;
    info.plane_count = a.obj.np;
    info.bvh2_nodes = n2;
    info.bvh4_nodes = n4;
    info.leaf_count = n ? w[kWordLeaves] : 0;
    info.max_depth = n ? w[kWordDepth] : 0;
    info.max_leaf_size = leaf;
    double sah;
    memcpy(&sah, &w[kWordSah], 8);
    info.sah_cost = n ? (float)sah : 0.f;
    float maxabs;
    memcpy(&maxabs, &w[kWordMaxAbs], 4);
    info.pad_abs = std::max(maxabs * 0x1p-18f, 1e-30f);
    for (int k = 0; k < 3; ++k) {
        info.bounds[k] = n ? key_to_float(~w[kWordLo + k]) : 0.f;
        info.bounds[3 + k] = n ? key_to_float(w[kWordHi + k]) : 0.f;
    }
    info.max_stack[IGXRT_LAYOUT_BVH2] = n ? w[kWordStack2] : 0;
    info.max_stack[IGXRT_LAYOUT_BVH4] = n ? w[kWordStack4] : 0;
    info.device_bytes = sizeof(igxrt_bvh2_node) * (uint64_t)n2 + sizeof(igxrt_bvh4_node) * (uint64_t)n4 +
                        sizeof(igxrt_prim_record) * (uint64_t)n + sizeof(igxrt_triangle) * (uint64_t)a.obj.nt +
                        16 * (uint64_t)a.obj.np;
    for (int l = 0; l < IGXRT_LAYOUT_COUNT; ++l)
        if (info.max_stack[l] > kStackCapacity)
            return fail(ctx, IGXRT_ERROR_INVALID_BVH,
                        format("layout %d needs a %u-entry stack (limit %u)", l, info.max_stack[l],
                               kStackCapacity));

    igxrt_scene* scene = nullptr;
    if ((st = allocate_scene(ctx, info, n2, n4, 0, scene)) != IGXRT_OK)
        return st;
    auto copy = [&](const void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyDeviceToDevice, s);
    };
    copy(scene->nodes[IGXRT_LAYOUT_BVH2], a.nodes2, sizeof(igxrt_bvh2_node) * (size_t)n2);
    copy(scene->nodes[IGXRT_LAYOUT_BVH4], a.nodes4, sizeof(igxrt_bvh4_node) * (size_t)n4);
    copy(scene->parents[IGXRT_LAYOUT_BVH2], a.parents2, 4 * (size_t)n2);
    copy(scene->parents[IGXRT_LAYOUT_BVH4], a.parents4, 4 * (size_t)n4);
    copy(scene->prims, a.prims, sizeof(igxrt_prim_record) * (size_t)n);
    copy(scene->tris, a.obj.tris, sizeof(igxrt_triangle) * (size_t)a.obj.nt);
    copy(scene->planes, a.obj.planes, 16 * (size_t)a.obj.np);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        igxrt_scene_destroy(scene);
        return cuda_fail(ctx, e, "GPU build copy");
    }
    *out = scene;
    return IGXRT_OK;
}

}  // extern "C"
