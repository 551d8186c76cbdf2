// geometry.cuh — device helpers shared by the GPU refit and the GPU build:
// object bounds by the host builder's rule, the scan that reduces them, and
// per-layout access to node slots.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include "engine.h"

namespace igxrt {

// The scene's primitive buffers as the kernels read them (device pointers).
struct SceneObjects {
    const igxrt_triangle* tris;
    const float* spheres;  // (centre, radius) per sphere
    const igxrt_cube* cubes;
    const float* planes;   // (n, d) per plane
    uint32_t nt, ns, nc, np;
    __host__ __device__ uint32_t count() const { return nt + ns + nc; }  // objects in the tree
};

// Device view of a scene description: host arrays (IGXRT_TRACE_HOST_MEMORY)
// are copied into the context's staging buffer on `s`; device arrays are
// checked and used in place.
igxrt_status stage_scene_desc(igxrt_context* ctx, const igxrt_scene_desc* desc, uint32_t flags,
                              cudaStream_t s, SceneObjects& o);
// The error message for the scan's non-finite state word.
std::string non_finite_message(uint32_t bad_word, uint32_t objects);

// std::min / std::max of the host builder, argument order included.
__device__ __forceinline__ float host_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float host_max(float a, float b) { return (a < b) ? b : a; }

// Arrival at a parent in a bottom-up climb: an acquire-release add at GPU
// scope, so this thread's writes are visible before the count moves, and the
// thread that sees the last arrival sees every sibling's writes.  Returns the
// count before the add.
__device__ __forceinline__ uint32_t arrive_at(uint32_t* counter) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(counter) : "memory");
    return old;
}

// Order-preserving map of a float to an unsigned word (for atomicMax/Min).
__device__ __forceinline__ uint32_t order_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

inline float key_to_float(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
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
    __device__ void pad(float p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = __fsub_rn(lo[k], p);
            hi[k] = __fadd_rn(hi[k], p);
        }
    }
    __device__ float half_area() const {
        if (!(hi[0] >= lo[0]))
            return 0.f;
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
};

// Object bounds by the builder's rule over the points it bounds: triangle
// vertices; sphere centre -/+ |radius|; cube start and end corners.  With
// CHECK, `finite` and `maxabs` cover the same points.
template <bool CHECK>
__device__ Box object_box(const SceneObjects& o, uint32_t id, bool* finite = nullptr,
                          float* maxabs = nullptr) {
    float v[3][3];
    int nv;
    if (id < o.nt) {
        const igxrt_triangle& t = o.tris[id];
        for (int k = 0; k < 3; ++k) {
            v[0][k] = t.p0[k];
            v[1][k] = t.p1[k];
            v[2][k] = t.p2[k];
        }
        nv = 3;
    } else if (id < o.nt + o.ns) {
        const float* s = o.spheres + 4 * (size_t)(id - o.nt);
        const float r = fabsf(s[3]);
        for (int k = 0; k < 3; ++k) {
            v[0][k] = __fsub_rn(s[k], r);
            v[1][k] = __fadd_rn(s[k], r);
        }
        nv = 2;
    } else {
        const igxrt_cube& c = o.cubes[id - o.nt - o.ns];
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

// The geometry fields of object `id`'s record, as the host builder writes
// them: triangle p0, e1 = p1 - p0, e2 = p2 - p0; sphere centre and radius;
// cube start and end corners.  Other fields are left as they are.
__device__ __forceinline__ void fill_record(const SceneObjects& o, uint32_t id, igxrt_prim_record& r) {
    if (id < o.nt) {
        const igxrt_triangle& t = o.tris[id];
        for (int k = 0; k < 3; ++k) {
            r.p0[k] = t.p0[k];
            r.e1[k] = __fsub_rn(t.p1[k], t.p0[k]);
            r.e2[k] = __fsub_rn(t.p2[k], t.p0[k]);
        }
    } else if (id < o.nt + o.ns) {
        const float* s = o.spheres + 4 * (size_t)(id - o.nt);
        for (int k = 0; k < 3; ++k)
            r.p0[k] = s[k];
        r.e1[0] = s[3];
    } else {
        const igxrt_cube& c = o.cubes[id - o.nt - o.ns];
        r.p0[0] = c.xy0[0];
        r.p0[1] = c.xy0[1];
        r.p0[2] = c.z0_x1[0];
        r.e1[0] = c.z0_x1[1];
        r.e1[1] = c.yz1[0];
        r.e1[2] = c.yz1[1];
    }
}

// Scan state words, all reduced with atomicMax from zero:
//   0        max |coordinate| as float bits (non-negative floats order as words)
//   1..3     ~order_key(scene lo) per axis
//   4..6     order_key(scene hi) per axis
//   7        ~(first object or plane with a non-finite value), 0 when none
//   8..10    ~order_key(centroid lo) per axis   (with centroids only)
//   11..13   order_key(centroid hi) per axis
constexpr int kWordMaxAbs = 0, kWordLo = 1, kWordHi = 4, kWordBad = 7, kWordCenLo = 8,
              kWordCenHi = 11;
constexpr int kScanBlock = 256;

// Grid-stride scan of every object (and plane), one block reduction, then
// one atomicMax per block and word.  Call from all threads of a kScanBlock
// block.
template <bool CENTROIDS>
__device__ void scan_objects(const SceneObjects& o, uint32_t* state) {
    constexpr int W = CENTROIDS ? 14 : 8;
    uint32_t w[W];
    for (int k = 0; k < W; ++k)
        w[k] = 0;
    const uint32_t n = o.count();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += stride) {
        bool finite = true;
        float m = 0.f;
        const Box b = object_box<true>(o, id, &finite, &m);
        if (!finite) {
            w[kWordBad] = max(w[kWordBad], ~id);
            continue;
        }
        w[kWordMaxAbs] = max(w[kWordMaxAbs], __float_as_uint(m));
        for (int k = 0; k < 3; ++k) {
            w[kWordLo + k] = max(w[kWordLo + k], ~order_key(b.lo[k]));
            w[kWordHi + k] = max(w[kWordHi + k], order_key(b.hi[k]));
            if (CENTROIDS) {
                const float c = __fmul_rn(__fadd_rn(b.lo[k], b.hi[k]), 0.5f);
                w[kWordCenLo + k] = max(w[kWordCenLo + k], ~order_key(c));
                w[kWordCenHi + k] = max(w[kWordCenHi + k], order_key(c));
            }
        }
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * o.np; i += stride)
        if (!isfinite(o.planes[i]))
            w[kWordBad] = max(w[kWordBad], ~(n + i / 4));
    __shared__ uint32_t red[kScanBlock / 32][W];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int k = 0; k < W; ++k) {
        const uint32_t v = __reduce_max_sync(0xffffffffu, w[k]);
        if (lane == 0)
            red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < W) {
        uint32_t v = 0;
        for (int i = 0; i < kScanBlock / 32; ++i)
            v = max(v, red[i][threadIdx.x]);
        if (v)
            atomicMax(state + threadIdx.x, v);
    }
}

// The padding of every box: max(2^-18 * max|coordinate|, 1e-30).
__device__ __forceinline__ float box_pad(const uint32_t* state) {
    return fmaxf(__fmul_rn(__uint_as_float(state[kWordMaxAbs]), 0x1p-18f), 1e-30f);
}

// Node access per layout: slot boxes, child refs and empty slots.  Loads go
// through L2 (ld.global.cg): another SM may have written the node in the
// same launch.
template <int LAYOUT>
struct NodeOps;

template <>
struct NodeOps<IGXRT_LAYOUT_BVH2> {
    static constexpr int kSlots = 2;
    static constexpr int kFloats = 16;
    using Node = igxrt_bvh2_node;
    __device__ static void load(const Node* p, float (&f)[kFloats]) {
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
    __device__ static bool empty(const float (&f)[kFloats], int c) {
        return f[4 * c] == INFINITY && f[4 * c + 1] == INFINITY;
    }
    __device__ static int32_t child(const float (&f)[kFloats], int c) { return __float_as_int(f[12 + c]); }
    __device__ static void get(const float (&f)[kFloats], int c, Box& b) {
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
    static constexpr int kFloats = 32;
    using Node = igxrt_bvh4_node;
    __device__ static void load(const Node* p, float (&f)[kFloats]) {
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
    __device__ static bool empty(const float (&f)[kFloats], int c) {
        return f[c] == INFINITY && f[4 + c] == INFINITY;
    }
    __device__ static int32_t child(const float (&f)[kFloats], int c) { return __float_as_int(f[24 + c]); }
    __device__ static void get(const float (&f)[kFloats], int c, Box& b) {
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
    float f[Ops::kFloats];
    Ops::load(node, f);
    int k = 0;
    for (int c = 0; c < Ops::kSlots; ++c)
        k += (!Ops::empty(f, c) && Ops::child(f, c) >= 0) ? 1 : 0;
    return k;
}

}  // namespace igxrt
