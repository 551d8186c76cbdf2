// internal.h — shared host-side definitions of the ray-query engine.
#pragma once

#include <math.h>

#include <cstdint>
#include <string>
#include <vector>

#include "igxrt.h"

// Deepest BVH the kernels' traversal stacks accept (entries per ray).
// The builder keeps the binary tree's depth at or below kMaxDepth, so the
// BVH2 stack needs at most kMaxDepth entries and the BVH4 stack at most
// 3 * kMaxDepth / 2.
constexpr uint32_t kMaxDepth = 80;
constexpr uint32_t kStackCapacity = 128;

// Primitive types, the last word of a primitive record.
constexpr uint32_t kPrimTriangle = 0;
constexpr uint32_t kPrimSphere = 1;
constexpr uint32_t kPrimCube = 2;

struct igxrt_bvh {
    std::vector<igxrt_triangle> tris;
    std::vector<float> spheres;      // 4 per sphere: centre, radius
    std::vector<igxrt_cube> cubes;
    std::vector<float> planes;       // 4 per plane: normal, offset (outside the tree)
    std::vector<igxrt_bvh2_node> nodes2;
    std::vector<igxrt_bvh4_node> nodes4;
    std::vector<igxrt_bvh8_node> nodes8;
    // per BVH8 node and slot: where the slot's exact (padded) box lives in the
    // BVH2 layout, 2 * node + slot, kNoSource for an empty slot (the refit
    // re-quantizes BVH8 nodes from these boxes)
    std::vector<uint32_t> src8;
    std::vector<igxrt_prim_record> prims;
    igxrt_bvh_info info{};
};

namespace igxrt {

constexpr uint32_t kNoSource = 0xffffffffu;

#ifdef __CUDACC__
#define IGXRT_HD __host__ __device__
#else
#define IGXRT_HD
#endif
// Full unrolling in device code (keeps small fixed-size arrays in registers).
#ifdef __CUDA_ARCH__
#define IGXRT_UNROLL _Pragma("unroll")
#else
#define IGXRT_UNROLL
#endif

// BVH8 quantization, compiled for the host builder and refit and for the GPU
// refit from this one definition so both produce the same bytes.  A node's
// grid on one axis has origin = the node's lo and step 2^exp, exp the
// smallest integer in [-126, 127] whose 255 steps, decoded in binary32,
// reach the node's hi.  A slot gets the largest lo byte and the smallest hi
// byte whose decodings fmaf(q, 2^exp, origin) still enclose its box.  The
// decoding is monotone in q, byte 0 decodes to origin <= every slot's lo and
// byte 255 to at least hi, so both searches end inside [0, 255].
// The loops settle on the smallest e in [-126, 127] with
// fmaf(255, 2^e, lo) >= hi (127 if none); that predicate only strengthens as
// e grows, so the result does not depend on the starting estimate, which
// binary32 arithmetic gives within a step or two (a GPU's binary64 is slow).
IGXRT_HD inline int bvh8_exponent(float lo, float hi) {
    int k = 0;
    const float ext = hi - lo;
    if (ext > 0.f) {
        if (ext <= 3.4028235e38f)
            frexpf(ext, &k);
        else
            k = 128;
    }
    int e = k - 8 < -126 ? -126 : (k - 8 > 127 ? 127 : k - 8);
    while (e < 127 && fmaf(255.f, ldexpf(1.f, e), lo) < hi)
        ++e;
    while (e > -126 && fmaf(255.f, ldexpf(1.f, e - 1), lo) >= hi)
        --e;
    return e;
}

// The loops settle on the largest byte a whose decoding fmaf(a, 2^exp,
// origin) is at most lo and the smallest byte b whose decoding is at least hi
// (decodings grow with the byte), whatever the starting estimate; binary32
// estimates land within a step or two.
IGXRT_HD inline void bvh8_quantize(float origin, int exp, float lo, float hi, uint8_t& qlo, uint8_t& qhi) {
    const float s = ldexpf(1.f, exp);
    const float ea = floorf(ldexpf(lo - origin, -exp));
    const float eb = ceilf(ldexpf(hi - origin, -exp));
    int a = (int)(ea > 0.f ? (ea < 255.f ? ea : 255.f) : 0.f);  // NaN -> 0
    int b = (int)(eb > 0.f ? (eb < 255.f ? eb : 255.f) : 0.f);
    while (a > 0 && fmaf((float)a, s, origin) > lo)
        --a;
    while (a < 255 && fmaf((float)(a + 1), s, origin) <= lo)
        ++a;
    while (b < 255 && fmaf((float)b, s, origin) < hi)
        ++b;
    while (b > 0 && fmaf((float)(b - 1), s, origin) >= hi)
        --b;
    qlo = (uint8_t)a;
    qhi = (uint8_t)b;
}

// Origin, exponents and bytes of a BVH8 node from the exact boxes of its
// slots, which live in the BVH2 layout at src[c] = 2 * node + slot
// (kNoSource for an empty slot).  `valid` and `child` are left as they are.
IGXRT_HD inline void bvh8_quantize_node(const igxrt_bvh2_node* nodes2, const uint32_t* src,
                                        igxrt_bvh8_node& n) {
    float lo[8][3], hi[8][3];
    bool used[8];
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    IGXRT_UNROLL
    for (int c = 0; c < 8; ++c) {
        used[c] = src[c] != kNoSource;
        if (!used[c])
            continue;
        const igxrt_bvh2_node& m = nodes2[src[c] >> 1];
        const int s = (int)(src[c] & 1u);
        const float* x = s ? m.c1_x : m.c0_x;
        const float* y = s ? m.c1_y : m.c0_y;
        const float* z = s ? m.c1_z : m.c0_z;
        lo[c][0] = x[0];
        hi[c][0] = x[1];
        lo[c][1] = y[0];
        hi[c][1] = y[1];
        lo[c][2] = z[0];
        hi[c][2] = z[1];
        IGXRT_UNROLL
        for (int a = 0; a < 3; ++a) {
            nlo[a] = lo[c][a] < nlo[a] ? lo[c][a] : nlo[a];
            nhi[a] = nhi[a] < hi[c][a] ? hi[c][a] : nhi[a];
        }
    }
    IGXRT_UNROLL
    for (int a = 0; a < 3; ++a) {
        const int e = bvh8_exponent(nlo[a], nhi[a]);
        n.origin[a] = nlo[a];
        n.exp[a] = (int8_t)e;
        uint8_t* qlo = a == 0 ? n.lo_x : (a == 1 ? n.lo_y : n.lo_z);
        uint8_t* qhi = a == 0 ? n.hi_x : (a == 1 ? n.hi_y : n.hi_z);
        IGXRT_UNROLL
        for (int c = 0; c < 8; ++c) {
            if (used[c])
                bvh8_quantize(nlo[a], e, lo[c][a], hi[c][a], qlo[c], qhi[c]);
            else
                qlo[c] = qhi[c] = 0;
        }
    }
}

// Thread-safe formatted message helper.
std::string format(const char* fmt, ...);

// Builds `out` from the triangles (host only).
igxrt_status build_bvh(const igxrt_triangle* tris, uint32_t count,
                       const igxrt_build_options* opts, igxrt_bvh& out, std::string& err);
// Builds `out` from all primitive buffers of a scene (host only).
igxrt_status build_bvh_mixed(const igxrt_scene_desc& d, const igxrt_build_options* opts,
                             igxrt_bvh& out, std::string& err);

// New primitive positions for a built tree: same topology and record order,
// every box recomputed with the builder's padding rule (host only).
igxrt_status refit_bvh(igxrt_bvh& bvh, const igxrt_scene_desc& d, std::string& err);

// Structural validation; returns IGXRT_OK or IGXRT_ERROR_INVALID_BVH with msg.
igxrt_status validate_bvh(const igxrt_bvh& bvh, std::string& msg);

}  // namespace igxrt
