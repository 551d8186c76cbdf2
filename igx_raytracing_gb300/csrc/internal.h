// internal.h — shared host-side definitions of the ray-query engine.
#pragma once

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
    std::vector<igxrt_prim_record> prims;
    igxrt_bvh_info info{};
};

namespace igxrt {

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
