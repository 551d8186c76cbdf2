/*
 * oracle.h — CPU restatement of igx_raytracing's ray-query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA engine is
 * tested against, and the timed CPU baseline; the engine never links, loads or calls
 * it.  Only the test suite, the smoke check and the benchmark's CPU-baseline
 * leg use it.
 *
 * Two parts:
 *  - orc_trace_geometry / orc_trace_occlusion: brute-force loops over every
 *    triangle in index order, restating traceGeometry / traceOcclusion
 *    (res/shaders/trace.glsl:9-66, 70-98) around rayIntersectTri
 *    (res/shaders/primitive.glsl:239-284) in IEEE binary32 with no FMA
 *    contraction.  These define the expected results.
 *  - orc_bvh_trace: the same triangle test driven by a traversal of the
 *    engine's exported BVH (the layouts in include/igxrt.h), visiting nodes in
 *    the order the CUDA kernels do.  It is the multi-threaded CPU baseline and
 *    counts node and primitive records fetched per ray (the roofline's bytes).
 */
#ifndef IGXRT_ORACLE_H
#define IGXRT_ORACLE_H

#include <stdint.h>
#include "igxrt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-ray event flags reported by the brute-force loops. */
#define ORC_EVENT_NAN_T 1u    /* a NaN t was accepted: the linear loop's later
                                 decisions then depend on index order alone */
#define ORC_EVENT_ZERO_DET 2u /* a == 0 for a triangle whose u, v tests passed */

/* Brute-force closest hit.  flags may be NULL.  threads <= 0: all cores. */
void orc_trace_geometry(const igxrt_triangle* tris, uint32_t ntri,
                        const igxrt_ray* rays, const uint32_t* prev_hit,
                        uint32_t nrays, igxrt_hit* out, uint32_t* flags,
                        int threads);

/* Brute-force occlusion: out[i] = traceOcclusion(ray, rays[i].tmax, prev). */
void orc_trace_occlusion(const igxrt_triangle* tris, uint32_t ntri,
                         const igxrt_ray* rays, const uint32_t* prev_hit,
                         uint32_t nrays, uint32_t* out, uint32_t* flags,
                         int threads);

/* Closest hit of one ray against one triangle in binary64, for logging
 * disagreements: returns 1 and fills t,u,v if the exact-arithmetic-style
 * test (same formulas, double precision) accepts. */
int orc_reintersect_f64(const igxrt_ray* ray, const igxrt_triangle* tri,
                        double* t, double* u, double* v);

/*
 * BVH traversal on the CPU.  layout = IGXRT_LAYOUT_BVH2, _BVH4 or _BVH8; nodes and
 * prims as returned by igxrt_bvh_get_data.  mode 0 = closest (out_hits),
 * mode 1 = any (out_occluded).  node_fetches / prim_fetches may be NULL.
 * Returns 0, or -1 on a malformed BVH (stack overflow / bad index).
 */
int orc_bvh_trace(uint32_t layout, const void* nodes, uint64_t node_count,
                  const igxrt_prim_record* prims, uint64_t prim_count,
                  const igxrt_ray* rays, const uint32_t* prev_hit, uint32_t nrays,
                  uint32_t mode, igxrt_hit* out_hits, uint32_t* out_occluded,
                  uint32_t* node_fetches, uint32_t* prim_fetches, int threads);

/*
 * The shadow pass of res/shaders/nv_all.shadow.comp:50-142 on the NVIDIA
 * subgroup layout: per pixel (x, y) and sample s with object != noRayHit,
 * traceOcclusion(ray, ray.tmax, object) by brute force; the results are
 * ballot-packed into words indexToLight(loc, res, s, (4,1), (15,1))
 * (res/shaders/light.glsl:221-229), bit (x & 15) | ((y & 1) << 4).  Every
 * word is written (0 where no pixel is occluded).  flags as for
 * orc_trace_occlusion, per ray (may be NULL).
 */
void orc_shadow_mask(const igxrt_triangle* tris, uint32_t ntri, const igxrt_ray* rays,
                     const uint32_t* object, uint32_t width, uint32_t height, uint32_t samples,
                     uint32_t* mask, uint32_t* flags, int threads);

/*
 * The primary pass of res/shaders/raygen.comp:16-52 (default projection):
 * calculateScreen's ray per pixel (camera.glsl:72-87, 113-116), brute-force
 * traceGeometry, and the shader's two rgba32f outputs (dir_object, uv_normal:
 * width*height*4 floats each, row-major; uv_normal untouched on a miss).
 * flags per pixel as for orc_trace_geometry (may be NULL).
 */
void orc_gbuffer(const igxrt_triangle* tris, uint32_t ntri, const igxrt_camera* cam,
                 float* dir_object, float* uv_normal, uint32_t* flags, int threads);

/* decodeSpheremap (primitive.glsl:95-104) and encodeNormal (:85-88). */
void orc_decode_spheremap(uint32_t n, float out[3]);
void orc_encode_normal(const float n[3], uint32_t out[2]);

/*
 * traceGeometry / traceOcclusion over all primitive buffers of a scene
 * (res/shaders/trace.glsl:22-46, 77-95): triangles, spheres, cubes and planes
 * in global index order with rayIntersectTri / Sphere / Cube / Plane
 * (primitive.glsl:173-333), brute force.  `tmin` of each ray generalises the
 * reference's zero bound as the engine does (t > tmin for triangles,
 * hitT >= tmin for spheres and planes, tmax >= tmin for cubes).
 */
void orc_trace_geometry_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays,
                              const uint32_t* prev_hit, uint32_t nrays, igxrt_hit* out,
                              uint32_t* flags, int threads);
void orc_trace_occlusion_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays,
                               const uint32_t* prev_hit, uint32_t nrays, uint32_t* out,
                               uint32_t* flags, int threads);

/*
 * The oracle's own BVH over `ntri` triangles (bvh_build_oracle.c: binned SAH,
 * leaves of at most 4 triangles, boxes padded outward) in the BVH2 node and
 * primitive-record formats orc_bvh_trace reads, so the CPU reference arm
 * traces without the engine's builder.  nodes must hold max(1, ntri) nodes and
 * prims ntri records.  Returns the node count (0 for no triangles), or -1 when
 * memory runs out.
 */
int64_t orc_bvh_build(const igxrt_triangle* tris, uint32_t ntri, igxrt_bvh2_node* nodes,
                      igxrt_prim_record* prims);

/* The primary rays orc_gbuffer traces, width*height records in pixel order
 * ({eye, 0, dir, IGXRT_NO_HIT}). */
void orc_camera_rays(const igxrt_camera* cam, igxrt_ray* rays);

/* orc_gbuffer / orc_shadow_mask over every primitive buffer of a mixed scene
 * (trace.glsl:22-46 order).  The G-buffer's object normal of a sphere, cube
 * or plane hit is its geometry normal (trace.glsl:59-63). */
void orc_gbuffer_mixed(const igxrt_scene_desc* scene, const igxrt_camera* cam, float* dir_object,
                       float* uv_normal, uint32_t* flags, int threads);
void orc_shadow_mask_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays, const uint32_t* object,
                           uint32_t width, uint32_t height, uint32_t samples, uint32_t* mask,
                           uint32_t* flags, int threads);

/* Number of hardware threads the oracle uses for threads <= 0. */
int orc_hardware_threads(void);

#ifdef __cplusplus
}
#endif

#endif
