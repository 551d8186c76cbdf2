// gbuffer.cuh — pieces of the reference's primary pass (raygen.comp) for
// the G-buffer kernel (gbuffer.cu): the camera ray of a pixel, the pixel
// order of the 8x4 tiles and the two output encodings of a triangle hit.
//
// Every step follows the shader's binary32 expression order with separately
// rounded operations: the screen mapping of calculateScreen
// (res/shaders/camera.glsl:72-87, 113-116), the hit encoding of
// raygen.comp:39-51, decodeSpheremap / interpolate / encodeNormal
// (res/shaders/primitive.glsl:85-104, 146-151) for the vertex normal of
// trace.glsl:48-57.
#pragma once

#include <cuda_fp16.h>

#include "engine.h"
#include "traverse.cuh"

namespace igxrt {

// The camera and the two images of a G-buffer pass.
struct GbufferSink {
    const igxrt_triangle* tris;
    igxrt_camera cam;
    float inv_w, inv_h;
    uint32_t tiles_x;
    float4* dir_object;
    float4* uv_normal;
};

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// decodeSpheremap, primitive.glsl:95-104.
__device__ __forceinline__ float3 decode_spheremap(uint32_t n) {
    const float x = __half2float(__ushort_as_half((unsigned short)(n & 0xffffu)));
    const float y = __half2float(__ushort_as_half((unsigned short)(n >> 16)));
    // l = dot(vec3(nn, 1), -vec3(nn, -1))
    const float l = dot3(x, y, 1.0f, -x, -y, 1.0f);
    const float s = __fsqrt_rn(l);
    const float sx = __fmul_rn(x, s), sy = __fmul_rn(y, s);
    // vec3(nn, l) * 2 + vec3(0, 0, -1)
    return make_float3(__fadd_rn(__fmul_rn(sx, 2.0f), 0.0f), __fadd_rn(__fmul_rn(sy, 2.0f), 0.0f),
                       __fadd_rn(__fmul_rn(l, 2.0f), -1.0f));
}

// encodeNormal, primitive.glsl:85-88.
__device__ __forceinline__ uint2 encode_normal(float3 n) {
    const float len = __fsqrt_rn(dot3(n.x, n.y, n.z, n.x, n.y, n.z));
    const float qx = __fdiv_rn(n.x, len), qy = __fdiv_rn(n.y, len), qz = __fdiv_rn(n.z, len);
    const uint32_t hx = __float2uint_rz(__fmul_rn(__fadd_rn(__fmul_rn(qx, 0.5f), 0.5f), 65535.0f));
    const uint32_t hy = __float2uint_rz(__fmul_rn(__fadd_rn(__fmul_rn(qy, 0.5f), 0.5f), 65535.0f));
    const uint32_t hz = __float2uint_rz(__fmul_rn(__fadd_rn(__fmul_rn(qz, 0.5f), 0.5f), 65535.0f));
    return make_uint2((hx << 16) | hy, hz);
}

// calculatePrimary / calculateScreen (camera.glsl:72-87, 113-116): the unit
// direction of pixel (x, y), every operation rounded separately.
__device__ __forceinline__ float3 camera_dir(const igxrt_camera& c, float inv_w, float inv_h, uint32_t x,
                                             uint32_t y) {
    const float cx = __fmul_rn(__fadd_rn((float)x, c.jitter_x), inv_w);
    const float cy = __fsub_rn(1.0f, __fmul_rn(__fadd_rn((float)y, c.jitter_y), inv_h));
    float d[3];
    for (int k = 0; k < 3; ++k) {
        const float right = __fsub_rn(c.p1[k], c.p0[k]), up = __fsub_rn(c.p2[k], c.p0[k]);
        const float pos = __fadd_rn(__fadd_rn(c.p0[k], __fmul_rn(cx, right)), __fmul_rn(cy, up));
        d[k] = __fsub_rn(pos, c.eye[k]);
    }
    const float len = __fsqrt_rn(dot3(d[0], d[1], d[2], d[0], d[1], d[2]));
    return make_float3(__fdiv_rn(d[0], len), __fdiv_rn(d[1], len), __fdiv_rn(d[2], len));
}

// The traversal state of a primary ray: from the eye along `dir`, tmin 0,
// no tmax (raygen.comp's ray), no previous hit.
__device__ __forceinline__ RayState camera_ray_state(const igxrt_camera& c, float3 dir) {
    RayState r;
    r.ox = c.eye[0];
    r.oy = c.eye[1];
    r.oz = c.eye[2];
    r.dx = dir.x;
    r.dy = dir.y;
    r.dz = dir.z;
    r.ix = __frcp_rn(safe_dir(dir.x));
    r.iy = __frcp_rn(safe_dir(dir.y));
    r.iz = __frcp_rn(safe_dir(dir.z));
    r.oix = __fmul_rn(r.ox, r.ix);
    r.oiy = __fmul_rn(r.oy, r.iy);
    r.oiz = __fmul_rn(r.oz, r.iz);
    r.tmin = 0.f;
    r.tmin_box = 0.f;
    r.tmax_eff = IGXRT_NO_HIT;
    r.prev = IGXRT_NO_RAY_HIT;
    return r;
}

// Pixel of tile-ordered index i: 8x4 tiles, row-major over the image, 32
// consecutive indices per tile (lane k of a tile at (k & 7, k >> 3)).
// False for the padding of the right and bottom tiles.
__device__ __forceinline__ bool gbuffer_pixel(const GbufferSink& g, uint32_t i, uint32_t& x, uint32_t& y) {
    const uint32_t t = i >> 5, k = i & 31u;
    const uint32_t ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
    x = tx * 8u + (k & 7u);
    y = ty * 4u + (k >> 3);
    return x < g.cam.width && y < g.cam.height;
}

// raygen.comp:39-51 for a triangle scene: on a hit dir * hitT and the
// object, then the barycentrics and the interpolated vertex normal through
// encodeNormal; on a miss the direction and noRayHit (uv_normal untouched).
__device__ __forceinline__ void write_gbuffer_triangle(const GbufferSink& g, size_t px, float dx, float dy,
                                                       float dz, const BestHit& best, bool hit) {
    if (!hit) {
        g.dir_object[px] = make_float4(dx, dy, dz, __uint_as_float(IGXRT_NO_RAY_HIT));
        return;
    }
    const uint32_t object = best.prim;
    g.dir_object[px] = make_float4(__fmul_rn(dx, best.t), __fmul_rn(dy, best.t), __fmul_rn(dz, best.t),
                                   __uint_as_float(object));
    const igxrt_triangle& t = g.tris[object];
    const float3 n0 = decode_spheremap(t.n0), n1 = decode_spheremap(t.n1), n2 = decode_spheremap(t.n2);
    // interpolate(n0, n1, n2, uv): (u*n1 + v*n2) + (1 - u - v)*n0
    const float u = best.u, v = best.v, bw = __fsub_rn(__fsub_rn(1.0f, u), v);
    const float3 n = make_float3(
        __fadd_rn(__fadd_rn(__fmul_rn(u, n1.x), __fmul_rn(v, n2.x)), __fmul_rn(bw, n0.x)),
        __fadd_rn(__fadd_rn(__fmul_rn(u, n1.y), __fmul_rn(v, n2.y)), __fmul_rn(bw, n0.y)),
        __fadd_rn(__fadd_rn(__fmul_rn(u, n1.z), __fmul_rn(v, n2.z)), __fmul_rn(bw, n0.z)));
    const uint2 e = encode_normal(n);
    g.uv_normal[px] = make_float4(u, v, __uint_as_float(e.x), __uint_as_float(e.y));
}

}  // namespace igxrt
