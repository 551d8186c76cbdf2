// gbuffer.cu — the reference's primary pass (raygen.comp): primary-ray
// generation, closest hit and the shader's two output encodings (gbuffer.cuh
// has the pieces and their reference lines).
//
// Two forms, the same images bit for bit.  Triangle scenes whose images are
// in device memory (or staged through it) trace the camera's rays with the
// persistent trace kernel (trace_kernels.cu, rays made in the kernel), which
// leaves each pixel's hit record in dir_object; an encoding kernel then turns
// the records into the two images, one thread per pixel.  Mixed scenes (a
// sphere, cube or plane hit's object normal is its geometry normal,
// trace.glsl:59-63) and host images written in place use the tile kernel:
// a warp per 8x4 tile, its pixels traced together and written together (four
// 128-byte row segments, which cross NVLink-C2C as whole lines where single
// pixels finishing one at a time would not).
#include <algorithm>

#include "engine.h"
#include "gbuffer.cuh"
#include "traverse.cuh"

namespace igxrt {

struct GbufferArgs {
    const float4* nodes;
    const float4* prims;
    uint32_t node_count;
    uint32_t tri_count;       // mixed scenes: objects below this id are triangles
    const float4* planes;     // mixed scenes: planes outside the tree
    uint32_t plane_count;
    uint32_t plane_base;
    GbufferSink g;            // camera, triangles and the two images
    uint32_t tiles;
    uint32_t* status;
    uint32_t sh_depth;
    uint32_t phase_break;  // node_phase's early end (igxrt_launch_params.phase_break)
};

// The primary rays of igxrt_trace_gbuffer as records: {eye, 0, dir, noHit}.
__global__ void camera_rays_kernel(igxrt_camera c, float inv_w, float inv_h, float4* rays) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)c.width * c.height)
        return;
    const uint32_t y = (uint32_t)(i / c.width), x = (uint32_t)(i - (uint64_t)y * c.width);
    const float3 d = camera_dir(c, inv_w, inv_h, x, y);
    rays[2 * i] = make_float4(c.eye[0], c.eye[1], c.eye[2], 0.f);
    rays[2 * i + 1] = make_float4(d.x, d.y, d.z, IGXRT_NO_HIT);
}

// geometryNormal of a non-triangle hit (primitive.glsl:190-192, 223, 311-327),
// recomputed from the hit's record (or plane) with the shader's operations:
// a sphere's normalize(centre - o) at o = hitT * dir + pos; a cube's axis
// normal, +1 when the entry plane is the start plane; a plane's
// normalize(n), negated when the ray runs along it (dif > 0).
__device__ __forceinline__ float3 mixed_geometry_normal(const RayState& r, const float4* __restrict__ prims,
                                                        const float4* __restrict__ planes, uint32_t rec,
                                                        float t) {
    if (rec & kRecPlane) {
        const float4 pl = __ldg(planes + (rec & ~kRecPlane));
        const float len = __fsqrt_rn(dot3(pl.x, pl.y, pl.z, pl.x, pl.y, pl.z));
        const float nx = __fdiv_rn(pl.x, len), ny = __fdiv_rn(pl.y, len), nz = __fdiv_rn(pl.z, len);
        const float dif = dot3(r.dx, r.dy, r.dz, -nx, -ny, -nz);
        return dif > 0.f ? make_float3(-nx, -ny, -nz) : make_float3(nx, ny, nz);
    }
    const float4* p = prims + 3 * (size_t)rec;
    const float4 v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2);
    if (__float_as_uint(v2.w) == kPrimSphere) {
        const float ox = __fadd_rn(__fmul_rn(t, r.dx), r.ox), oy = __fadd_rn(__fmul_rn(t, r.dy), r.oy),
                    oz = __fadd_rn(__fmul_rn(t, r.dz), r.oz);
        const float nx = __fsub_rn(v0.x, ox), ny = __fsub_rn(v0.y, oy), nz = __fsub_rn(v0.z, oz);
        const float len = __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz));
        return make_float3(__fdiv_rn(nx, len), __fdiv_rn(ny, len), __fdiv_rn(nz, len));
    }
    // cube {start, id}{end, leaf_end}: the entry distances of cube_hit
    const float rx = __frcp_rn(r.dx), ry = __frcp_rn(r.dy), rz = __frcp_rn(r.dz);
    const float sx = __fmul_rn(__fsub_rn(v0.x, r.ox), rx), sy = __fmul_rn(__fsub_rn(v0.y, r.oy), ry),
                sz = __fmul_rn(__fsub_rn(v0.z, r.oz), rz);
    const float ex = __fmul_rn(__fsub_rn(v1.x, r.ox), rx), ey = __fmul_rn(__fsub_rn(v1.y, r.oy), ry),
                ez = __fmul_rn(__fsub_rn(v1.z, r.oz), rz);
    const float mix = gmin(sx, ex), miy = gmin(sy, ey), miz = gmin(sz, ez);
    const float tmin = gmax(gmax(mix, miy), miz);
    if (tmin == mix)
        return make_float3(mix == sx ? 1.f : -1.f, 0.f, 0.f);
    if (tmin == miy)
        return make_float3(0.f, miy == sy ? 1.f : -1.f, 0.f);
    return make_float3(0.f, 0.f, miz == sz ? 1.f : -1.f);
}

// MIXED: scenes with spheres, cubes and planes; the object normal of a
// non-triangle hit is its geometry normal (trace.glsl:59-63).
template <int LAYOUT, bool MIXED>
__global__ void __launch_bounds__(256) gbuffer_kernel(GbufferArgs a) {
    extern __shared__ uint32_t smem[];
    TraversalStack st;
    st.sh = reinterpret_cast<uint2*>(smem) + threadIdx.x;
    st.stride = blockDim.x;
    st.sh_depth = a.sh_depth;
    st.sp = 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const GbufferSink& g = a.g;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < a.tiles; w += warps) {
        // tile w's pixel of this lane (gbuffer_pixel's order, 32 indices per tile);
        // the tile's pixels inside the image trace together (trace_warp), the
        // lanes outside it take part in the warp's ballots only
        uint32_t x, y;
        const bool inside = gbuffer_pixel(g, w * 32u + lane, x, y);
        const RayState r = camera_ray_state(g.cam, camera_dir(g.cam, g.inv_w, g.inv_h, inside ? x : 0u,
                                                              inside ? y : 0u));
        BestHit best;
        bool overflow = false;
        uint32_t rec = 0;
        const uint32_t gave_up = trace_warp<LAYOUT, MIXED>(a.nodes, a.prims, a.node_count, a.planes,
                                                           a.plane_count, a.plane_base, inside, a.phase_break, r,
                                                           best, st, overflow, rec);
        if (overflow)
            atomicOr(a.status, kStatusStackOverflow);
        if (gave_up && lane == 0)
            atomicOr(a.status, gave_up);
        if (!inside)
            continue;
        const size_t px = (size_t)y * g.cam.width + x;
        // raygen.comp:39-44: a miss is hitT == noHit
        const bool hit = best.t < IGXRT_NO_HIT;
        if (MIXED && hit && id_of_prio(best.prim) >= a.tri_count) {
            const uint32_t object = id_of_prio(best.prim);
            g.dir_object[px] = make_float4(__fmul_rn(r.dx, best.t), __fmul_rn(r.dy, best.t),
                                           __fmul_rn(r.dz, best.t), __uint_as_float(object));
            const uint2 e = encode_normal(mixed_geometry_normal(r, a.prims, a.planes, rec, best.t));
            g.uv_normal[px] = make_float4(best.u, best.v, __uint_as_float(e.x), __uint_as_float(e.y));
            continue;
        }
        BestHit tri = best;
        if (MIXED)
            tri.prim = id_of_prio(best.prim);
        write_gbuffer_triangle(g, px, r.dx, r.dy, r.dz, tri, hit);
    }
}

// After the camera-ray trace: pixel i's hit record {t, u, v, prim} (the
// trace kernel's output, written into dir_object) becomes its two images.
// The direction is the camera's again (camera_dir, the trace's own rays).
__global__ void __launch_bounds__(256) gbuffer_encode_kernel(GbufferSink g, uint32_t pixels) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pixels)
        return;
    const float4 h = g.dir_object[i];
    const uint32_t y = i / g.cam.width, x = i - y * g.cam.width;
    const float3 d = camera_dir(g.cam, g.inv_w, g.inv_h, x, y);
    BestHit best;
    best.t = h.x;
    best.u = h.y;
    best.v = h.z;
    best.prim = __float_as_uint(h.w);
    write_gbuffer_triangle(g, i, d.x, d.y, d.z, best, best.prim != IGXRT_NO_RAY_HIT);
}

// The tile kernel: a warp per 8x4 tile, a grid of at most the resident
// CTAs striding over the tiles.
igxrt_status launch_tiles(igxrt_context* ctx, const igxrt_scene* scene, const igxrt_launch_params& p,
                          GbufferArgs& a, cudaStream_t stream) {
    a.nodes = reinterpret_cast<const float4*>(scene->nodes[p.layout]);
    a.prims = reinterpret_cast<const float4*>(scene->prims);
    a.node_count = scene->node_count[p.layout];
    a.tri_count = scene->info.triangle_count;
    a.planes = reinterpret_cast<const float4*>(scene->planes);
    a.plane_count = scene->plane_count;
    a.plane_base = scene->plane_base;
    a.status = status_word(ctx);
    a.sh_depth = p.stack_depth;
    a.phase_break = p.phase_break;
    constexpr int B2 = IGXRT_LAYOUT_BVH2, B4 = IGXRT_LAYOUT_BVH4, B8 = IGXRT_LAYOUT_BVH8;
    auto fn = scene->mixed ? (p.layout == B8 ? gbuffer_kernel<B8, true>
                              : p.layout == B4 ? gbuffer_kernel<B4, true> : gbuffer_kernel<B2, true>)
                           : (p.layout == B8 ? gbuffer_kernel<B8, false>
                              : p.layout == B4 ? gbuffer_kernel<B4, false> : gbuffer_kernel<B2, false>);
    const size_t smem = (size_t)p.stack_depth * p.block_size * kStackEntryBytes;
    int per_sm = 0;
    cudaError_t e = allow_smem((const void*)fn, smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)p.block_size, smem);
    if (e != cudaSuccess || per_sm < 1)
        return e != cudaSuccess ? cuda_fail(ctx, e, "occupancy query")
                                : fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "no resident CTA");
    const uint64_t wpb = p.block_size / 32;
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, (a.tiles + wpb - 1) / wpb));
    fn<<<grid, p.block_size, smem, stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "g-buffer kernel launch");
    return IGXRT_OK;
}

}  // namespace igxrt

using namespace igxrt;

extern "C" igxrt_status igxrt_trace_gbuffer(igxrt_context* ctx, const igxrt_scene* scene,
                                            const igxrt_camera* cam, float* dir_object,
                                            float* uv_normal, uint32_t flags, void* stream_ptr) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    if (!cam || !dir_object || !uv_normal)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "camera and both images must be non-NULL");
    if (!cam->width || !cam->height)
        return IGXRT_OK;
    const uint64_t pixels = (uint64_t)cam->width * cam->height;
    if (pixels > 0x7fffffffu || cam->width > (1u << 24) || cam->height > (1u << 24))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "image too large");
    if (((uintptr_t)dir_object % 16) || ((uintptr_t)uv_normal % 16))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "images must be 16-byte aligned");
    if ((st = check_trace_flags(ctx, flags)) != IGXRT_OK)
        return st;
    igxrt_launch_params p;
    st = resolve_params(ctx, ctx->params, p);
    if (st != IGXRT_OK)
        return st;
    if (!scene->has_layout(p.layout))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, format("the scene has no layout %u", p.layout));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    const bool host = flags & IGXRT_TRACE_HOST_MEMORY;
    float4* d_do = reinterpret_cast<float4*>(dir_object);
    float4* d_uv = reinterpret_cast<float4*>(uv_normal);
    const size_t ib = pixels * sizeof(float4);
    // host images the kernel can address are written in place (a miss leaves
    // the caller's uv_normal as it is); others are staged
    const bool staged = host && ((flags & IGXRT_TRACE_STAGED) || !host_direct(ctx, dir_object) ||
                                 !host_direct(ctx, uv_normal));
    if (staged) {
        st = grow_stage(ctx, 2 * ((ib + 255) / 256 * 256));
        if (st != IGXRT_OK)
            return st;
        d_do = static_cast<float4*>(ctx->d_stage);
        d_uv = reinterpret_cast<float4*>(static_cast<char*>(ctx->d_stage) + (ib + 255) / 256 * 256);
        // uv_normal is not written on a miss: carry the caller's contents
        const cudaError_t e = cudaMemcpyAsync(d_uv, uv_normal, ib, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "g-buffer upload");
    } else if (!host && (!device_accessible(dir_object) || !device_accessible(uv_normal))) {
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    "a buffer is not device memory: pass IGXRT_TRACE_HOST_MEMORY for host arrays");
    }
    GbufferArgs a;
    a.g.tris = scene->tris;
    a.g.cam = *cam;
    a.g.inv_w = 1.0f / (float)cam->width;
    a.g.inv_h = 1.0f / (float)cam->height;
    a.g.tiles_x = (cam->width + 7) / 8;
    a.g.dir_object = d_do;
    a.g.uv_normal = d_uv;
    a.tiles = a.g.tiles_x * ((cam->height + 3) / 4);
    cudaError_t e = cudaSuccess;
    if (!scene->mixed && (!host || staged)) {
        CameraSource cs{*cam, a.g.inv_w, a.g.inv_h};
        TraceRequest req{scene, nullptr, nullptr, (uint32_t)pixels, 0, reinterpret_cast<igxrt_hit*>(d_do),
                         nullptr, nullptr, nullptr};
        req.camera = &cs;
        if ((st = launch_trace(ctx, req, p, stream)) != IGXRT_OK)
            return st;
        gbuffer_encode_kernel<<<(uint32_t)((pixels + 255) / 256), 256, 0, stream>>>(a.g, (uint32_t)pixels);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return cuda_fail(ctx, e, "g-buffer encoding launch");
    } else if ((st = launch_tiles(ctx, scene, p, a, stream)) != IGXRT_OK) {
        return st;
    }
    if (!host)
        return IGXRT_OK;
    if (staged) {
        e = cudaMemcpyAsync(dir_object, d_do, ib, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(uv_normal, d_uv, ib, cudaMemcpyDeviceToHost, stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "g-buffer download");
    }
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "g-buffer pass");
    return read_status(ctx);
}



extern "C" igxrt_status igxrt_camera_rays(igxrt_context* ctx, const igxrt_camera* cam, igxrt_ray* rays,
                                          uint32_t flags, void* stream_ptr) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (!cam || !rays)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "camera and rays must be non-NULL");
    if (const igxrt_status fst = check_trace_flags(ctx, flags))
        return fst;
    const uint64_t pixels = (uint64_t)cam->width * cam->height;
    if (!pixels)
        return IGXRT_OK;
    if (pixels > 0x7fffffffu || cam->width > (1u << 24) || cam->height > (1u << 24))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "image too large");
    if ((uintptr_t)rays % 16)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "rays must be 16-byte aligned");
    const bool host = flags & IGXRT_TRACE_HOST_MEMORY;
    if (!host && !device_accessible(rays))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    "rays is not device memory: pass IGXRT_TRACE_HOST_MEMORY for a host array");
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    const size_t bytes = pixels * sizeof(igxrt_ray);
    float4* d_rays = reinterpret_cast<float4*>(rays);
    // host rays the kernel can address are written in place, others staged
    const bool staged = host && ((flags & IGXRT_TRACE_STAGED) || !host_direct(ctx, rays));
    if (staged) {
        igxrt_status st = grow_stage(ctx, bytes);
        if (st != IGXRT_OK)
            return st;
        d_rays = static_cast<float4*>(ctx->d_stage);
    }
    camera_rays_kernel<<<(uint32_t)((pixels + 255) / 256), 256, 0, stream>>>(
        *cam, 1.0f / (float)cam->width, 1.0f / (float)cam->height, d_rays);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && staged)
        e = cudaMemcpyAsync(rays, d_rays, bytes, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess && host)
        e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "camera rays");
    return IGXRT_OK;
}
