// shadow.cu — the reference's shadow pass as one kernel: any-hit rays per
// pixel and sample, packed into its 32-bit ballot words.
//
// res/shaders/nv_all.shadow.comp:50-142 runs one thread per pixel and sample
// in 16x16x2 work groups; on NVIDIA each 32-lane subgroup covers a 16x2 pixel
// tile of one sample, traces traceOcclusion for pixels whose primary object
// is not noRayHit (:108-126), and lane 0 stores ballotARB(hit) at
// indexToLight(loc, res, sample, shift = (4,1), mask = (15,1))
// (light.glsl:221-229).  Here a warp owns one tile word: lane l handles pixel
// (16*tx + (l & 15), 2*ty + (l >> 4)), so the warp's ballot is that word
// directly and the traversal of the 32 rays of a tile (neighbouring pixels,
// one light) stays coherent.
#include <algorithm>

#include "engine.h"
#include "traverse.cuh"

namespace igxrt {

struct ShadowArgs {
    const float4* nodes;
    const float4* prims;
    uint32_t node_count;
    const igxrt_ray* rays;
    const uint32_t* object;
    uint32_t width, height;
    uint32_t tiles_x, tiles_y;
    uint32_t words;
    uint32_t* mask;
    uint32_t* status;
    uint32_t sh_depth;
};

template <int LAYOUT>
__global__ void __launch_bounds__(256) shadow_mask_kernel(ShadowArgs a) {
    extern __shared__ uint32_t smem[];
    TraversalStack st;
    st.sh = reinterpret_cast<uint2*>(smem) + threadIdx.x;
    st.stride = blockDim.x;
    st.sh_depth = a.sh_depth;
    st.sp = 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t per_sample = a.tiles_x * a.tiles_y;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < a.words; w += warps) {
        const uint32_t s = w / per_sample, rem = w - s * per_sample;
        const uint32_t ty = rem / a.tiles_x, tx = rem - ty * a.tiles_x;
        const uint32_t x = tx * 16u + (lane & 15u), y = ty * 2u + (lane >> 4);
        bool occ = false;
        if (x < a.width && y < a.height) {
            const uint32_t obj = __ldg(a.object + (size_t)y * a.width + x);
            if (obj != IGXRT_NO_RAY_HIT) {
                const uint32_t i = (uint32_t)(((size_t)s * a.height + y) * a.width + x);
                const RayState r = load_ray(a.rays, i, obj);
                BestHit best;
                bool overflow = false;
                occ = trace_single<LAYOUT, true>(a.nodes, a.prims, a.node_count, r, best, st, overflow);
                if (overflow)
                    atomicOr(a.status, kStatusStackOverflow);
            }
        }
        const uint32_t bits = __ballot_sync(0xffffffffu, occ);
        if (lane == 0)
            __stcs(a.mask + w, bits);
    }
}

}  // namespace igxrt

using namespace igxrt;

extern "C" igxrt_status igxrt_trace_shadow_mask(igxrt_context* ctx, const igxrt_scene* scene,
                                                const igxrt_ray* rays, const uint32_t* object,
                                                uint32_t width, uint32_t height, uint32_t samples,
                                                uint32_t* mask, uint32_t flags, void* stream_ptr) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    if (scene->mixed)
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, "the shadow pass takes triangle-only scenes");
    if (!width || !height || !samples)
        return IGXRT_OK;
    const uint64_t pixels = (uint64_t)width * height, nrays = pixels * samples;
    const uint64_t tiles_x = (width + 15) / 16, tiles_y = (height + 1) / 2;
    const uint64_t words = tiles_x * tiles_y * samples;
    if (nrays > 0x7fffffffu || words > 0x7fffffffu)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "more than 2^31-1 rays in one shadow pass");
    if (!rays || !object || !mask)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "rays, object and mask must be non-NULL");
    if (((uintptr_t)rays % 16) || ((uintptr_t)object % 4) || ((uintptr_t)mask % 4))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "rays 16-byte aligned, object/mask 4-byte aligned");
    if (flags & ~IGXRT_TRACE_HOST_MEMORY)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown flags 0x%x", flags));
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
    const igxrt_ray* d_rays = rays;
    const uint32_t* d_obj = object;
    uint32_t* d_mask = mask;
    if (host) {
        const size_t rb = (nrays * sizeof(igxrt_ray) + 255) / 256 * 256;
        const size_t ob = (pixels * 4 + 255) / 256 * 256;
        st = grow_stage(ctx, rb + ob + words * 4);
        if (st != IGXRT_OK)
            return st;
        char* base = static_cast<char*>(ctx->d_stage);
        d_rays = reinterpret_cast<const igxrt_ray*>(base);
        d_obj = reinterpret_cast<const uint32_t*>(base + rb);
        d_mask = reinterpret_cast<uint32_t*>(base + rb + ob);
        cudaError_t e = cudaMemcpyAsync(base, rays, nrays * sizeof(igxrt_ray), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(base + rb, object, pixels * 4, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "shadow upload");
    } else if (!device_accessible(rays) || !device_accessible(object) || !device_accessible(mask)) {
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    "a buffer is not device memory: pass IGXRT_TRACE_HOST_MEMORY for host arrays");
    }
    ShadowArgs a;
    a.nodes = reinterpret_cast<const float4*>(scene->nodes[p.layout]);
    a.prims = reinterpret_cast<const float4*>(scene->prims);
    a.node_count = scene->node_count[p.layout];
    a.rays = d_rays;
    a.object = d_obj;
    a.width = width;
    a.height = height;
    a.tiles_x = (uint32_t)tiles_x;
    a.tiles_y = (uint32_t)tiles_y;
    a.words = (uint32_t)words;
    a.mask = d_mask;
    a.status = status_word(ctx);
    a.sh_depth = p.stack_depth;
    auto fn = p.layout == IGXRT_LAYOUT_BVH8   ? shadow_mask_kernel<IGXRT_LAYOUT_BVH8>
              : p.layout == IGXRT_LAYOUT_BVH4 ? shadow_mask_kernel<IGXRT_LAYOUT_BVH4>
                                              : shadow_mask_kernel<IGXRT_LAYOUT_BVH2>;
    const size_t smem = (size_t)p.stack_depth * p.block_size * kStackEntryBytes;
    int per_sm = 0;
    cudaError_t e = allow_smem((const void*)fn, smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)p.block_size, smem);
    if (e != cudaSuccess || per_sm < 1)
        return e != cudaSuccess ? cuda_fail(ctx, e, "occupancy query")
                                : fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "no resident CTA");
    const uint64_t warps_per_block = p.block_size / 32;
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, (words + warps_per_block - 1) / warps_per_block));
    fn<<<grid, p.block_size, smem, stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "shadow kernel launch");
    if (host) {
        e = cudaMemcpyAsync(mask, d_mask, words * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "shadow download");
        return read_status(ctx);
    }
    return IGXRT_OK;
}
