// shadow.cu — the reference's shadow pass: any-hit rays per pixel and sample,
// packed into its 32-bit ballot words.
//
// res/shaders/nv_all.shadow.comp:50-142 runs one thread per pixel and sample
// in 16x16x2 work groups; on NVIDIA each 32-lane subgroup covers a 16x2 pixel
// tile of one sample, traces traceOcclusion for pixels whose primary object
// is not noRayHit (:108-126), and lane 0 stores ballotARB(hit) at
// indexToLight(loc, res, sample, shift = (4,1), mask = (15,1))
// (light.glsl:221-229).  A thread per pixel leaves every lane of a pixel
// that missed the scene idle; here the pass runs in three kernels:
//   1. compact: the (sample, pixel) pairs whose object is not noRayHit get a
//      slot (one warp-aggregated atomicAdd per warp); their ray and object
//      (the prevHit) are gathered into the slot, and the pair remembers its
//      slot;
//   2. trace: the persistent any-hit kernel over the slots, its ray count
//      read from the device word the compaction filled (no host round trip);
//   3. pack: a warp per tile word reads its 32 pixels' results through their
//      slots and stores the ballot.
// The words equal the shader's: every ray is traced with the plain kernel's
// arithmetic, and a pixel without a ray contributes a zero bit.
#include <algorithm>

#include "engine.h"

namespace igxrt {

namespace {

constexpr uint32_t kNoSlot = 0xffffffffu;

__global__ void shadow_compact_kernel(const igxrt_ray* __restrict__ rays, const uint32_t* __restrict__ object,
                                      uint32_t pixels, uint32_t nrays, igxrt_ray* __restrict__ crays,
                                      uint32_t* __restrict__ cprev, uint32_t* __restrict__ slot_of,
                                      uint32_t* __restrict__ count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t obj = IGXRT_NO_RAY_HIT;
    if (i < nrays)
        obj = __ldg(object + i % pixels);
    const bool traced = obj != IGXRT_NO_RAY_HIT;
    const uint32_t want = __ballot_sync(0xffffffffu, traced);
    uint32_t base = 0;
    if (lane == 0 && want)
        base = atomicAdd(count, (uint32_t)__popc(want));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (i >= nrays)
        return;
    if (!traced) {
        slot_of[i] = kNoSlot;
        return;
    }
    const uint32_t slot = base + __popc(want & ((1u << lane) - 1u));
    const float4* src = reinterpret_cast<const float4*>(rays) + 2 * (size_t)i;
    float4* dst = reinterpret_cast<float4*>(crays) + 2 * (size_t)slot;
    dst[0] = __ldg(src);
    dst[1] = __ldg(src + 1);
    cprev[slot] = obj;
    slot_of[i] = slot;
}

__global__ void shadow_pack_kernel(const uint32_t* __restrict__ slot_of, const uint32_t* __restrict__ occluded,
                                   uint32_t width, uint32_t height, uint32_t tiles_x, uint32_t tiles_y,
                                   uint32_t words, uint32_t* __restrict__ mask) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= words)
        return;  // whole warps leave together (words are per warp)
    const uint32_t per_sample = tiles_x * tiles_y;
    const uint32_t s = w / per_sample, rem = w - s * per_sample;
    const uint32_t ty = rem / tiles_x, tx = rem - ty * tiles_x;
    const uint32_t x = tx * 16u + (lane & 15u), y = ty * 2u + (lane >> 4);
    bool occ = false;
    if (x < width && y < height) {
        const uint32_t slot = __ldg(slot_of + ((size_t)s * height + y) * width + x);
        occ = slot != kNoSlot && __ldg(occluded + slot) != 0u;
    }
    const uint32_t bits = __ballot_sync(0xffffffffu, occ);
    if (lane == 0)
        __stcs(mask + w, bits);
}

}  // namespace

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
    if ((st = check_trace_flags(ctx, flags)) != IGXRT_OK)
        return st;
    igxrt_launch_params p;
    st = resolve_params(ctx, ctx->params, p);
    if (st != IGXRT_OK)
        return st;
    if (!scene->has_layout(p.layout))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, format("the scene has no layout %u", p.layout));
    const bool host = flags & IGXRT_TRACE_HOST_MEMORY;
    if (!host && (!device_accessible(rays) || !device_accessible(object) || !device_accessible(mask)))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    "a buffer is not device memory: pass IGXRT_TRACE_HOST_MEMORY for host arrays");
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    // host arrays the kernels can address are read and written in place
    // (the compaction gathers the traced rays into device memory); others
    // are staged
    const bool staged = host && ((flags & IGXRT_TRACE_STAGED) || !host_direct(ctx, rays) ||
                                 !host_direct(ctx, object) || !host_direct(ctx, mask));

    // staging and the pass's scratch, one growable buffer:
    // [rays][object][mask] when staged, then [count][slot_of][cprev][occluded][crays]
    const size_t rb = staged ? round_up(nrays * sizeof(igxrt_ray), 256) : 0;
    const size_t ob = staged ? round_up(pixels * 4, 256) : 0;
    const size_t mb = staged ? round_up(words * 4, 256) : 0;
    const size_t cb = 256, sb = round_up(nrays * 4, 256), pb = sb, occb = sb,
                 crb = round_up(nrays * sizeof(igxrt_ray), 256);
    st = grow_stage(ctx, rb + ob + mb + cb + sb + pb + occb + crb);
    if (st != IGXRT_OK)
        return st;
    char* base = static_cast<char*>(ctx->d_stage);
    const igxrt_ray* d_rays = rays;
    const uint32_t* d_obj = object;
    uint32_t* d_mask = mask;
    cudaError_t e = cudaSuccess;
    if (staged) {
        d_rays = reinterpret_cast<const igxrt_ray*>(base);
        d_obj = reinterpret_cast<const uint32_t*>(base + rb);
        d_mask = reinterpret_cast<uint32_t*>(base + rb + ob);
        e = cudaMemcpyAsync(base, rays, nrays * sizeof(igxrt_ray), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(base + rb, object, pixels * 4, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "shadow upload");
    }
    char* scratch = base + rb + ob + mb;
    uint32_t* d_count = reinterpret_cast<uint32_t*>(scratch);
    uint32_t* d_slot = reinterpret_cast<uint32_t*>(scratch + cb);
    uint32_t* d_prev = reinterpret_cast<uint32_t*>(scratch + cb + sb);
    uint32_t* d_occ = reinterpret_cast<uint32_t*>(scratch + cb + sb + pb);
    igxrt_ray* d_crays = reinterpret_cast<igxrt_ray*>(scratch + cb + sb + pb + occb);

    if ((e = cudaMemsetAsync(d_count, 0, 4, stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "shadow count reset");
    shadow_compact_kernel<<<(uint32_t)((nrays + 255) / 256), 256, 0, stream>>>(
        d_rays, d_obj, (uint32_t)pixels, (uint32_t)nrays, d_crays, d_prev, d_slot, d_count);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return cuda_fail(ctx, e, "shadow compaction");
    TraceRequest req{scene, d_crays, d_prev, (uint32_t)nrays, 1, nullptr, d_occ, nullptr, nullptr};
    req.count_dev = d_count;
    if ((st = launch_trace(ctx, req, p, stream)) != IGXRT_OK)
        return st;
    shadow_pack_kernel<<<(uint32_t)((words * 32 + 255) / 256), 256, 0, stream>>>(
        d_slot, d_occ, width, height, (uint32_t)tiles_x, (uint32_t)tiles_y, (uint32_t)words, d_mask);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return cuda_fail(ctx, e, "shadow packing");
    if (!host)
        return IGXRT_OK;
    if (staged)
        e = cudaMemcpyAsync(mask, d_mask, words * 4, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "shadow download");
    return read_status(ctx);
}
