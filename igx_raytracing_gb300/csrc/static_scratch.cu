// static_scratch.cu — igxrt_trace_closest_static: a closest-hit query from
// host arrays that allocates no device memory.
//
// Who needs it: a caller that must not call cudaMalloc while tracing (a render
// loop whose device memory belongs to another allocator's budget, or whose
// frame cannot absorb the synchronisation an allocation may cause).  The
// regular host-memory path (igxrt_trace_closest + IGXRT_TRACE_HOST_MEMORY)
// grows a staging buffer with cudaMalloc; this one stages through the fixed
// file-scope array below, so a call costs copies and one kernel launch only.
//
// Layout of the array (IGXRT_STATIC_SCRATCH_BYTES = 16 MiB):
//   [0, 256)            word 0: work-queue counter, word 1: error word
//   [256, ...)          rays (32 B each), then prev_hit (4 B each, if given),
//                       then hits (16 B each), each region 256-byte aligned.
// IGXRT_STATIC_MAX_RAYS = 320,000 rays fit: 256 + 3*256 + 52 * 320000 bytes.
//
// The array persists for the process on every device that loads the library;
// every call shares it, so calls that overlap on the GPU race.  Each call
// clears the counter and the error word before its launch.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "engine.h"

namespace igxrt {
namespace {

constexpr size_t kHeaderBytes = 256;
constexpr int kMaxDevices = 64;

static_assert(kHeaderBytes + 3 * 256 + (size_t)52 * IGXRT_STATIC_MAX_RAYS <= IGXRT_STATIC_SCRATCH_BYTES,
              "IGXRT_STATIC_MAX_RAYS does not fit the static scratch array");

// The scratch itself.  In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_static_scratch[IGXRT_STATIC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

// Looks the array's device address up once per device (the device must be
// current).  This is the only CUDA call of the set-up; it allocates nothing.
igxrt_status scratch_address(igxrt_context* ctx, int device, char** out) {
    if (device < 0 || device >= kMaxDevices)
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED, format("device %d beyond the static table", device));
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return cuda_fail(ctx, e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                             "static scratch address lookup");
        g_scratch_addr[device] = p;
    }
    *out = static_cast<char*>(g_scratch_addr[device]);
    return IGXRT_OK;
}

}  // namespace
}  // namespace igxrt

using namespace igxrt;

extern "C" igxrt_status igxrt_trace_closest_static(igxrt_context* ctx, const igxrt_scene* scene,
                                                   const igxrt_ray* rays, const uint32_t* prev_hit,
                                                   uint32_t count, igxrt_hit* hits, void* stream_ptr) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (!scene)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "scene is NULL");
    if (scene->device != ctx->device)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("scene lives on device %d, context on %d", scene->device, ctx->device));
    if (count == 0)
        return IGXRT_OK;
    if (count > IGXRT_STATIC_MAX_RAYS)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("igxrt_trace_closest_static: %u rays exceed the static scratch limit of "
                           "%u rays per call (IGXRT_STATIC_MAX_RAYS); split the batch",
                           count, IGXRT_STATIC_MAX_RAYS));
    if (!rays || !hits)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "rays and hits must be non-NULL");
    igxrt_launch_params p;
    igxrt_status st = resolve_params(ctx, ctx->params, p);
    if (st != IGXRT_OK)
        return st;
    // a tree without the context's layout (a GPU-built scene has no BVH8)
    // would trace every ray as a miss: refuse it as igxrt_trace_closest does
    if (!scene->has_layout(p.layout))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED,
                    format("the scene has no layout %u (GPU-built trees have BVH2 and BVH4)", p.layout));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    char* base = nullptr;
    st = scratch_address(ctx, ctx->device, &base);
    if (st != IGXRT_OK)
        return st;

    cudaStream_t stream = (cudaStream_t)stream_ptr;
    uint32_t* words = reinterpret_cast<uint32_t*>(base);
    const size_t rb = round256((size_t)count * sizeof(igxrt_ray));
    const size_t pb = prev_hit ? round256((size_t)count * sizeof(uint32_t)) : 0;
    igxrt_ray* d_rays = reinterpret_cast<igxrt_ray*>(base + kHeaderBytes);
    uint32_t* d_prev = prev_hit ? reinterpret_cast<uint32_t*>(base + kHeaderBytes + rb) : nullptr;
    igxrt_hit* d_hits = reinterpret_cast<igxrt_hit*>(base + kHeaderBytes + rb + pb);

    cudaError_t e = cudaMemsetAsync(words, 0, kHeaderBytes, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_rays, rays, (size_t)count * sizeof(igxrt_ray), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && prev_hit)
        e = cudaMemcpyAsync(d_prev, prev_hit, (size_t)count * sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "static scratch upload");
    TraceRequest req{scene, d_rays, d_prev, count, 0, d_hits, nullptr, nullptr, nullptr};
    st = launch_trace_words(ctx, req, p, stream, words, words + 1);
    if (st != IGXRT_OK)
        return st;
    uint32_t status_word = 0;
    e = cudaMemcpyAsync(hits, d_hits, (size_t)count * sizeof(igxrt_hit), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&status_word, words + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "static scratch trace");
    if (status_word)
        return fail(ctx, IGXRT_ERROR_KERNEL_STATUS,
                    format("kernel error word 0x%x (1 = traversal stack overflow, 2 = round limit)", status_word));
    return IGXRT_OK;
}
