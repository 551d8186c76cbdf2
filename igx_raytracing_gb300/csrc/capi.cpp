// capi.cpp — C ABI: contexts, resident scenes and ray-query entry points.
//
// Replaces the reference's dispatch boundary: RaygenTask / ShadowTask bind the
// SceneGraph's scene buffers and Dispatch a compute shader
// (src/rt/task/raygen_task.cpp:88-94, src/rt/task/shadow_task.cpp:194-213);
// here a scene is uploaded once (igxrt_scene_create) and each query is one
// stream-ordered call (igxrt_trace_closest / igxrt_trace_any).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>

#include "engine.h"

namespace igxrt {

igxrt_status fail(igxrt_context* ctx, igxrt_status st, const std::string& msg) {
    if (ctx)
        ctx->last_error = msg;
    return st;
}

igxrt_status cuda_fail(igxrt_context* ctx, cudaError_t e, const char* what) {
    const igxrt_status st = e == cudaErrorMemoryAllocation ? IGXRT_ERROR_OUT_OF_MEMORY : IGXRT_ERROR_CUDA;
    return fail(ctx, st, format("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e)));
}

DeviceGuard::DeviceGuard(int device) {
    if (cudaGetDevice(&prev_) != cudaSuccess)
        prev_ = -1;
    ok_ = (prev_ == device) || cudaSetDevice(device) == cudaSuccess;
}

DeviceGuard::~DeviceGuard() {
    int cur = -1;
    if (prev_ >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev_)
        cudaSetDevice(prev_);
}

uint32_t* take_queue_slot(igxrt_context* ctx) {
    const uint32_t s = ctx->next_slot;
    ctx->next_slot = (s + 1) % kQueueSlots;
    return ctx->d_words + s;
}

uint32_t* status_word(igxrt_context* ctx) { return ctx->d_words + kQueueSlots; }

igxrt_status resolve_params(igxrt_context* ctx, const igxrt_launch_params& in, igxrt_launch_params& out) {
    out = in;
    if (!out.block_size)
        out.block_size = 128;
    if (!out.packet_size)
        out.packet_size = 16;
    if (out.stack_depth == 0 && in.block_size == 0 && in.packet_size == 0)
        out.stack_depth = 16;
    if (!out.refill_lanes)
        out.refill_lanes = 8;
    if (out.refill_lanes > 32)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("refill_lanes %u: at most 32", out.refill_lanes));
    if (!out.phase_break)
        out.phase_break = 2;
    if (out.phase_break > 32)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("phase_break %u: 1..31, or 32 for no early end of the node phase",
                           out.phase_break));
    if (out.block_size < 32 || out.block_size > 256 || out.block_size % 32)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("block_size %u: use a multiple of 32 up to 256", out.block_size));
    if (out.packet_size < 8 || out.packet_size > 4096 || out.packet_size % 8)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("packet_size %u: use a multiple of 8 up to 4096", out.packet_size));
    if (out.stack_depth > 64)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("stack_depth %u: at most 64 shared entries", out.stack_depth));
    if (out.layout >= IGXRT_LAYOUT_COUNT)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown layout %u", out.layout));
    return IGXRT_OK;
}

// One device allocation per scene, 256-byte aligned sub-buffers in this
// order: BVH2 nodes, BVH4 nodes, records, triangles, planes, parent links of
// BVH2 and BVH4, refit words, BVH8 nodes, BVH8 slot sources.  Fills every
// pointer and count of the scene from `info` and the node counts; the
// contents are the caller's to write.
igxrt_status allocate_scene(igxrt_context* ctx, const igxrt_bvh_info& info, uint32_t n2, uint32_t n4,
                            uint32_t n8, igxrt_scene*& out) {
    out = nullptr;
    igxrt_scene* s = new (std::nothrow) igxrt_scene();
    if (!s)
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "scene object");
    s->device = ctx->device;
    s->info = info;
    const size_t records = (size_t)info.triangle_count + info.sphere_count + info.cube_count;
    const size_t b2 = round_up((size_t)n2 * sizeof(igxrt_bvh2_node), 256);
    const size_t b4 = round_up((size_t)n4 * sizeof(igxrt_bvh4_node), 256);
    const size_t bp = round_up(records * sizeof(igxrt_prim_record), 256);
    const size_t bt = round_up((size_t)info.triangle_count * sizeof(igxrt_triangle), 256);
    const size_t bl = round_up((size_t)info.plane_count * 16, 256);
    const size_t nn = (size_t)n2 + n4;
    const size_t bpar = round_up(nn * sizeof(uint32_t), 256);
    const size_t bw = round_up((kRefitStateWords + nn) * sizeof(uint32_t), 256);
    const size_t b8 = round_up((size_t)n8 * sizeof(igxrt_bvh8_node), 256);
    const size_t bs8 = round_up((size_t)n8 * 8 * sizeof(uint32_t), 256);
    const size_t o8 = b2 + b4 + bp + bt + bl + bpar + bw;
    cudaError_t e = cudaMalloc(&s->d_mem, o8 + b8 + bs8);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(ctx, e, "scene allocation");
    }
    char* base = (char*)s->d_mem;
    s->nodes[IGXRT_LAYOUT_BVH8] = base + o8;
    s->node_count[IGXRT_LAYOUT_BVH8] = n8;
    s->src8 = (const uint32_t*)(base + o8 + b8);
    s->nodes[IGXRT_LAYOUT_BVH2] = base;
    s->nodes[IGXRT_LAYOUT_BVH4] = base + b2;
    s->prims = (const igxrt_prim_record*)(base + b2 + b4);
    s->tris = (const igxrt_triangle*)(base + b2 + b4 + bp);
    s->planes = (const float*)(base + b2 + b4 + bp + bt);
    uint32_t* parents = (uint32_t*)(base + b2 + b4 + bp + bt + bl);
    s->parents[IGXRT_LAYOUT_BVH2] = parents;
    s->parents[IGXRT_LAYOUT_BVH4] = parents + n2;
    s->refit_words = (uint32_t*)(base + b2 + b4 + bp + bt + bl + bpar);
    s->node_count[IGXRT_LAYOUT_BVH2] = n2;
    s->node_count[IGXRT_LAYOUT_BVH4] = n4;
    s->mixed = info.sphere_count || info.cube_count || info.plane_count;
    s->plane_count = info.plane_count;
    s->plane_base = (uint32_t)records;
    out = s;
    return IGXRT_OK;
}

}  // namespace igxrt

using namespace igxrt;

namespace {

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

}  // namespace

// Rejects host pointers passed without IGXRT_TRACE_HOST_MEMORY: a kernel
// would fault on them.
bool igxrt::device_accessible(const void* p) {
    if (!p)
        return true;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged ||
           (attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr);
}

bool igxrt::host_direct(const igxrt_context* ctx, const void* p) {
    if (!p)
        return true;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged)
        return true;
    if (attr.type == cudaMemoryTypeHost)
        return attr.devicePointer == p;  // pinned and mapped at the host address
    return ctx->pageable_access;        // pageable memory
}

igxrt_status igxrt::check_trace_flags(igxrt_context* ctx, uint32_t flags, uint32_t extra) {
    if (flags & ~(IGXRT_TRACE_HOST_MEMORY | IGXRT_TRACE_STAGED | extra))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, format("unknown flags 0x%x", flags));
    if ((flags & IGXRT_TRACE_STAGED) && !(flags & IGXRT_TRACE_HOST_MEMORY))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "IGXRT_TRACE_STAGED needs IGXRT_TRACE_HOST_MEMORY");
    return IGXRT_OK;
}

igxrt_status igxrt::check_scene(igxrt_context* ctx, const igxrt_scene* scene) {
    if (!scene)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "scene is NULL");
    if (scene->device != ctx->device)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    format("scene lives on device %d, context on %d", scene->device, ctx->device));
    return IGXRT_OK;
}

igxrt_status igxrt::grow_stage(igxrt_context* ctx, size_t bytes) {
    if (ctx->stage_bytes >= bytes)
        return IGXRT_OK;
    if (ctx->d_stage) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "staging resize");
        cudaFree(ctx->d_stage);
        ctx->d_stage = nullptr;
        ctx->stage_bytes = 0;
    }
    size_t want = std::max(bytes, ctx->stage_bytes * 2);
    cudaError_t e = cudaMalloc(&ctx->d_stage, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&ctx->d_stage, bytes);
        want = bytes;
    }
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "staging allocation");
    ctx->stage_bytes = want;
    return IGXRT_OK;
}

igxrt_status igxrt::read_status(igxrt_context* ctx) {
    uint32_t word = 0;
    cudaError_t e = cudaMemcpy(&word, status_word(ctx), sizeof(word), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "status read");
    if (word) {
        cudaMemset(status_word(ctx), 0, sizeof(uint32_t));
        return fail(ctx, IGXRT_ERROR_KERNEL_STATUS,
                    format("kernel error word 0x%x (1 = traversal stack overflow, 2 = round limit)", word));
    }
    return IGXRT_OK;
}

namespace {

igxrt_status trace_common(igxrt_context* ctx, const igxrt_scene* scene, const igxrt_ray* rays,
                          const uint32_t* prev, uint32_t count, uint32_t mode, void* out,
                          uint32_t flags, void* stream_ptr, uint32_t* nf, uint32_t* pf,
                          const igxrt_launch_params& params) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    if (count == 0)
        return IGXRT_OK;
    if (count > 0x7fffffffu)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "more than 2^31-1 rays in one call");
    if (!rays || !out)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "rays and output must be non-NULL");
    if ((st = check_trace_flags(ctx, flags, IGXRT_TRACE_INDEPENDENT)) != IGXRT_OK)
        return st;
    if (!aligned(rays, 16) || (mode == 0 && !aligned(out, 16)) || !aligned(out, 4) ||
        !aligned(prev, 4) || !aligned(nf, 4) || !aligned(pf, 4))
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                    "rays and hits must be 16-byte aligned, other arrays 4-byte aligned");
    igxrt_launch_params p;
    st = resolve_params(ctx, params, p);
    if (st != IGXRT_OK)
        return st;
    if (!scene->has_layout(p.layout))
        return fail(ctx, IGXRT_ERROR_UNSUPPORTED,
                    format("the scene has no layout %u (GPU-built trees have BVH2 and BVH4)", p.layout));
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    const size_t out_elem = mode == 0 ? sizeof(igxrt_hit) : sizeof(uint32_t);

    if (!(flags & IGXRT_TRACE_HOST_MEMORY)) {
        if (!device_accessible(rays) || !device_accessible(prev) || !device_accessible(out) ||
            !device_accessible(nf) || !device_accessible(pf))
            return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT,
                        "a buffer is not device memory: pass IGXRT_TRACE_HOST_MEMORY for host arrays");
        TraceRequest req{scene, rays, prev, count, mode, mode == 0 ? (igxrt_hit*)out : nullptr,
                         mode == 1 ? (uint32_t*)out : nullptr, nf, pf};
        req.independent = (flags & IGXRT_TRACE_INDEPENDENT) != 0;
        return launch_trace(ctx, req, p, stream);
    }

    // Host arrays the kernel can address (pinned, or pageable on a device
    // that reads it through the host's page tables): the kernel loads each
    // ray once from host memory and stores each result once into it, over
    // the chip-to-chip link, with no staging copies.
    if (!(flags & IGXRT_TRACE_STAGED) && host_direct(ctx, rays) && host_direct(ctx, prev) &&
        host_direct(ctx, out) && host_direct(ctx, nf) && host_direct(ctx, pf)) {
        TraceRequest req{scene, rays, prev, count, mode, mode == 0 ? (igxrt_hit*)out : nullptr,
                         mode == 1 ? (uint32_t*)out : nullptr, nf, pf};
        if ((st = launch_trace(ctx, req, p, stream)) != IGXRT_OK)
            return st;
        const cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "trace");
        return read_status(ctx);
    }

    // Other host arrays: stage through the context's device buffer.
    const size_t rb = round_up((size_t)count * sizeof(igxrt_ray), 256);
    const size_t pb = prev ? round_up((size_t)count * 4, 256) : 0;
    const size_t ob = round_up((size_t)count * out_elem, 256);
    const size_t cb = nf ? 2 * round_up((size_t)count * 4, 256) : 0;
    st = grow_stage(ctx, rb + pb + ob + cb);
    if (st != IGXRT_OK)
        return st;
    char* base = (char*)ctx->d_stage;
    igxrt_ray* d_rays = (igxrt_ray*)base;
    uint32_t* d_prev = prev ? (uint32_t*)(base + rb) : nullptr;
    void* d_out = base + rb + pb;
    uint32_t* d_nf = nf ? (uint32_t*)(base + rb + pb + ob) : nullptr;
    uint32_t* d_pf = nf ? (uint32_t*)(base + rb + pb + ob + cb / 2) : nullptr;
    cudaError_t e = cudaMemcpyAsync(d_rays, rays, (size_t)count * sizeof(igxrt_ray),
                                    cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && prev)
        e = cudaMemcpyAsync(d_prev, prev, (size_t)count * 4, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "ray upload");
    TraceRequest req{scene, d_rays, d_prev, count, mode, mode == 0 ? (igxrt_hit*)d_out : nullptr,
                     mode == 1 ? (uint32_t*)d_out : nullptr, d_nf, d_pf};
    if ((st = launch_trace(ctx, req, p, stream)) != IGXRT_OK)
        return st;
    e = cudaMemcpyAsync(out, d_out, (size_t)count * out_elem, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess && nf) {
        e = cudaMemcpyAsync(nf, d_nf, (size_t)count * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pf, d_pf, (size_t)count * 4, cudaMemcpyDeviceToHost, stream);
    }
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "result download");
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "trace");
    return read_status(ctx);
}

}  // namespace

extern "C" {

const char* igxrt_status_string(igxrt_status s) {
    switch (s) {
        case IGXRT_OK: return "ok";
        case IGXRT_ERROR_INVALID_ARGUMENT: return "invalid argument";
        case IGXRT_ERROR_CUDA: return "CUDA error";
        case IGXRT_ERROR_OUT_OF_MEMORY: return "out of memory";
        case IGXRT_ERROR_INVALID_BVH: return "invalid BVH";
        case IGXRT_ERROR_KERNEL_STATUS: return "kernel raised its error word";
        case IGXRT_ERROR_ADMISSION: return "request exceeds the admission cap";
        case IGXRT_ERROR_TIMEOUT: return "timed out";
        case IGXRT_ERROR_UNSUPPORTED: return "unsupported";
        case IGXRT_ERROR_NOT_READY: return "not ready";
        case IGXRT_ERROR_IO: return "I/O error";
    }
    return "unknown status";
}

igxrt_status igxrt_create(int device, igxrt_context** out) {
    if (!out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return IGXRT_ERROR_CUDA;
    }
    if (device < 0 || device >= n)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(device);
    if (!guard.ok())
        return IGXRT_ERROR_CUDA;
    igxrt_context* ctx = new (std::nothrow) igxrt_context();
    if (!ctx)
        return IGXRT_ERROR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess)
        ctx->device_name = prop.name;
    if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&ctx->d_words, (2 * kQueueSlots + 1) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_words, 0, (2 * kQueueSlots + 1) * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        if (ctx->d_words)
            cudaFree(ctx->d_words);
        delete ctx;
        return IGXRT_ERROR_CUDA;
    }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    ctx->pageable_access = pageable != 0;
    igxrt_launch_params defaults{};
    resolve_params(ctx, defaults, ctx->params);
    *out = ctx;
    return IGXRT_OK;
}

igxrt_status igxrt_destroy(igxrt_context* ctx) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    {
        DeviceGuard guard(ctx->device);
        cudaDeviceSynchronize();
        if (ctx->d_batch) {
            cudaFree(ctx->d_batch);
            for (uint32_t i = 0; i < kBatchSlots; ++i)
                if (ctx->batch_events[i])
                    cudaEventDestroy(ctx->batch_events[i]);
        }
        if (ctx->d_stage)
            cudaFree(ctx->d_stage);
        if (ctx->d_words)
            cudaFree(ctx->d_words);
    }
    delete ctx;
    return IGXRT_OK;
}

const char* igxrt_last_error(const igxrt_context* ctx) {
    if (!ctx)
        return "context is NULL";
    return ctx->last_error.c_str();
}

igxrt_status igxrt_set_launch_params(igxrt_context* ctx, const igxrt_launch_params* p) {
    if (!ctx || !p)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    igxrt_launch_params r;
    const igxrt_status st = resolve_params(ctx, *p, r);
    if (st == IGXRT_OK)
        ctx->params = r;
    return st;
}

igxrt_status igxrt_get_launch_params(const igxrt_context* ctx, igxrt_launch_params* p) {
    if (!ctx || !p)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *p = ctx->params;
    return IGXRT_OK;
}

igxrt_status igxrt_scene_create_from_bvh(igxrt_context* ctx, const igxrt_bvh* bvh, igxrt_scene** out) {
    if (!ctx || !bvh || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    std::vector<uint32_t> par2, par4;
    try {
        node_parents(*bvh, par2, par4);
    } catch (const std::bad_alloc&) {
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "parent links");
    }
    igxrt_scene* s = nullptr;
    igxrt_status st = allocate_scene(ctx, bvh->info, (uint32_t)bvh->nodes2.size(),
                                     (uint32_t)bvh->nodes4.size(), (uint32_t)bvh->nodes8.size(), s);
    if (st != IGXRT_OK)
        return st;
    cudaError_t e = cudaSuccess;
    auto up = [&e](const void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpy(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice);
    };
    up(s->nodes[IGXRT_LAYOUT_BVH8], bvh->nodes8.data(), bvh->nodes8.size() * sizeof(igxrt_bvh8_node));
    up(s->src8, bvh->src8.data(), bvh->src8.size() * sizeof(uint32_t));
    up(s->parents[IGXRT_LAYOUT_BVH2], par2.data(), par2.size() * sizeof(uint32_t));
    up(s->parents[IGXRT_LAYOUT_BVH4], par4.data(), par4.size() * sizeof(uint32_t));
    up(s->planes, bvh->planes.data(), bvh->planes.size() * sizeof(float));
    up(s->nodes[IGXRT_LAYOUT_BVH2], bvh->nodes2.data(), bvh->nodes2.size() * sizeof(igxrt_bvh2_node));
    up(s->nodes[IGXRT_LAYOUT_BVH4], bvh->nodes4.data(), bvh->nodes4.size() * sizeof(igxrt_bvh4_node));
    up(s->prims, bvh->prims.data(), bvh->prims.size() * sizeof(igxrt_prim_record));
    up(s->tris, bvh->tris.data(), bvh->tris.size() * sizeof(igxrt_triangle));
    if (e != cudaSuccess) {
        igxrt_scene_destroy(s);
        return cuda_fail(ctx, e, "scene upload");
    }
    *out = s;
    return IGXRT_OK;
}

igxrt_status igxrt_scene_create(igxrt_context* ctx, const igxrt_triangle* tris, uint32_t count,
                                const igxrt_build_options* opts, igxrt_scene** out) {
    if (!ctx || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_bvh bvh;
    std::string err;
    igxrt_status st;
    try {
        st = build_bvh(tris, count, opts, bvh, err);
    } catch (const std::bad_alloc&) {
        st = IGXRT_ERROR_OUT_OF_MEMORY;
        err = "host memory exhausted during the BVH build";
    }
    if (st != IGXRT_OK)
        return fail(ctx, st, err);
    return igxrt_scene_create_from_bvh(ctx, &bvh, out);
}

igxrt_status igxrt_scene_create_mixed(igxrt_context* ctx, const igxrt_scene_desc* desc,
                                      const igxrt_build_options* opts, igxrt_scene** out) {
    if (!ctx || !out || !desc)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_bvh bvh;
    std::string err;
    igxrt_status st;
    try {
        st = build_bvh_mixed(*desc, opts, bvh, err);
    } catch (const std::bad_alloc&) {
        st = IGXRT_ERROR_OUT_OF_MEMORY;
        err = "host memory exhausted during the BVH build";
    }
    if (st != IGXRT_OK)
        return fail(ctx, st, err);
    return igxrt_scene_create_from_bvh(ctx, &bvh, out);
}

igxrt_status igxrt_scene_destroy(igxrt_scene* scene) {
    if (!scene)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    {
        DeviceGuard guard(scene->device);
        cudaDeviceSynchronize();
        cudaFree(scene->d_mem);
        cudaFree(scene->refit_boxes);
        cudaFree(scene->refit_unions);
    }
    delete scene;
    return IGXRT_OK;
}

igxrt_status igxrt_scene_get_info(const igxrt_scene* scene, igxrt_bvh_info* info) {
    if (!scene || !info)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *info = scene->info;
    return IGXRT_OK;
}

igxrt_status igxrt_scene_download(igxrt_context* ctx, const igxrt_scene* scene, igxrt_bvh** out) {
    if (!ctx || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_status st = check_scene(ctx, scene);
    if (st != IGXRT_OK)
        return st;
    DeviceGuard guard(ctx->device);
    if (!guard.ok())
        return fail(ctx, IGXRT_ERROR_CUDA, "cannot select the context's device");
    igxrt_bvh* b = new (std::nothrow) igxrt_bvh();
    if (!b)
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "BVH object");
    const igxrt_bvh_info& info = scene->info;
    const size_t records = (size_t)info.triangle_count + info.sphere_count + info.cube_count;
    cudaError_t e = cudaSuccess;
    try {
        b->info = info;
        b->nodes2.resize(scene->node_count[IGXRT_LAYOUT_BVH2]);
        b->nodes4.resize(scene->node_count[IGXRT_LAYOUT_BVH4]);
        b->nodes8.resize(scene->node_count[IGXRT_LAYOUT_BVH8]);
        b->src8.resize(8 * (size_t)scene->node_count[IGXRT_LAYOUT_BVH8]);
        b->prims.resize(records);
        b->tris.resize(info.triangle_count);
        b->planes.resize(4 * (size_t)info.plane_count);
        b->spheres.resize(4 * (size_t)info.sphere_count);
        b->cubes.resize(info.cube_count);
    } catch (const std::bad_alloc&) {
        delete b;
        return fail(ctx, IGXRT_ERROR_OUT_OF_MEMORY, "host memory for the BVH");
    }
    e = cudaDeviceSynchronize();
    auto down = [&e](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    };
    down(b->nodes2.data(), scene->nodes[IGXRT_LAYOUT_BVH2], b->nodes2.size() * sizeof(igxrt_bvh2_node));
    down(b->nodes4.data(), scene->nodes[IGXRT_LAYOUT_BVH4], b->nodes4.size() * sizeof(igxrt_bvh4_node));
    down(b->nodes8.data(), scene->nodes[IGXRT_LAYOUT_BVH8], b->nodes8.size() * sizeof(igxrt_bvh8_node));
    down(b->src8.data(), scene->src8, b->src8.size() * sizeof(uint32_t));
    down(b->prims.data(), scene->prims, records * sizeof(igxrt_prim_record));
    down(b->tris.data(), scene->tris, b->tris.size() * sizeof(igxrt_triangle));
    down(b->planes.data(), scene->planes, b->planes.size() * sizeof(float));
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(ctx, e, "scene download");
    }
    // spheres and cubes live only in their records: (centre, radius), (start, end)
    const uint32_t nt = info.triangle_count, ns = info.sphere_count;
    for (const igxrt_prim_record& r : b->prims) {
        if (r.prim >= records)
            continue;  // the validator below reports it
        if (r.prim >= nt && r.prim < nt + ns) {
            float* s = &b->spheres[4 * (size_t)(r.prim - nt)];
            s[0] = r.p0[0];
            s[1] = r.p0[1];
            s[2] = r.p0[2];
            s[3] = r.e1[0];
        } else if (r.prim >= nt + ns) {
            igxrt_cube& c = b->cubes[r.prim - nt - ns];
            c.xy0[0] = r.p0[0];
            c.xy0[1] = r.p0[1];
            c.z0_x1[0] = r.p0[2];
            c.z0_x1[1] = r.e1[0];
            c.yz1[0] = r.e1[1];
            c.yz1[1] = r.e1[2];
        }
    }
    std::string msg;
    if ((st = validate_bvh(*b, msg)) != IGXRT_OK) {
        delete b;
        return fail(ctx, st, "downloaded scene: " + msg);
    }
    *out = b;
    return IGXRT_OK;
}

igxrt_status igxrt_trace_closest(igxrt_context* ctx, const igxrt_scene* scene, const igxrt_ray* rays,
                                 const uint32_t* prev_hit, uint32_t count, igxrt_hit* hits,
                                 uint32_t flags, void* stream) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    return trace_common(ctx, scene, rays, prev_hit, count, 0, hits, flags, stream, nullptr, nullptr,
                        ctx->params);
}

igxrt_status igxrt_trace_any(igxrt_context* ctx, const igxrt_scene* scene, const igxrt_ray* rays,
                             const uint32_t* prev_hit, uint32_t count, uint32_t* occluded,
                             uint32_t flags, void* stream) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    return trace_common(ctx, scene, rays, prev_hit, count, 1, occluded, flags, stream, nullptr,
                        nullptr, ctx->params);
}

igxrt_status igxrt_count_fetches(igxrt_context* ctx, const igxrt_scene* scene, const igxrt_ray* rays,
                                 const uint32_t* prev_hit, uint32_t count, uint32_t mode,
                                 uint32_t layout, uint32_t* node_fetches, uint32_t* prim_fetches,
                                 void* stream) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (mode > 1 || layout >= IGXRT_LAYOUT_COUNT || !node_fetches || !prim_fetches)
        return fail(ctx, IGXRT_ERROR_INVALID_ARGUMENT, "mode 0/1, a valid layout and both count arrays");
    if (count == 0)
        return IGXRT_OK;
    // The instrumented kernel also writes the query's results; they go to a
    // scratch area inside the staging buffer.
    igxrt_launch_params p = ctx->params;
    p.layout = layout;
    DeviceGuard guard(ctx->device);
    cudaPointerAttributes attr;
    const bool host = cudaPointerGetAttributes(&attr, node_fetches) != cudaSuccess ||
                      attr.type == cudaMemoryTypeUnregistered;
    cudaGetLastError();
    const size_t ob = round_up((size_t)count * (mode == 0 ? sizeof(igxrt_hit) : 4), 256);
    if (host) {
        // Host count arrays: the results buffer is host memory too.
        std::vector<char> scratch_out(ob);
        return trace_common(ctx, scene, rays, prev_hit, count, mode, scratch_out.data(),
                            IGXRT_TRACE_HOST_MEMORY, stream, node_fetches, prim_fetches, p);
    }
    void* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_out, ob);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "count scratch");
    const igxrt_status st = trace_common(ctx, scene, rays, prev_hit, count, mode, d_out, 0, stream,
                                         node_fetches, prim_fetches, p);
    cudaStreamSynchronize((cudaStream_t)stream);
    cudaFree(d_out);
    return st;
}

igxrt_status igxrt_fetch_hits(igxrt_context* ctx, const igxrt_hit* device_hits, uint32_t count,
                              igxrt_hit* host_hits, void* stream) {
    if (!ctx || (count && (!device_hits || !host_hits)))
        return IGXRT_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    cudaError_t e = cudaMemcpyAsync(host_hits, device_hits, (size_t)count * sizeof(igxrt_hit),
                                    cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "fetch hits");
    return IGXRT_OK;
}

igxrt_status igxrt_sync(igxrt_context* ctx, void* stream) {
    if (!ctx)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "stream synchronize");
    return read_status(ctx);
}

}  // extern "C"
