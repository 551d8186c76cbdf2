// engine.h — host-side engine objects shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "internal.h"

struct igxrt_context {
    int device = 0;
    int sm_count = 0;
    std::string last_error;
    // Device words: kQueueSlots work-queue counters, then the error word.
    uint32_t* d_words = nullptr;
    uint32_t next_slot = 0;
    igxrt_launch_params params{};
    // Staging for IGXRT_TRACE_HOST_MEMORY traces (grown on demand).
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
};

struct igxrt_scene {
    int device = 0;
    igxrt_bvh_info info{};
    void* d_mem = nullptr;
    const void* nodes[IGXRT_LAYOUT_COUNT] = {nullptr, nullptr};
    uint32_t node_count[IGXRT_LAYOUT_COUNT] = {0, 0};
    const igxrt_prim_record* prims = nullptr;
    const igxrt_triangle* tris = nullptr;
};

namespace igxrt {

constexpr uint32_t kQueueSlots = 4096;

// One traversal launch over `count` rays of one scene (device pointers).
struct TraceRequest {
    const igxrt_scene* scene;
    const igxrt_ray* rays;
    const uint32_t* prev;
    uint32_t count;
    uint32_t mode;  // 0 closest, 1 any
    igxrt_hit* hits;
    uint32_t* occluded;
    uint32_t* node_fetches;  // non-null: instrumented kernel
    uint32_t* prim_fetches;
};

// Records `msg` as the context's last error and returns `st`.
igxrt_status fail(igxrt_context* ctx, igxrt_status st, const std::string& msg);
igxrt_status cuda_fail(igxrt_context* ctx, cudaError_t e, const char* what);

// Checks the launch parameters and fills defaults.
igxrt_status resolve_params(igxrt_context* ctx, const igxrt_launch_params& in,
                            igxrt_launch_params& out);

// Queues the traversal kernel (with its queue reset) on `stream`.
igxrt_status launch_trace(igxrt_context* ctx, const TraceRequest& req,
                          const igxrt_launch_params& params, cudaStream_t stream);

// Same launch, with the work-queue counter and error word supplied by the
// caller (device addresses); the counter is not reset here.
igxrt_status launch_trace_words(igxrt_context* ctx, const TraceRequest& req,
                                const igxrt_launch_params& params, cudaStream_t stream,
                                uint32_t* queue, uint32_t* status);

// Next work-queue counter of the context (a ring of kQueueSlots words).
uint32_t* take_queue_slot(igxrt_context* ctx);
uint32_t* status_word(igxrt_context* ctx);

// Makes ctx->device current for the lifetime of the guard.
class DeviceGuard {
   public:
    explicit DeviceGuard(int device);
    ~DeviceGuard();
    bool ok() const { return ok_; }

   private:
    int prev_ = -1;
    bool ok_ = false;
};

}  // namespace igxrt
