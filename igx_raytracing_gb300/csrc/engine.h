// engine.h — host-side engine objects shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace igxrt {
// Ring of item tables used by igxrt_trace_batch.
constexpr uint32_t kBatchSlots = 16;
constexpr uint32_t kBatchSlotItems = 4096;
}  // namespace igxrt

struct igxrt_context {
    int device = 0;
    int sm_count = 0;
    std::string device_name;
    std::string last_error;
    // igxrt_trace_batch item tables and the events guarding their reuse.
    void* d_batch = nullptr;
    cudaEvent_t batch_events[igxrt::kBatchSlots] = {};
    uint32_t next_batch_slot = 0;
    // Device words: kQueueSlots work-queue counters, the error word, then one
    // exit counter per queue slot (see launch_trace).
    uint32_t* d_words = nullptr;
    uint32_t next_slot = 0;
    igxrt_launch_params params{};
    // Staging for IGXRT_TRACE_HOST_MEMORY calls on host memory the kernels
    // cannot address (grown on demand).
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    // The device loads and stores pageable host memory through the host's
    // page tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables).
    bool pageable_access = false;
};

struct igxrt_scene {
    int device = 0;
    igxrt_bvh_info info{};
    void* d_mem = nullptr;
    const void* nodes[IGXRT_LAYOUT_COUNT] = {nullptr, nullptr, nullptr};
    uint32_t node_count[IGXRT_LAYOUT_COUNT] = {0, 0, 0};
    const igxrt_prim_record* prims = nullptr;
    const igxrt_triangle* tris = nullptr;
    // mixed scenes: spheres and cubes are in the tree, planes are not
    bool mixed = false;
    const float* planes = nullptr;  // 4 floats per plane
    uint32_t plane_count = 0;
    uint32_t plane_base = 0;        // object id of the first plane
    // refit: the parent of every node per layout (kNoParent at the root), and
    // kRefitStateWords state words followed by one arrival counter per node
    // of BVH2, then of BVH4 (zeroed before each refit)
    const uint32_t* parents[IGXRT_LAYOUT_COUNT] = {nullptr, nullptr, nullptr};
    uint32_t* refit_words = nullptr;
    // BVH8 slots' sources in the BVH2 layout (8 per BVH8 node), for the refit
    const uint32_t* src8 = nullptr;
    // GPU refit scratch, two float4 per record ({box lo, leaf_end}, {box hi,
    // 0}), written by the record pass and read by the node climb; allocated
    // at the scene's first GPU refit, freed with the scene
    float4* refit_boxes = nullptr;
    // GPU refit scratch, two float4 per node of BVH2, then of BVH4: the union
    // of the node's slot boxes ({lo, 0}, {hi, 0}), written by the climb for
    // the parent's thread; allocated and freed with refit_boxes
    float4* refit_unions = nullptr;

    // A layout can be traced when the tree has it; an empty scene has none
    // and traces as all misses in every layout.
    bool has_layout(uint32_t layout) const {
        return layout < IGXRT_LAYOUT_COUNT &&
               (node_count[layout] > 0 || info.triangle_count + info.sphere_count + info.cube_count == 0);
    }
};

namespace igxrt {

constexpr uint32_t kQueueSlots = 4096;
constexpr uint32_t kNoParent = 0xffffffffu;
constexpr uint32_t kRefitStateWords = 8;

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// One device allocation for a scene of `info`'s primitive counts and n2 / n4
// / n8 nodes; every pointer of the scene is set, the contents are unwritten.
igxrt_status allocate_scene(igxrt_context* ctx, const igxrt_bvh_info& info, uint32_t n2, uint32_t n4,
                            uint32_t n8, igxrt_scene*& out);

// Parent links of both layouts, computed on the host at scene creation and
// stored after the scene's other buffers (see refit.cu).
void node_parents(const igxrt_bvh& bvh, std::vector<uint32_t>& parents2,
                  std::vector<uint32_t>& parents4);

// Camera rays as a traversal launch's ray source: ray i is the primary ray
// of pixel (i mod width, i / width) (igxrt_trace_gbuffer's first step).
struct CameraSource {
    igxrt_camera cam;
    float inv_w, inv_h;
};

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
    // non-null: the number of rays is this device word (written by an earlier
    // kernel on the stream), at most `count`, which sizes the launch
    const uint32_t* count_dev = nullptr;
    // IGXRT_TRACE_INDEPENDENT: the kernel need not wait for the kernel
    // queued before it on the stream
    bool independent = false;
    // non-null: the rays are this camera's, one per pixel (closest hit on a
    // triangle scene; `rays` and `prev` unused)
    const CameraSource* camera = nullptr;
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

// Device descriptor of one batch item (see batch.cu).
struct BatchItemDev {
    const float4* nodes;
    const float4* prims;
    const igxrt_ray* rays;
    const uint32_t* prev;
    void* out;
    const float4* planes;   // mixed scenes: the planes outside the tree (else NULL)
    uint32_t count;
    uint32_t mode;
    uint32_t node_count;
    uint32_t packet_begin;  // first packet of this item in the batch's packet space
    uint32_t plane_count;
    uint32_t plane_base;    // object id of the scene's first plane
};

// Fills the device table of `count` items; `mixed` is set when an item's
// scene holds spheres, cubes or planes (the batch then runs the mixed kernel,
// which traces triangle-only items as well).
igxrt_status build_batch_table(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                               const igxrt_launch_params& p, std::vector<BatchItemDev>& table,
                               uint32_t& total_packets, uint64_t& total_rays, bool& mixed);
// One item table entry for rays [first, first + count) of a scene (the
// server's request slices); `rays`, `prev` and `out` already point at the
// slice's first element.
void batch_item_for(const igxrt_scene* scene, const igxrt_launch_params& p, const igxrt_ray* rays,
                    const uint32_t* prev, void* out, uint32_t count, uint32_t mode, BatchItemDev& d);
// `times` (optional, device memory): the earliest CTA start and the latest
// warp exit of the launch, %globaltimer nanoseconds, folded in by atomicMin /
// atomicMax (the caller sets them to ~0 and 0 first).
igxrt_status launch_batch(igxrt_context* ctx, const BatchItemDev* d_table, uint32_t count,
                          uint32_t total_packets, uint64_t total_rays, const igxrt_launch_params& p,
                          uint32_t* queue, cudaStream_t stream, bool mixed,
                          unsigned long long* times = nullptr);

// Next work-queue counter of the context (a ring of kQueueSlots words); the
// slot's exit counter is exit_word(slot).
uint32_t* take_queue_slot(igxrt_context* ctx);
inline uint32_t* exit_word(uint32_t* queue_slot) { return queue_slot + kQueueSlots + 1; }
uint32_t* status_word(igxrt_context* ctx);

// Opts a kernel into more than 48 KB of dynamic shared memory when `smem`
// needs it (the traversal stacks of deep shared stacks and large blocks).
inline cudaError_t allow_smem(const void* kernel, size_t smem) {
    if (smem <= 48 * 1024)
        return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Scene belongs to the context's device.
igxrt_status check_scene(igxrt_context* ctx, const igxrt_scene* scene);
// Grows the context's staging buffer for host-memory calls to `bytes`.
igxrt_status grow_stage(igxrt_context* ctx, size_t bytes);
// Reads and clears the context's kernel error word (synchronous).
igxrt_status read_status(igxrt_context* ctx);

// True when a kernel may dereference p: device, managed or mapped pinned
// memory (NULL counts as accessible).  Pageable host memory is not.
bool device_accessible(const void* p);

// True when the context's kernels may load and store p in place for a
// host-memory call: device or managed memory, pinned host memory mapped at
// the same address, or any host memory when the device reads pageable memory
// through the host's page tables (Grace over NVLink-C2C).  NULL counts.
bool host_direct(const igxrt_context* ctx, const void* p);

// Flags of a trace-like call: IGXRT_TRACE_HOST_MEMORY, IGXRT_TRACE_STAGED
// only together with it, and the bits of `extra` the call also takes.
igxrt_status check_trace_flags(igxrt_context* ctx, uint32_t flags, uint32_t extra = 0);

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
