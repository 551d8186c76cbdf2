/*
 * igxrt.h — C ABI of the GB300 ray-query engine.
 *
 * This boundary replaces the compute dispatches through which igx_raytracing
 * runs its ray queries:
 *
 *   - RaygenTask::prepareCommandList  (src/rt/task/raygen_task.cpp:88-94)
 *       BindDescriptors + BindPipeline + Dispatch(W,H) of res/shaders/raygen.comp,
 *       whose per-thread body is traceGeometry (res/shaders/trace.glsl:9-66);
 *   - ShadowTask::prepareCommandList  (src/rt/task/shadow_task.cpp:194-213)
 *       Dispatch(W,H,samples) of res/shaders/nv_all.shadow.comp, whose
 *       per-thread body is traceOcclusion (res/shaders/trace.glsl:70-98);
 *   - the scene buffers bound by SceneGraph::getDescriptors()
 *       (res/shaders/scene.glsl:22-52; the SceneGraph class lives in the igx
 *       submodule, which the reference checkout leaves empty).
 *
 * The reference loops linearly over every primitive; this engine builds a BVH
 * (on the host, or on the GPU for per-frame geometry) and traverses it with
 * CUDA kernels for sm_103a.  The result of
 * every query equals the linear loop's: the closest hit is the smallest t
 * accepted by the reference's triangle test (res/shaders/primitive.glsl:239-284),
 * ties going to the lowest primitive index (the loop runs in index order and
 * accepts only t < hit.hitT).
 *
 * Conventions
 *   - Every call returns igxrt_status; nothing throws across the ABI.
 *   - igxrt_last_error(ctx) holds a message for the last failing call on ctx.
 *   - The caller owns all arrays it passes.  The library owns device memory of
 *     scenes and BVHs and the staging buffers of host-memory traces.
 *   - Trace calls are ordered on the CUDA stream passed as `stream`
 *     (a cudaStream_t cast to void*; NULL = the legacy default stream).
 *     Without IGXRT_TRACE_HOST_MEMORY they return as soon as the work is queued.
 *   - A context is used by one host thread at a time.  Scenes change only
 *     through igxrt_scene_refit and may be traced from any context on the
 *     same device.
 */
#ifndef IGXRT_H
#define IGXRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IGXRT_ABI_VERSION 3u

/* res/shaders/primitive.glsl:6-7: the miss distance and the "no object" id. */
#define IGXRT_NO_HIT 3.4028235e38f
#define IGXRT_NO_RAY_HIT 0xFFFFFFFFu

typedef enum igxrt_status {
    IGXRT_OK = 0,
    IGXRT_ERROR_INVALID_ARGUMENT = 1,
    IGXRT_ERROR_CUDA = 2,
    IGXRT_ERROR_OUT_OF_MEMORY = 3,
    IGXRT_ERROR_INVALID_BVH = 4,
    IGXRT_ERROR_KERNEL_STATUS = 5,  /* a kernel raised its error word */
    IGXRT_ERROR_ADMISSION = 6,      /* request can never fit the memory cap */
    IGXRT_ERROR_TIMEOUT = 7,
    IGXRT_ERROR_UNSUPPORTED = 8,
    IGXRT_ERROR_NOT_READY = 9,
    IGXRT_ERROR_IO = 10
} igxrt_status;

/*
 * Triangle record, 48 bytes: the std430 layout of GLSL `struct Triangle`
 * (res/shaders/primitive.glsl:28-38).  n0..n2 are per-vertex normals packed
 * as two halves (decoded by decodeSpheremap, primitive.glsl:95-104); the
 * traversal ignores them.
 */
typedef struct igxrt_triangle {
    float p0[3];
    uint32_t n0;
    float p1[3];
    uint32_t n1;
    float p2[3];
    uint32_t n2;
} igxrt_triangle;

/*
 * Ray, 32 bytes: the std430 layout of GLSL `struct Ray { vec3 pos; vec3 dir; }`
 * (primitive.glsl:23-26) with the two padding words used for the interval.
 * A triangle is accepted when t > tmin (the reference rejects t <= 0,
 * primitive.glsl:276, so tmin = 0 reproduces it) and t < min(tmax, IGXRT_NO_HIT)
 * (the reference starts hit.hitT at noHit, trace.glsl:14; for the any-hit
 * query tmax is traceOcclusion's maxDist, trace.glsl:70,97).
 * The direction need not be normalised; t is in units of |dir|.
 */
typedef struct igxrt_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} igxrt_ray;

/*
 * Closest-hit record, 16 bytes: the fields of GLSL `struct Hit`
 * (primitive.glsl:9-21) that the traversal decides: hitT, uv and object.
 * A miss is {IGXRT_NO_HIT, 0, 0, IGXRT_NO_RAY_HIT}.
 */
typedef struct igxrt_hit {
    float t;
    float u;
    float v;
    uint32_t prim;
} igxrt_hit;

/* ---- BVH layouts (device and export format) ---------------------------- */

/* Node layouts the builder can emit. */
#define IGXRT_LAYOUT_BVH2 0u /* binary, 64-byte nodes holding both child boxes */
#define IGXRT_LAYOUT_BVH4 1u /* 4-wide, 128-byte nodes holding four child boxes */
#define IGXRT_LAYOUT_BVH8 2u /* 8-wide, 96-byte nodes with 8-bit quantized child boxes */
#define IGXRT_LAYOUT_COUNT 3u

/*
 * BVH2 node, 64 bytes, 64-byte aligned; read as four 128-bit loads.
 * Child c's box is [x[c][0],x[c][1]] x [y[c][0],y[c][1]] x [z[c][0],z[c][1]],
 * already widened outward by the builder's padding.  child[c] >= 0 is the
 * index of an interior node; child[c] < 0 is a leaf whose first primitive
 * record is ~child[c]; the leaf runs to the record flagged leaf_end.
 * An absent child has the box {+inf,+inf} on every axis, which no ray enters.
 */
typedef struct igxrt_bvh2_node {
    float c0_x[2], c0_y[2];
    float c1_x[2], c1_y[2];
    float c0_z[2], c1_z[2];
    int32_t child[2];
    uint32_t pad[2];
} igxrt_bvh2_node;

/*
 * BVH4 node, 128 bytes, 128-byte aligned; read as eight 128-bit loads.
 * Per axis a, lo[a][i] / hi[a][i] is child i's slab.  child[i] as in BVH2;
 * unused slots carry the {+inf,+inf} box.
 */
typedef struct igxrt_bvh4_node {
    float lo_x[4], hi_x[4];
    float lo_y[4], hi_y[4];
    float lo_z[4], hi_z[4];
    int32_t child[4];
    uint32_t pad[4];
} igxrt_bvh4_node;

/*
 * BVH8 node, 96 bytes, 32-byte aligned; read as three 256-bit loads.  Child
 * c's box on axis a is [origin[a] + lo_a[c] * 2^exp[a], origin[a] + hi_a[c] *
 * 2^exp[a]], each bound decoded as fmaf(q, 2^exp[a], origin[a]) in binary32;
 * the builder rounds the bytes outward so the decoded box contains the child's
 * padded box.  Bit c of `valid` marks a used slot; child[c] as in BVH2.
 */
typedef struct igxrt_bvh8_node {
    float origin[3];
    int8_t exp[3];
    uint8_t valid;
    uint8_t lo_x[8], hi_x[8];
    uint8_t lo_y[8], hi_y[8];
    uint8_t lo_z[8], hi_z[8];
    int32_t child[8];
} igxrt_bvh8_node;

/*
 * Primitive record, 48 bytes, in leaf order.  e1 = p1 - p0 and e2 = p2 - p0
 * are the same binary32 subtractions rayIntersectTri performs
 * (primitive.glsl:245-246), stored so the kernel does not repeat them.
 */
typedef struct igxrt_prim_record {
    float p0[3];
    uint32_t prim;     /* index of the triangle in the caller's array */
    float e1[3];
    uint32_t leaf_end; /* 1 on the last record of a leaf, else 0 */
    float e2[3];
    uint32_t pad;
} igxrt_prim_record;

/* std430 layout of GLSL `struct Cube` (primitive.glsl:40-44): corners
 * start = (xy0[0], xy0[1], z0_x1[0]), end = (z0_x1[1], yz1[0], yz1[1]). */
typedef struct igxrt_cube {
    float xy0[2];
    float z0_x1[2];
    float yz1[2];
} igxrt_cube;

/*
 * All primitive buffers of a reference scene (res/shaders/scene.glsl:22-39):
 * triangles, spheres (4 floats: centre xyz, radius w), cubes and planes
 * (4 floats: normal xyz, offset w).  Object ids are global in that order:
 * triangle i is i, sphere i is triangle_count + i, and so on
 * (the loops of trace.glsl:22-46).
 */
typedef struct igxrt_scene_desc {
    const igxrt_triangle* triangles;
    uint32_t triangle_count;
    uint32_t sphere_count;
    const float* spheres;
    const igxrt_cube* cubes;
    uint32_t cube_count;
    uint32_t plane_count;
    const float* planes;
} igxrt_scene_desc;

typedef struct igxrt_build_options {
    uint32_t max_leaf_size; /* 0 = 8; at most 16 */
    uint32_t sah_bins;      /* 0 = 32 */
    float node_cost;        /* SAH cost of a node visit, 0 = 1.0 */
    float tri_cost;         /* SAH cost of a triangle test, 0 = 1.0 */
    uint32_t threads;       /* host build threads, 0 = all cores */
    uint32_t reserved[3];
} igxrt_build_options;

typedef struct igxrt_bvh_info {
    uint32_t triangle_count;
    uint32_t bvh2_nodes;
    uint32_t bvh4_nodes;
    uint32_t leaf_count;
    uint32_t max_depth;
    uint32_t max_leaf_size;
    float sah_cost;
    float bounds[6]; /* min xyz, max xyz of the triangles */
    float pad_abs;   /* absolute outward padding added to every node box */
    uint32_t max_stack[IGXRT_LAYOUT_COUNT]; /* deepest traversal stack per layout */
    uint32_t bvh8_nodes; /* 0: the tree has no BVH8 layout (GPU builds) */
    uint64_t device_bytes;
    uint32_t sphere_count, cube_count, plane_count;
    uint32_t reserved;
} igxrt_bvh_info;

typedef struct igxrt_bvh igxrt_bvh;
typedef struct igxrt_context igxrt_context;
typedef struct igxrt_scene igxrt_scene;

/* ---- Host-side BVH (no GPU needed) --------------------------------------- */

/* Builds a binned-SAH BVH over `count` triangles on the host (count may be 0).
 * Rejects non-finite vertex coordinates with IGXRT_ERROR_INVALID_ARGUMENT. */
igxrt_status igxrt_bvh_build(const igxrt_triangle* tris, uint32_t count,
                             const igxrt_build_options* opts, igxrt_bvh** out);
/* Builds one BVH over triangles, spheres and cubes of a mixed scene; planes
 * are unbounded and stay outside the tree (tested by every ray).  Primitive
 * records of spheres hold {centre, id}{radius, 0, 0, leaf_end}{0, 0, 0, 1},
 * of cubes {start, id}{end, leaf_end}{0, 0, 0, 2}; the last word of a
 * record is its type (0 triangle, 1 sphere, 2 cube). */
igxrt_status igxrt_bvh_build_mixed(const igxrt_scene_desc* desc, const igxrt_build_options* opts,
                                   igxrt_bvh** out);
igxrt_status igxrt_bvh_destroy(igxrt_bvh* bvh);
igxrt_status igxrt_bvh_get_info(const igxrt_bvh* bvh, igxrt_bvh_info* info);
/* Borrowed pointers to the node array of `layout` and the primitive records;
 * valid until igxrt_bvh_destroy. */
igxrt_status igxrt_bvh_get_data(const igxrt_bvh* bvh, uint32_t layout,
                                const void** nodes, uint64_t* node_count,
                                const igxrt_prim_record** prims, uint64_t* prim_count);
/* Checks structure and boxes: every triangle in exactly one leaf, every child
 * box contains its subtree, node indices in range, depth within the limit. */
igxrt_status igxrt_bvh_validate(const igxrt_bvh* bvh, char* msg, size_t msg_len);
/* Moves the primitives of a built BVH (same counts as at the build: an
 * animated frame) and recomputes the primitive records and every node box,
 * keeping the tree topology.  The boxes follow the builder's rule (bounds of
 * the subtree widened by 2^-18 * max|coordinate|), so a refit BVH is exactly
 * what the builder would emit for this topology. */
igxrt_status igxrt_bvh_refit(igxrt_bvh* bvh, const igxrt_scene_desc* desc);
/* Serialises a built BVH (both layouts and the triangle array) to a file and
 * loads it back, so a server can warm-start without rebuilding. */
igxrt_status igxrt_bvh_save(const igxrt_bvh* bvh, const char* path);
igxrt_status igxrt_bvh_load(const char* path, igxrt_bvh** out);

/* ---- Context and resident scenes ---------------------------------------- */

igxrt_status igxrt_create(int device, igxrt_context** out);
igxrt_status igxrt_destroy(igxrt_context* ctx);
const char* igxrt_last_error(const igxrt_context* ctx);
/* Static description of a status code. */
const char* igxrt_status_string(igxrt_status status);

/* Builds the BVH on the host and uploads nodes, primitive records and the
 * triangle array to the context's device. */
igxrt_status igxrt_scene_create(igxrt_context* ctx, const igxrt_triangle* tris,
                                uint32_t count, const igxrt_build_options* opts,
                                igxrt_scene** out);
/* Builds and uploads a mixed scene.  igxrt_trace_closest and igxrt_trace_any
 * then follow the reference's rules per primitive type (rayIntersectSphere,
 * rayIntersectCube, rayIntersectPlane, primitive.glsl:173-333): a sphere hit
 * needs t >= tmin, a plane hit t >= tmin, a cube hit only tmax >= tmin (a
 * cube around the origin is hit at its negative entry distance), and at equal
 * t a cube beats any other primitive and the later of two cubes wins (the
 * cube test rejects only tmin > hit.hitT).  Every pass takes mixed scenes:
 * batches, the server, the shadow mask and the G-buffer (whose object normal
 * of a sphere, cube or plane is its geometry normal, trace.glsl:59-63). */
igxrt_status igxrt_scene_create_mixed(igxrt_context* ctx, const igxrt_scene_desc* desc,
                                      const igxrt_build_options* opts, igxrt_scene** out);
/* Uploads an already built BVH. */
igxrt_status igxrt_scene_create_from_bvh(igxrt_context* ctx, const igxrt_bvh* bvh,
                                         igxrt_scene** out);
/*
 * Builds the BVH on the GPU (a linear BVH: Morton order and radix tree) for
 * geometry that changes every frame; no reference counterpart (the reference
 * re-uploads its scene per frame, test/scene/niels_scene.cpp:61-70, and has no
 * acceleration structure).  Same node formats, records, padding rule and
 * query results as igxrt_scene_create_mixed; the tree differs (Morton splits,
 * not SAH), so traversal visits more nodes.  Primitive buffers are device
 * pointers, or host pointers with IGXRT_TRACE_HOST_MEMORY.  opts: only
 * max_leaf_size is used (0 = 4): a subtree of at most that many objects
 * becomes one leaf.  The work is ordered on `stream`; the call returns once
 * the scene is ready.
 */
igxrt_status igxrt_scene_create_gpu(igxrt_context* ctx, const igxrt_scene_desc* desc,
                                    const igxrt_build_options* opts, uint32_t flags, void* stream,
                                    igxrt_scene** out);
igxrt_status igxrt_scene_destroy(igxrt_scene* scene);
/*
 * GPU refit for per-frame animation (the reference re-uploads moving spheres
 * every frame, test/scene/niels_scene.cpp:61-70): new primitive buffers with
 * the counts of the scene's creation (device pointers, or host pointers with
 * IGXRT_TRACE_HOST_MEMORY) replace the old ones; primitive records and node
 * boxes of both layouts are recomputed on the GPU bottom-up, the topology is
 * kept.  The result equals igxrt_bvh_refit on the host.  The work is ordered
 * on `stream` after what the caller queued there (e.g. the kernel that moved
 * the geometry), and the call returns once it has finished, so the status can
 * report a non-finite coordinate (IGXRT_ERROR_INVALID_ARGUMENT; the scene is
 * then left unchanged) and igxrt_scene_get_info sees the new bounds.  Traces
 * of the scene must not overlap the refit on another stream.
 */
igxrt_status igxrt_scene_refit(igxrt_context* ctx, igxrt_scene* scene, const igxrt_scene_desc* desc,
                               uint32_t flags, void* stream);
/* Copies a resident scene (both layouts, records, primitive buffers, info)
 * into a new host BVH and validates it, e.g. to save a GPU-built or refit
 * tree for a warm start (synchronous; free with igxrt_bvh_destroy). */
igxrt_status igxrt_scene_download(igxrt_context* ctx, const igxrt_scene* scene, igxrt_bvh** out);
/* Copies a resident scene's nodes of `layout` and its primitive records to
 * host arrays (sizes from igxrt_scene_get_info; synchronous). */
igxrt_status igxrt_scene_read_bvh(igxrt_context* ctx, const igxrt_scene* scene, uint32_t layout,
                                  void* nodes, uint64_t node_count, igxrt_prim_record* prims,
                                  uint64_t prim_count);
igxrt_status igxrt_scene_get_info(const igxrt_scene* scene, igxrt_bvh_info* info);

/* ---- Ray queries --------------------------------------------------------- */

/* rays, prev_hit and the output are host pointers; the call returns once the
 * results are in host memory.  When the kernels can address every one of
 * them (pinned memory, or any host memory on a device that reads pageable
 * memory through the host's page tables, as a GB300 does over NVLink-C2C)
 * the kernels load the rays and store the results in place, each once;
 * otherwise the call stages them through device buffers.  Trace, fetch
 * count, G-buffer, camera-ray and shadow-mask calls take the flag. */
#define IGXRT_TRACE_HOST_MEMORY 1u
/* With IGXRT_TRACE_HOST_MEMORY (trace, G-buffer, camera-ray and shadow-mask
 * calls): stage the host arrays through device buffers even when the kernels
 * could address them in place. */
#define IGXRT_TRACE_STAGED 2u
/* igxrt_trace_closest / igxrt_trace_any on device memory: the caller states
 * that this call reads nothing the kernel queued just before it on `stream`
 * writes, and writes nothing that kernel reads or writes (e.g. shadow rays
 * traced after bounce rays, both made from the same primary hits).  The
 * traversal kernel may then start while that kernel drains its last rays
 * (programmatic dependent launch).  Without the flag a trace kernel starts
 * its work only after the kernel before it has finished and its writes are
 * visible, as for any stream-ordered launch. */
#define IGXRT_TRACE_INDEPENDENT 4u

/* Launch shape of the traversal kernels. Zero fields take the defaults. */
typedef struct igxrt_launch_params {
    uint32_t block_size;  /* threads per CTA: 64, 128 or 256; 0 = 128 */
    uint32_t stack_depth; /* shared-memory stack entries per thread (at most 64);
                             deeper entries spill to local memory; 0 = 16 */
    uint32_t packet_size; /* rays a warp claims per queue fetch: a multiple of
                             8 up to 4096; 0 = 16 */
    uint32_t layout;      /* IGXRT_LAYOUT_* */
    uint32_t ctas_per_sm; /* persistent CTAs per SM, 0 = as many as fit */
    uint32_t refill_lanes;/* a warp refetches rays once this many of its lanes
                             are idle (1..32); 0 = 8 */
    uint32_t phase_break; /* a warp's lanes descend through interior nodes
                             together, then test their leaves together; the
                             descent ends early once phase_break times the
                             lanes still descending is at most the number of
                             lanes waiting (at a leaf, or done), and those
                             lanes resume after the leaves.  1..31; 32 = no
                             early end (every lane reaches a leaf first);
                             0 = 2.  Results do not depend on it. */
    uint32_t reserved;
} igxrt_launch_params;

igxrt_status igxrt_set_launch_params(igxrt_context* ctx, const igxrt_launch_params* p);
igxrt_status igxrt_get_launch_params(const igxrt_context* ctx, igxrt_launch_params* p);

/*
 * Closest hit (traceGeometry, trace.glsl:9-66) for `count` rays.
 * prev_hit may be NULL; otherwise prev_hit[i] is a triangle index that ray i
 * must not hit (the reference's prevHit; IGXRT_NO_RAY_HIT excludes nothing).
 */
igxrt_status igxrt_trace_closest(igxrt_context* ctx, const igxrt_scene* scene,
                                 const igxrt_ray* rays, const uint32_t* prev_hit,
                                 uint32_t count, igxrt_hit* hits, uint32_t flags,
                                 void* stream);

/*
 * Occlusion (traceOcclusion, trace.glsl:70-98): occluded[i] = 1 when some
 * triangle other than prev_hit[i] is accepted with tmin < t < tmax, else 0.
 * The kernel stops at the first such triangle.
 */
igxrt_status igxrt_trace_any(igxrt_context* ctx, const igxrt_scene* scene,
                             const igxrt_ray* rays, const uint32_t* prev_hit,
                             uint32_t count, uint32_t* occluded, uint32_t flags,
                             void* stream);

/*
 * Closest hit for host arrays without allocating anything.  This entry point
 * has no counterpart in the reference: it serves callers that must not call
 * cudaMalloc while they trace, such as a render loop whose device memory is
 * budgeted by another allocator or whose frame time cannot absorb the
 * device-wide synchronisation an allocation may cause.  igxrt_trace_closest
 * with IGXRT_TRACE_HOST_MEMORY may grow its staging buffer with cudaMalloc;
 * this call stages through a fixed 16 MiB device array instead
 * (IGXRT_STATIC_SCRATCH_BYTES, a file-scope __device__ array that every GPU
 * loading the library keeps until the process exits).
 *   - count may not exceed IGXRT_STATIC_MAX_RAYS; larger calls return
 *     IGXRT_ERROR_INVALID_ARGUMENT (with a message in igxrt_last_error) and
 *     launch nothing.  Split bigger batches across calls.
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture begins.
 *   - All calls share the one array.  Each call clears its work counter and
 *     error word before launching, and returns only after its hits are back
 *     in host memory, but calls that overlap on the GPU (from several host
 *     threads or contexts at once) race on the array: serialise them.
 * Inputs and outputs are as for igxrt_trace_closest with host arrays.
 */
#define IGXRT_STATIC_SCRATCH_BYTES (16u << 20)
#define IGXRT_STATIC_MAX_RAYS 320000u
igxrt_status igxrt_trace_closest_static(igxrt_context* ctx, const igxrt_scene* scene,
                                        const igxrt_ray* rays, const uint32_t* prev_hit,
                                        uint32_t count, igxrt_hit* hits, void* stream);

/* ---- Batched multi-scene queries ------------------------------------------ */

#define IGXRT_MODE_CLOSEST 0u
#define IGXRT_MODE_ANY 1u

/* One ray batch of a batched launch.  All pointers are device memory. */
/* A batch item's arrays are device memory, or pinned host memory that the
 * kernel reads and writes in place. */
typedef struct igxrt_batch_item {
    const igxrt_scene* scene;
    const igxrt_ray* rays;
    const uint32_t* prev_hit; /* may be NULL */
    void* out;                /* igxrt_hit[count] (closest) or uint32_t[count] (any) */
    uint32_t count;
    uint32_t mode;            /* IGXRT_MODE_CLOSEST or IGXRT_MODE_ANY */
} igxrt_batch_item;

typedef struct igxrt_batch igxrt_batch;

/*
 * Prepares one persistent launch over `count` items (different scenes, uneven
 * ray counts, closest and any queries mixed): the rays of all items form one
 * work queue of packets, so the GPU stays full across item boundaries.  The
 * item table is uploaded once and the queue reset plus the kernel are
 * captured in a CUDA graph; igxrt_batch_launch replays it.  params NULL
 * takes the context's launch parameters.  Results are identical to tracing
 * each item on its own.
 */
igxrt_status igxrt_batch_create(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                                const igxrt_launch_params* params, igxrt_batch** out);
igxrt_status igxrt_batch_launch(igxrt_batch* batch, void* stream);
igxrt_status igxrt_batch_destroy(igxrt_batch* batch);

/* The same launch without a graph: uploads the item table on `stream` into
 * the context's batch staging and launches once. */
igxrt_status igxrt_trace_batch(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                               void* stream);

/* Autotuner: times candidate launch parameters (node layout, block size,
 * shared stack depth, packet size, refill threshold, phase break) on the given items and
 * returns the fastest.  With a cache file, results are stored under
 * (GPU name, class key) and reused without timing.  By default a candidate
 * is timed as one batched launch over the items (igxrt_trace_batch); with
 * IGXRT_TUNE_PLAIN it is timed as one plain launch per item, in item order,
 * on one stream (the igxrt_trace_closest / igxrt_trace_any path), so the
 * result fits callers that trace the items one call at a time. */
#define IGXRT_TUNE_PLAIN 1u

typedef struct igxrt_tune_options {
    uint32_t reps;         /* timed repetitions per candidate, 0 = 3 */
    uint32_t layouts_mask; /* bit per IGXRT_LAYOUT_*, 0 = all */
    const char* cache_path;/* NULL = no cache */
    const char* class_key; /* cache key of this workload class, NULL = derived */
    uint32_t force;        /* 1 = ignore a cached entry */
    uint32_t flags;        /* IGXRT_TUNE_PLAIN, or 0 */
    uint32_t reserved[2];
} igxrt_tune_options;

igxrt_status igxrt_autotune(igxrt_context* ctx, const igxrt_batch_item* items, uint32_t count,
                            const igxrt_tune_options* opts, igxrt_launch_params* best,
                            float* best_ms);

/* ---- Serving: resident scenes, admission by memory, continuous batching ---- */

typedef struct igxrt_server igxrt_server;

typedef struct igxrt_server_options {
    uint64_t memory_cap_bytes;   /* device bytes for the ray, prev_hit and result
                                    buffers of admitted requests; 0 = 24 GiB */
    uint32_t max_batch_rays;     /* rays coalesced into one launch, 0 = 1M */
    uint32_t max_batch_requests; /* request slices per launch, 0 = 1024 (at most 4096) */
    uint32_t streams;            /* batches in flight at once, 0 = 2 */
    uint32_t slice_rays;         /* a request enters a launch with at most this many
                                    of its rays (the rest go into the next launches,
                                    beside the requests queued behind it), so a large
                                    request cannot hold small ones back; 0 = 256K */
    uint32_t reserved[2];
} igxrt_server_options;

/* A ray-query request.  The arrays are host memory owned by the caller and
 * must stay valid until the request completes.  Pinned memory makes the
 * server's copies asynchronous; a copy to or from pageable memory holds the
 * scheduler thread until it is done, so batches on other streams wait. */
typedef struct igxrt_request {
    uint32_t scene_id;        /* from igxrt_server_add_scene */
    uint32_t mode;            /* IGXRT_MODE_CLOSEST or IGXRT_MODE_ANY */
    uint32_t count;
    uint32_t reserved;
    const igxrt_ray* rays;
    const uint32_t* prev_hit; /* may be NULL */
    void* out;                /* igxrt_hit[count] or uint32_t[count] */
} igxrt_request;

/* Timestamps in seconds since the server started (host steady clock). */
typedef struct igxrt_request_stats {
    double submitted;
    double admitted;  /* its buffers were reserved under the cap */
    double launched;  /* its first slice's batch was queued on a stream */
    double completed; /* all its results were in host memory */
    uint32_t batch;   /* sequence number of the launch that carried its last slice */
    uint32_t status;  /* igxrt_status of the request */
    double arrival;   /* its scheduled arrival (igxrt_server_replay), else = submitted;
                         latency is completed - arrival */
} igxrt_request_stats;

typedef struct igxrt_server_stats {
    uint64_t submitted, completed, rejected;
    uint64_t rays_completed;
    uint64_t batches;
    double p50_ms, p99_ms, mean_ms, max_ms; /* arrival -> completed */
    double first_submit, last_complete;     /* seconds since start */
    uint64_t peak_memory_bytes;             /* peak reserved under the cap */
    uint32_t peak_pending;                  /* most requests waiting for admission */
    uint32_t peak_in_flight_batches;
} igxrt_server_stats;

/* Starts a server on the context's device (one scheduler thread).  The
 * context must not be used by other threads while the server runs. */
igxrt_status igxrt_server_create(igxrt_context* ctx, const igxrt_server_options* opts,
                                 igxrt_server** out);
/* Registers a resident scene (triangle-only or mixed); it must outlive the
 * server.  Scenes without the server's node layout are refused with
 * IGXRT_ERROR_UNSUPPORTED. */
igxrt_status igxrt_server_add_scene(igxrt_server* server, const igxrt_scene* scene,
                                    uint32_t* scene_id);
/* Queues a request and returns at once.  A request whose buffers can never
 * fit the memory cap is refused with IGXRT_ERROR_ADMISSION; others wait in
 * FIFO order until their buffers fit. */
igxrt_status igxrt_server_submit(igxrt_server* server, const igxrt_request* req, uint64_t* ticket);
/* Submits `count` requests at scheduled times, pacing them natively on the
 * calling thread: request i is submitted once arrival_s[i] seconds have passed
 * since the call began (a sleep, then a spin for the last 200 us), and its
 * latency is counted from that scheduled time, so a late submission counts
 * against the server.  tickets[i] receives its ticket (0 when refused with
 * IGXRT_ERROR_ADMISSION, which the call skips).  Returns after the last
 * submission; the requests complete as usual. */
igxrt_status igxrt_server_replay(igxrt_server* server, const igxrt_request* reqs,
                                 const double* arrival_s, uint32_t count, uint64_t* tickets);
/* Blocks until the request completes (IGXRT_ERROR_TIMEOUT after timeout_s,
 * < 0 = no limit); stats may be NULL. */
igxrt_status igxrt_server_wait(igxrt_server* server, uint64_t ticket, double timeout_s,
                               igxrt_request_stats* stats);
igxrt_status igxrt_server_get_stats(igxrt_server* server, igxrt_server_stats* stats);
/* Device-side interval of one completed batch launch: the earliest CTA start
 * and the latest warp exit of its kernel, read from %globaltimer by the kernel
 * itself (nanoseconds, one clock for all streams), so intervals of batches on
 * different streams show whether their kernels ran at the same time. */
typedef struct igxrt_batch_time {
    uint64_t start_ns;
    uint64_t end_ns;
    uint32_t batch;    /* sequence number, as igxrt_request_stats.batch */
    uint32_t stream;   /* the server's stream slot it ran on */
    uint64_t rays;
} igxrt_batch_time;
/* Copies the intervals of up to `max_batches` completed batches, in
 * completion order, and sets *count to the number copied. */
igxrt_status igxrt_server_batch_times(igxrt_server* server, igxrt_batch_time* times,
                                      uint32_t max_batches, uint32_t* count);
/* Finishes all queued work, then stops the scheduler and frees its memory. */
igxrt_status igxrt_server_destroy(igxrt_server* server);

/*
 * Fused shadow pass: nv_all.shadow.comp (res/shaders/nv_all.shadow.comp:50-142)
 * as one kernel.  One any-hit ray per pixel and sample; the results are packed
 * into the 32-bit ballot words the lighting pass reads (light_rt.glsl:17-28):
 * a word per 16x2 pixel tile and sample at indexToLight(loc, res, sample)
 * (light.glsl:221-229) = tile.x + tile.y*tiles_x + sample*tiles_x*tiles_y with
 * tiles_x = ceil(width/16), tiles_y = ceil(height/2); pixel (x, y) owns bit
 * (x & 15) | ((y & 1) << 4).
 *   rays:   width*height*samples rays, ray (sample*height + y)*width + x;
 *           its tmax is the shadow distance (traceOcclusion's maxDist).
 *   object: width*height primary objects (dirObject.w of raygen.comp); a
 *           pixel whose object is IGXRT_NO_RAY_HIT casts no ray and its bit is
 *           0; otherwise its rays exclude that object (prevHit).
 *   mask:   tiles_x*tiles_y*samples words, every one written (the shader's
 *           non-DEBUG build leaves all-empty tiles unwritten; here they are 0).
 * The pass compacts the traced rays into the context's staging buffer, so two
 * shadow passes (or a shadow pass and a host-memory call) of one context must
 * not overlap on different streams.
 */
igxrt_status igxrt_trace_shadow_mask(igxrt_context* ctx, const igxrt_scene* scene,
                                     const igxrt_ray* rays, const uint32_t* object,
                                     uint32_t width, uint32_t height, uint32_t samples,
                                     uint32_t* mask, uint32_t flags, void* stream);

/*
 * Camera of the reference's default projection (res/shaders/camera.glsl:14-42):
 * the eye and three corners of the image plane, p0 top left, p1 top right,
 * p2 bottom left.  jitter is added to the pixel index before the division by
 * the resolution (the reference adds rand(loc + seed); 0.5 = pixel centres).
 */
typedef struct igxrt_camera {
    float eye[3];
    uint32_t width;
    float p0[3];
    uint32_t height;
    float p1[3];
    float jitter_x;
    float p2[3];
    float jitter_y;
} igxrt_camera;

/*
 * Primary pass: raygen.comp (res/shaders/raygen.comp:16-52) with the default
 * projection, no ray buffer in between.  For pixel (x, y), y = loc.y:
 *   c = ((x, y) + jitter) * (1/width, 1/height), c.y = 1 - c.y
 *   dir = normalize(p0 + c.x*(p1 - p0) + c.y*(p2 - p0) - eye)   (camera.glsl:72-87, 113-116)
 *   hit = traceGeometry((eye, dir), noRayHit)
 * and the shader's two rgba32f images, row-major (pixel y*width + x):
 *   dir_object = {dir*t, bits(object)} on a hit, {dir, bits(noRayHit)} on a miss (:39-44);
 *   uv_normal  = {u, v, bits(encodeNormal(objectNormal))} on a hit, not written on a miss (:46-51),
 * with objectNormal = interpolate(decodeSpheremap(n0), decodeSpheremap(n1),
 * decodeSpheremap(n2), uv) of the hit triangle (trace.glsl:48-57).  Device
 * images of a triangle scene are written in two kernels (the persistent
 * trace with rays made in the kernel leaves each pixel's hit record in
 * dir_object, then one encoding thread per pixel); mixed scenes and host
 * images written in place use one kernel of 8x4 pixel tiles.
 */
igxrt_status igxrt_trace_gbuffer(igxrt_context* ctx, const igxrt_scene* scene,
                                 const igxrt_camera* camera, float* dir_object, float* uv_normal,
                                 uint32_t flags, void* stream);
/* The primary rays igxrt_trace_gbuffer traces, written as width*height ray
 * records {eye, 0, dir, IGXRT_NO_HIT} in pixel order (the same binary32
 * steps), so the pass can be split into ray generation and
 * igxrt_trace_closest.  rays is device memory, or host memory with
 * IGXRT_TRACE_HOST_MEMORY. */
igxrt_status igxrt_camera_rays(igxrt_context* ctx, const igxrt_camera* camera, igxrt_ray* rays,
                               uint32_t flags, void* stream);

/* Copies `count` device hits to host memory and waits for them. */
igxrt_status igxrt_fetch_hits(igxrt_context* ctx, const igxrt_hit* device_hits,
                              uint32_t count, igxrt_hit* host_hits, void* stream);

/* Waits for the stream and reports a kernel error word raised since the last
 * call (IGXRT_ERROR_KERNEL_STATUS). */
igxrt_status igxrt_sync(igxrt_context* ctx, void* stream);

/*
 * Instrumented traversal: per ray, the number of node records and primitive
 * records the closest (mode 0) or any-hit (mode 1) kernel fetches.  Used for
 * the bytes-per-ray roofline; the traversal order is the production kernel's.
 */
igxrt_status igxrt_count_fetches(igxrt_context* ctx, const igxrt_scene* scene,
                                 const igxrt_ray* rays, const uint32_t* prev_hit,
                                 uint32_t count, uint32_t mode, uint32_t layout,
                                 uint32_t* node_fetches, uint32_t* prim_fetches,
                                 void* stream);

#ifdef __cplusplus
}
#endif

#endif /* IGXRT_H */
