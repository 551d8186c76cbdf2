/*
 * ref_shim.cpp — host build of igx_raytracing's own traversal shaders.
 *
 * TEST INFRASTRUCTURE ONLY.  The recipe in oracle/Makefile (target `ref`)
 * compiles this file against the reference's res/shaders/defines.glsl,
 * primitive.glsl (with `inout T name` rewritten to `T &name`) and trace.glsl,
 * so traceGeometry / traceOcclusion below are the reference's code, run on
 * the CPU.  Its outputs pin the oracle restatement in trace_oracle.c and the
 * golden fixtures under tests/golden/.
 *
 * scene.glsl, camera.glsl and rand_util.glsl are GLSL interface blocks and
 * sampling code that trace.glsl includes but does not need for traversal;
 * their include guards are predefined and the buffers they declare
 * (sceneInfo, triangles, spheres, cubes, planes: scene.glsl:6-39) are
 * provided here as host pointers.
 */
#include "glsl_compat.hpp"

#define RAND_UTIL
#define CAMERA
#define SCENE

#include "defines.glsl"
#include "primitive.glsl"

/* scene.glsl:6-20 */
struct SceneInfo {
    uint lightCount;
    uint materialCount;
    uint triangleCount;
    uint sphereCount;
    uint cubeCount;
    uint planeCount;
    uint directionalLightCount;
    uint spotLightCount;
    uint pointLightCount;
};

static thread_local SceneInfo sceneInfo;
static thread_local const Triangle* triangles;
static thread_local const vec4* spheres;
static thread_local const Cube* cubes;
static thread_local const vec4* planes;

#include "trace.glsl"

extern "C" {

/* Scene arrays in the std430 layouts of scene.glsl (Triangle 48 B, sphere
 * vec4 16 B, Cube 24 B, plane vec4 16 B). */
typedef struct igxref_scene {
    const void* triangles;
    uint32_t triangle_count;
    const void* spheres;
    uint32_t sphere_count;
    const void* cubes;
    uint32_t cube_count;
    const void* planes;
    uint32_t plane_count;
} igxref_scene;

/* One full GLSL Hit (primitive.glsl:9-21) flattened. */
typedef struct igxref_hit {
    float rayDir[3];
    float hitT;
    float uv[2];
    uint32_t object;
    float geometryNormal[3];
    float objectNormal[3];
} igxref_hit;

static void bind(const igxref_scene* s) {
    memset(&sceneInfo, 0, sizeof(sceneInfo));
    sceneInfo.triangleCount = s->triangle_count;
    sceneInfo.sphereCount = s->sphere_count;
    sceneInfo.cubeCount = s->cube_count;
    sceneInfo.planeCount = s->plane_count;
    triangles = (const Triangle*)s->triangles;
    spheres = (const vec4*)s->spheres;
    cubes = (const Cube*)s->cubes;
    planes = (const vec4*)s->planes;
}

/* rays: n records of {pos xyz, dir xyz} (6 floats). */
void igxref_trace_geometry(const igxref_scene* s, const float* rays, const uint32_t* prev,
                           uint32_t n, igxref_hit* out) {
    bind(s);
    for (uint32_t i = 0; i < n; ++i) {
        Ray r;
        r.pos = vec3(rays[6 * i + 0], rays[6 * i + 1], rays[6 * i + 2]);
        r.dir = vec3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
        const Hit h = traceGeometry(r, prev ? prev[i] : noRayHit);
        igxref_hit* o = &out[i];
        o->rayDir[0] = h.rayDir.x;
        o->rayDir[1] = h.rayDir.y;
        o->rayDir[2] = h.rayDir.z;
        o->hitT = h.hitT;
        o->uv[0] = h.uv.x;
        o->uv[1] = h.uv.y;
        o->object = h.object;
        o->geometryNormal[0] = h.geometryNormal.x;
        o->geometryNormal[1] = h.geometryNormal.y;
        o->geometryNormal[2] = h.geometryNormal.z;
        o->objectNormal[0] = h.objectNormal.x;
        o->objectNormal[1] = h.objectNormal.y;
        o->objectNormal[2] = h.objectNormal.z;
    }
}

void igxref_trace_occlusion(const igxref_scene* s, const float* rays, const float* max_dist,
                            const uint32_t* prev, uint32_t n, uint32_t* out) {
    bind(s);
    for (uint32_t i = 0; i < n; ++i) {
        Ray r;
        r.pos = vec3(rays[6 * i + 0], rays[6 * i + 1], rays[6 * i + 2]);
        r.dir = vec3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
        out[i] = traceOcclusion(r, max_dist[i], prev ? prev[i] : noRayHit) ? 1u : 0u;
    }
}

/* encodeNormal (primitive.glsl:85-88), for the G-buffer output encoding. */
void igxref_encode_normal(const float* n, uint32_t count, uint32_t* out2) {
    for (uint32_t i = 0; i < count; ++i) {
        const uvec2 e = encodeNormal(vec3(n[3 * i], n[3 * i + 1], n[3 * i + 2]));
        out2[2 * i] = e.x;
        out2[2 * i + 1] = e.y;
    }
}

/* decodeSpheremap (primitive.glsl:95-104). */
void igxref_decode_spheremap(const uint32_t* packed, uint32_t count, float* out3) {
    for (uint32_t i = 0; i < count; ++i) {
        const vec3 v = decodeSpheremap(packed[i]);
        out3[3 * i] = v.x;
        out3[3 * i + 1] = v.y;
        out3[3 * i + 2] = v.z;
    }
}

}
