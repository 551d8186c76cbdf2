/*
 * trace_oracle.c — CPU restatement of igx_raytracing's ray-query path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA engine is tested against,
 * and the timed CPU baseline.  The engine never links or calls this file.
 *
 * Arithmetic contract (the same one the CUDA kernels follow):
 *   - IEEE binary32, round to nearest, denormals kept (no flush to zero);
 *   - compiled with -ffp-contract=off: no multiply-add fusion anywhere in the
 *     triangle test;
 *   - GLSL dot(a,b) = a.x*b.x + a.y*b.y + a.z*b.z summed left to right;
 *   - GLSL cross(a,b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
 *   - 1/a is a correctly rounded division.
 * The BVH box test uses explicit fmaf(), which is correctly rounded on the
 * host and on the GPU alike, so both make identical culling decisions.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef struct {
    float x, y, z;
} v3;

static inline v3 mk(const float* p) {
    v3 r = {p[0], p[1], p[2]};
    return r;
}
static inline v3 sub(v3 a, v3 b) {
    v3 r = {a.x - b.x, a.y - b.y, a.z - b.z};
    return r;
}
/* GLSL cross() component order. */
static inline v3 cross(v3 a, v3 b) {
    v3 r = {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
    return r;
}
/* GLSL dot(), summed left to right. */
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

static inline float tmax_effective(float tmax) {
    /* The reference starts hit.hitT at noHit (trace.glsl:14, 73); a larger
     * or NaN tmax therefore behaves as noHit. */
    return tmax < IGXRT_NO_HIT ? tmax : IGXRT_NO_HIT;
}

/* ------------------------------------------------------------------------ */
/* Brute force: traceGeometry / traceOcclusion around rayIntersectTri.      */
/* ------------------------------------------------------------------------ */

typedef struct {
    float hitT;
    float u, v;
    uint32_t object;
    uint32_t events;
    float gn[3]; /* hit.geometryNormal of a sphere, cube or plane hit (the
                    G-buffer's object normal for those, trace.glsl:59-63) */
} hitstate;

/*
 * rayIntersectTri, res/shaders/primitive.glsl:239-284, step for step.
 * `tmin` generalises the reference's `t <= 0` rejection (tmin = 0 there).
 */
static int ray_intersect_tri(v3 pos, v3 dir, float tmin, const igxrt_triangle* tri,
                             uint64_t obj, uint64_t prevObj, hitstate* hit) {
    const v3 p0 = mk(tri->p0);
    const v3 p1 = mk(tri->p1);
    const v3 p2 = mk(tri->p2);

    const v3 p1_p0 = sub(p1, p0); /* :245 */
    const v3 p2_p0 = sub(p2, p0); /* :246 */

    const v3 h = cross(dir, p2_p0); /* :255 */
    const float a = dot(p1_p0, h);  /* :256 */

    if (fabsf(a) < 0) /* :258, never true: kept as written */
        return 0;

    const float f = 1 / a;          /* :261 */
    const v3 s = sub(pos, p0);      /* :262 */
    const float u = f * dot(s, h);  /* :263 */

    if (u < 0 || u > 1) /* :265 */
        return 0;

    const v3 q = cross(s, p1_p0);     /* :268 */
    const float v = f * dot(dir, q);  /* :269 */

    if (v < 0 || u + v > 1) /* :271 */
        return 0;

    if (a == 0)
        hit->events |= ORC_EVENT_ZERO_DET;

    const float t = f * dot(p2_p0, q); /* :274 */

    if (t <= tmin || obj == prevObj || t >= hit->hitT) /* :276 */
        return 0;

    if (t != t)
        hit->events |= ORC_EVENT_NAN_T;

    hit->u = u; /* :279-280 */
    hit->v = v;
    hit->hitT = t;
    return 1;
}

/* traceGeometry, res/shaders/trace.glsl:9-66 (triangle loop :24-28). */
static void trace_geometry_one(const igxrt_triangle* tris, uint32_t ntri,
                               const igxrt_ray* ray, uint32_t prev, igxrt_hit* out,
                               uint32_t* flags) {
    hitstate hit;
    hit.hitT = tmax_effective(ray->tmax); /* :14 (noHit at the default tmax) */
    hit.u = hit.v = 0;                    /* :16 */
    hit.object = 0;                       /* :17 */
    hit.events = 0;
    const v3 pos = mk(ray->org), dir = mk(ray->dir);
    int found = 0;
    uint32_t j = 0;
    for (uint32_t i = 0; i < ntri; ++i, ++j)
        if (ray_intersect_tri(pos, dir, ray->tmin, &tris[i], j, (uint64_t)prev, &hit)) {
            hit.object = j; /* :27 */
            found = 1;
        }
    if (found) {
        out->t = hit.hitT;
        out->u = hit.u;
        out->v = hit.v;
        out->prim = hit.object;
    } else {
        /* raygen.comp:40-41 encodes a miss as object = noRayHit. */
        out->t = IGXRT_NO_HIT;
        out->u = 0;
        out->v = 0;
        out->prim = IGXRT_NO_RAY_HIT;
    }
    if (flags)
        *flags = hit.events;
}

/* traceOcclusion, res/shaders/trace.glsl:70-98. */
static void trace_occlusion_one(const igxrt_triangle* tris, uint32_t ntri,
                                const igxrt_ray* ray, uint32_t prev, uint32_t* out,
                                uint32_t* flags) {
    hitstate hit;
    hit.hitT = IGXRT_NO_HIT; /* :73 */
    hit.u = hit.v = 0;
    hit.object = 0;
    hit.events = 0;
    const v3 pos = mk(ray->org), dir = mk(ray->dir);
    uint32_t j = 0;
    for (uint32_t i = 0; i < ntri; ++i, ++j) /* :77-79 */
        ray_intersect_tri(pos, dir, ray->tmin, &tris[i], j, (uint64_t)prev, &hit);
    const float maxDist = tmax_effective(ray->tmax);
    *out = hit.hitT < maxDist ? 1u : 0u; /* :97 */
    if (flags)
        *flags = hit.events;
}

/* ------------------------------------------------------------------------ */
/* Thread pool over ray chunks.                                             */
/* ------------------------------------------------------------------------ */

typedef void (*chunk_fn)(void* ctx, uint32_t begin, uint32_t end);

typedef struct {
    chunk_fn fn;
    void* ctx;
    uint32_t n;
    uint32_t chunk;
    _Atomic uint32_t next;
} pool_job;

static void* pool_worker(void* arg) {
    pool_job* job = (pool_job*)arg;
    for (;;) {
        uint32_t b = atomic_fetch_add(&job->next, job->chunk);
        if (b >= job->n)
            break;
        uint32_t e = b + job->chunk;
        if (e > job->n || e < b)
            e = job->n;
        job->fn(job->ctx, b, e);
    }
    return NULL;
}

int orc_hardware_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

static void run_parallel(chunk_fn fn, void* ctx, uint32_t n, uint32_t chunk, int threads) {
    if (threads <= 0)
        threads = orc_hardware_threads();
    if (n == 0)
        return;
    pool_job job;
    job.fn = fn;
    job.ctx = ctx;
    job.n = n;
    job.chunk = chunk;
    atomic_init(&job.next, 0);
    if (threads == 1) {
        pool_worker(&job);
        return;
    }
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    int started = 0;
    for (int i = 0; i < threads; ++i)
        if (pthread_create(&tid[i], NULL, pool_worker, &job) == 0)
            ++started;
    if (started == 0)
        pool_worker(&job);
    for (int i = 0; i < started; ++i)
        pthread_join(tid[i], NULL);
    free(tid);
}

typedef struct {
    const igxrt_triangle* tris;
    uint32_t ntri;
    const igxrt_ray* rays;
    const uint32_t* prev;
    igxrt_hit* hits;
    uint32_t* occ;
    uint32_t* flags;
} brute_ctx;

static void brute_closest_chunk(void* p, uint32_t b, uint32_t e) {
    brute_ctx* c = (brute_ctx*)p;
    for (uint32_t i = b; i < e; ++i)
        trace_geometry_one(c->tris, c->ntri, &c->rays[i],
                           c->prev ? c->prev[i] : IGXRT_NO_RAY_HIT, &c->hits[i],
                           c->flags ? &c->flags[i] : NULL);
}

static void brute_any_chunk(void* p, uint32_t b, uint32_t e) {
    brute_ctx* c = (brute_ctx*)p;
    for (uint32_t i = b; i < e; ++i)
        trace_occlusion_one(c->tris, c->ntri, &c->rays[i],
                            c->prev ? c->prev[i] : IGXRT_NO_RAY_HIT, &c->occ[i],
                            c->flags ? &c->flags[i] : NULL);
}

void orc_trace_geometry(const igxrt_triangle* tris, uint32_t ntri, const igxrt_ray* rays,
                        const uint32_t* prev_hit, uint32_t nrays, igxrt_hit* out,
                        uint32_t* flags, int threads) {
    brute_ctx c = {tris, ntri, rays, prev_hit, out, NULL, flags};
    run_parallel(brute_closest_chunk, &c, nrays, 64, threads);
}

void orc_trace_occlusion(const igxrt_triangle* tris, uint32_t ntri, const igxrt_ray* rays,
                         const uint32_t* prev_hit, uint32_t nrays, uint32_t* out,
                         uint32_t* flags, int threads) {
    brute_ctx c = {tris, ntri, rays, prev_hit, NULL, out, flags};
    run_parallel(brute_any_chunk, &c, nrays, 64, threads);
}

/* ------------------------------------------------------------------------ */
/* Spheres, cubes and planes (mixed scenes).                                */
/* ------------------------------------------------------------------------ */

/* GLSL min / max as the specification defines them. */
static inline float gmin(float x, float y) { return y < x ? y : x; }
static inline float gmax(float x, float y) { return x < y ? y : x; }
static inline v3 scale(v3 a, float s) {
    v3 r = {a.x * s, a.y * s, a.z * s};
    return r;
}
static inline v3 add(v3 a, v3 b) {
    v3 r = {a.x + b.x, a.y + b.y, a.z + b.z};
    return r;
}
static inline v3 normalize3(v3 a) {
    const float len = sqrtf(dot(a, a));
    v3 r = {a.x / len, a.y / len, a.z / len};
    return r;
}

/* rayIntersectSphere, res/shaders/primitive.glsl:173-210. */
static int ray_intersect_sphere(v3 pos, v3 dir, float tmin, const float* sphere, uint64_t obj,
                                uint64_t prevObj, hitstate* hit) {
    const v3 c = mk(sphere);
    const v3 dif = sub(c, pos);                /* :175 */
    const float t = dot(dif, dir);             /* :176 */
    const v3 Q = sub(dif, scale(dir, t));      /* :178 */
    const float Q2 = dot(Q, Q);                /* :179 */
    const float R2 = sphere[3] * sphere[3];    /* :180 */
    const int outOfSphere = Q2 > R2;           /* :182 */
    const float hitT = t - sqrtf(R2 - Q2);     /* :183 */
    if (!outOfSphere && obj != prevObj && hitT >= tmin && hitT < hit->hitT) { /* :185 */
        hit->hitT = hitT;
        const v3 o = add(scale(dir, hitT), pos);          /* :189 */
        const v3 normal = normalize3(sub(c, o));          /* :190 */
        hit->gn[0] = normal.x;                            /* :192 */
        hit->gn[1] = normal.y;
        hit->gn[2] = normal.z;
        /* asin / atan correctly rounded to binary32 (binary64, rounded once) */
        const float latitude = (float)asin((double)normal.z);            /* :198 */
        float longitude = (float)atan((double)(normal.y / normal.x));    /* :199 */
        if (longitude != longitude)                       /* :201-202 */
            longitude = 0;
        const float k = (float)(0.636619746685 * 0.5);    /* :204 */
        hit->u = latitude * k + 0.5f;
        hit->v = longitude * k + 0.5f;
        return 1;
    }
    return 0;
}

/* rayIntersectPlane, res/shaders/primitive.glsl:212-237. */
static int ray_intersect_plane(v3 pos, v3 dir, float tmin, const float* plane, uint64_t obj,
                               uint64_t prevObj, hitstate* hit) {
    const v3 n = mk(plane);
    const v3 pdir = normalize3(n);                      /* :214 */
    const v3 neg = {-pdir.x, -pdir.y, -pdir.z};
    const float dif = dot(dir, neg);                    /* :215 */
    const float hitT = -(dot(pos, neg) + plane[3]) / dif; /* :219 */
    if (hitT >= tmin && obj != prevObj && hitT < hit->hitT) { /* :221 */
        hit->hitT = hitT;
        const v3 gn = dif > 0 ? neg : pdir;             /* :224 */
        hit->gn[0] = gn.x;
        hit->gn[1] = gn.y;
        hit->gn[2] = gn.z;
        const v3 o = add(scale(dir, hitT), pos);        /* :226 */
        const v3 z = {0, 0, 1}, x = {1, 0, 0};
        const v3 planeX = cross(n, z);                  /* :228 */
        const v3 planeZ = cross(n, x);                  /* :229 */
        hit->u = dot(o, planeX);                        /* :231 */
        hit->v = dot(o, planeZ);
        return 1;
    }
    return 0;
}

/* rayIntersectCube, res/shaders/primitive.glsl:286-333. */
static int ray_intersect_cube(v3 pos, v3 dir, float tmin_ray, const igxrt_cube* cube, uint64_t obj,
                              uint64_t prevObj, hitstate* hit) {
    const v3 revDir = {1 / dir.x, 1 / dir.y, 1 / dir.z};               /* :288 */
    const v3 start = {cube->xy0[0], cube->xy0[1], cube->z0_x1[0]};     /* :290 */
    const v3 end = {cube->z0_x1[1], cube->yz1[0], cube->yz1[1]};       /* :291 */
    const v3 sd = sub(start, pos), ed = sub(end, pos);
    const v3 startDir = {sd.x * revDir.x, sd.y * revDir.y, sd.z * revDir.z}; /* :293 */
    const v3 endDir = {ed.x * revDir.x, ed.y * revDir.y, ed.z * revDir.z};
    const v3 mi = {gmin(startDir.x, endDir.x), gmin(startDir.y, endDir.y), gmin(startDir.z, endDir.z)};
    const v3 ma = {gmax(startDir.x, endDir.x), gmax(startDir.y, endDir.y), gmax(startDir.z, endDir.z)};
    const float tmin = gmax(gmax(mi.x, mi.y), mi.z);    /* :299 */
    const float tmax = gmin(gmin(ma.x, ma.y), ma.z);    /* :300 */
    if (tmax < tmin_ray || tmin > tmax || tmin > hit->hitT || obj == prevObj) /* :302 */
        return 0;
    v3 p = sub(add(scale(dir, tmin), pos), start);      /* :308 */
    p.x = p.x / end.x;                                  /* :309 */
    p.y = p.y / end.y;
    p.z = p.z / end.z;
    hit->gn[0] = hit->gn[1] = hit->gn[2] = 0;
    if (tmin == mi.x) {                                 /* :311-327 */
        hit->gn[0] = mi.x == startDir.x ? 1.0f : -1.0f; /* isLeft * 2 - 1 */
        hit->u = p.y;
        hit->v = p.z;
    } else if (tmin == mi.y) {
        hit->gn[1] = mi.y == startDir.y ? 1.0f : -1.0f; /* isDown * 2 - 1 */
        hit->u = p.x;
        hit->v = p.z;
    } else {
        hit->gn[2] = mi.z == startDir.z ? 1.0f : -1.0f; /* isBack * 2 - 1 */
        hit->u = p.x;
        hit->v = p.y;
    }
    hit->hitT = tmin;                                   /* :331 */
    return 1;
}

/* The loops of traceGeometry / traceOcclusion over every buffer
 * (trace.glsl:22-46, 75-95); returns whether anything was accepted. */
static int trace_mixed_one(const igxrt_scene_desc* d, const igxrt_ray* ray, uint32_t prev,
                           hitstate* hit) {
    const v3 pos = mk(ray->org), dir = mk(ray->dir);
    const uint64_t p = prev;
    int found = 0;
    uint32_t j = 0;
    for (uint32_t i = 0; i < d->triangle_count; ++i, ++j)
        if (ray_intersect_tri(pos, dir, ray->tmin, &d->triangles[i], j, p, hit)) {
            hit->object = j;
            found = 1;
        }
    for (uint32_t i = 0; i < d->sphere_count; ++i, ++j)
        if (ray_intersect_sphere(pos, dir, ray->tmin, d->spheres + 4 * (size_t)i, j, p, hit)) {
            hit->object = j;
            found = 1;
        }
    for (uint32_t i = 0; i < d->cube_count; ++i, ++j)
        if (ray_intersect_cube(pos, dir, ray->tmin, &d->cubes[i], j, p, hit)) {
            hit->object = j;
            found = 1;
        }
    for (uint32_t i = 0; i < d->plane_count; ++i, ++j)
        if (ray_intersect_plane(pos, dir, ray->tmin, d->planes + 4 * (size_t)i, j, p, hit)) {
            hit->object = j;
            found = 1;
        }
    return found;
}

typedef struct {
    const igxrt_scene_desc* d;
    const igxrt_ray* rays;
    const uint32_t* prev;
    igxrt_hit* hits;
    uint32_t* occ;
    uint32_t* flags;
} mixed_ctx;

static void mixed_closest_chunk(void* p, uint32_t b, uint32_t e) {
    mixed_ctx* c = (mixed_ctx*)p;
    for (uint32_t i = b; i < e; ++i) {
        hitstate hit;
        hit.hitT = tmax_effective(c->rays[i].tmax);
        hit.u = hit.v = 0;
        hit.object = 0;
        hit.events = 0;
        const int found = trace_mixed_one(c->d, &c->rays[i], c->prev ? c->prev[i] : IGXRT_NO_RAY_HIT, &hit);
        igxrt_hit* o = &c->hits[i];
        if (found) {
            o->t = hit.hitT;
            o->u = hit.u;
            o->v = hit.v;
            o->prim = hit.object;
        } else {
            o->t = IGXRT_NO_HIT;
            o->u = o->v = 0;
            o->prim = IGXRT_NO_RAY_HIT;
        }
        if (c->flags)
            c->flags[i] = hit.events;
    }
}

static void mixed_any_chunk(void* p, uint32_t b, uint32_t e) {
    mixed_ctx* c = (mixed_ctx*)p;
    for (uint32_t i = b; i < e; ++i) {
        hitstate hit;
        hit.hitT = IGXRT_NO_HIT;
        hit.u = hit.v = 0;
        hit.object = 0;
        hit.events = 0;
        trace_mixed_one(c->d, &c->rays[i], c->prev ? c->prev[i] : IGXRT_NO_RAY_HIT, &hit);
        c->occ[i] = hit.hitT < tmax_effective(c->rays[i].tmax) ? 1u : 0u;
        if (c->flags)
            c->flags[i] = hit.events;
    }
}

void orc_trace_geometry_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays,
                              const uint32_t* prev_hit, uint32_t nrays, igxrt_hit* out,
                              uint32_t* flags, int threads) {
    mixed_ctx c = {scene, rays, prev_hit, out, NULL, flags};
    run_parallel(mixed_closest_chunk, &c, nrays, 64, threads);
}

void orc_trace_occlusion_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays,
                               const uint32_t* prev_hit, uint32_t nrays, uint32_t* out,
                               uint32_t* flags, int threads) {
    mixed_ctx c = {scene, rays, prev_hit, NULL, out, flags};
    run_parallel(mixed_any_chunk, &c, nrays, 64, threads);
}

/* unpackHalf2x16 component: exact binary16 -> binary32. */
static float half_to_float(uint32_t h) {
    const uint32_t sign = (h >> 15) & 1u, ex = (h >> 10) & 31u, man = h & 1023u;
    float mag;
    if (ex == 0) {
        mag = (float)man * 0x1p-24f;
    } else if (ex == 31) {
        mag = man ? NAN : INFINITY;
    } else {
        const uint32_t bits = ((ex + 112u) << 23) | (man << 13);
        memcpy(&mag, &bits, 4);
    }
    return sign ? -mag : mag;
}

/* decodeSpheremap, primitive.glsl:95-104. */
void orc_decode_spheremap(uint32_t n, float out[3]) {
    float x = half_to_float(n & 0xffffu), y = half_to_float(n >> 16);
    const v3 a = {x, y, 1.0f}, b = {-x, -y, 1.0f}; /* vec3(nn, 1), -vec3(nn, -1) */
    const float l = dot(a, b);
    const float s = sqrtf(l);
    x = x * s; /* nn *= sqrt(l) */
    y = y * s;
    out[0] = x * 2 + 0.0f; /* vec3(nn, l) * 2 + vec3(0, 0, -1) */
    out[1] = y * 2 + 0.0f;
    out[2] = l * 2 + -1.0f;
}

/* float -> uint conversion with the GPU's rule for the out-of-range
 * values GLSL leaves undefined: NaN and negatives give 0. */
static uint32_t f2u(float f) {
    if (!(f > 0.0f))
        return 0u;
    if (f >= 4294967296.0f)
        return 0xffffffffu;
    return (uint32_t)f;
}

/* encodeNormal, primitive.glsl:85-88. */
void orc_encode_normal(const float n[3], uint32_t out[2]) {
    const v3 v = {n[0], n[1], n[2]};
    const float len = sqrtf(dot(v, v)); /* normalize(n) = n / length(n) */
    const uint32_t hx = f2u((n[0] / len * 0.5f + 0.5f) * 65535.0f);
    const uint32_t hy = f2u((n[1] / len * 0.5f + 0.5f) * 65535.0f);
    const uint32_t hz = f2u((n[2] / len * 0.5f + 0.5f) * 65535.0f);
    out[0] = (hx << 16) | hy;
    out[1] = hz;
}

typedef struct {
    const igxrt_triangle* tris;
    uint32_t ntri;
    const igxrt_camera* cam;
    float inv_w, inv_h;
    float* dir_object;
    float* uv_normal;
    uint32_t* flags;
    const igxrt_scene_desc* scene; /* non-NULL: every primitive type (mixed scenes) */
} gbuffer_ctx;

/* The primary ray of pixel (x, y): calculatePrimary (camera.glsl:115-116)
 * and calculateScreen (:72-87), origin at the eye. */
static void camera_ray(const igxrt_camera* c, float inv_w, float inv_h, uint32_t x, uint32_t y,
                       igxrt_ray* ray) {
    const float cx = ((float)x + c->jitter_x) * inv_w;
    const float cy = 1 - ((float)y + c->jitter_y) * inv_h;
    float d[3];
    for (int k = 0; k < 3; ++k) {
        const float right = c->p1[k] - c->p0[k], up = c->p2[k] - c->p0[k];
        const float pos = c->p0[k] + cx * right + cy * up;
        d[k] = pos - c->eye[k];
    }
    const v3 dv = {d[0], d[1], d[2]};
    const float len = sqrtf(dot(dv, dv));
    for (int k = 0; k < 3; ++k) {
        ray->org[k] = c->eye[k];
        ray->dir[k] = d[k] / len;
    }
    ray->tmin = 0.0f;
    ray->tmax = IGXRT_NO_HIT;
}

void orc_camera_rays(const igxrt_camera* cam, igxrt_ray* rays) {
    const float inv_w = 1.0f / (float)cam->width, inv_h = 1.0f / (float)cam->height;
    for (uint32_t y = 0; y < cam->height; ++y)
        for (uint32_t x = 0; x < cam->width; ++x)
            camera_ray(cam, inv_w, inv_h, x, y, &rays[(size_t)y * cam->width + x]);
}

static void gbuffer_chunk(void* p, uint32_t b, uint32_t e) {
    gbuffer_ctx* g = (gbuffer_ctx*)p;
    const igxrt_camera* c = g->cam;
    for (uint32_t i = b; i < e; ++i) {
        igxrt_ray ray;
        camera_ray(c, g->inv_w, g->inv_h, i % c->width, i / c->width, &ray);
        igxrt_hit h;
        uint32_t f = 0;
        float gn[3] = {0, 0, 0};
        if (g->scene) {
            hitstate hs;
            hs.hitT = IGXRT_NO_HIT;
            hs.u = hs.v = 0;
            hs.object = 0;
            hs.events = 0;
            trace_mixed_one(g->scene, &ray, IGXRT_NO_RAY_HIT, &hs);
            f = hs.events;
            /* raygen.comp:40: a miss is hitT == noHit */
            h.t = hs.hitT;
            h.u = hs.u;
            h.v = hs.v;
            h.prim = hs.hitT == IGXRT_NO_HIT ? IGXRT_NO_RAY_HIT : hs.object;
            memcpy(gn, hs.gn, sizeof(gn));
        } else {
            trace_geometry_one(g->tris, g->ntri, &ray, IGXRT_NO_RAY_HIT, &h, &f);
        }
        if (g->flags)
            g->flags[i] = f;
        float* dob = g->dir_object + 4 * (size_t)i;
        if (h.prim != IGXRT_NO_RAY_HIT) {
            /* raygen.comp:39: vec4(hit.rayDir * hit.hitT, uintBitsToFloat(hit.object)) */
            for (int k = 0; k < 3; ++k)
                dob[k] = ray.dir[k] * h.t;
            memcpy(&dob[3], &h.prim, 4);
            /* trace.glsl:50-63, raygen.comp:46-51: a triangle's interpolated
             * vertex normal, any other object's geometry normal */
            float n[3];
            if (h.prim < g->ntri) {
                const igxrt_triangle* t = &g->tris[h.prim];
                float n0[3], n1[3], n2[3];
                orc_decode_spheremap(t->n0, n0);
                orc_decode_spheremap(t->n1, n1);
                orc_decode_spheremap(t->n2, n2);
                const float bw = 1 - h.u - h.v; /* interpolate, primitive.glsl:146-151 */
                for (int k = 0; k < 3; ++k)
                    n[k] = h.u * n1[k] + h.v * n2[k] + bw * n0[k];
            } else {
                memcpy(n, gn, sizeof(n));
            }
            uint32_t enc[2];
            orc_encode_normal(n, enc);
            float* uvn = g->uv_normal + 4 * (size_t)i;
            uvn[0] = h.u;
            uvn[1] = h.v;
            memcpy(&uvn[2], enc, 8);
        } else {
            /* raygen.comp:40-41: vec4(hit.rayDir, uintBitsToFloat(noRayHit)) */
            const uint32_t none = IGXRT_NO_RAY_HIT;
            for (int k = 0; k < 3; ++k)
                dob[k] = ray.dir[k];
            memcpy(&dob[3], &none, 4);
        }
    }
}

void orc_gbuffer(const igxrt_triangle* tris, uint32_t ntri, const igxrt_camera* cam,
                 float* dir_object, float* uv_normal, uint32_t* flags, int threads) {
    gbuffer_ctx g = {tris, ntri, cam, 1.0f / (float)cam->width, 1.0f / (float)cam->height,
                     dir_object, uv_normal, flags, NULL};
    run_parallel(gbuffer_chunk, &g, cam->width * cam->height, 64, threads);
}

void orc_gbuffer_mixed(const igxrt_scene_desc* scene, const igxrt_camera* cam, float* dir_object,
                       float* uv_normal, uint32_t* flags, int threads) {
    gbuffer_ctx g = {scene->triangles, scene->triangle_count, cam, 1.0f / (float)cam->width,
                     1.0f / (float)cam->height, dir_object, uv_normal, flags, scene};
    run_parallel(gbuffer_chunk, &g, cam->width * cam->height, 64, threads);
}

/* indexToLight, res/shaders/light.glsl:221-229. */
static uint32_t index_to_light(uint32_t lx, uint32_t ly, uint32_t rx, uint32_t ry, uint32_t light,
                               uint32_t shx, uint32_t shy, uint32_t mx, uint32_t my) {
    const uint32_t tile_x = lx >> shx, tile_y = ly >> shy;
    uint32_t tiles_x = rx >> shx, tiles_y = ry >> shy;
    tiles_x += (rx & mx) != 0; /* ceil(res / threads) */
    tiles_y += (ry & my) != 0;
    return tile_x + tile_y * tiles_x + light * tiles_y * tiles_x;
}

typedef struct {
    const igxrt_triangle* tris;
    uint32_t ntri;
    const igxrt_ray* rays;
    const uint32_t* object;
    uint32_t w, h;
    uint32_t* occ;
    uint32_t* flags;
    const igxrt_scene_desc* scene; /* non-NULL: every primitive type (mixed scenes) */
} shadow_ctx;

static void shadow_chunk(void* p, uint32_t b, uint32_t e) {
    shadow_ctx* c = (shadow_ctx*)p;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t pix = i % (c->w * c->h);
        const uint32_t obj = c->object[pix];
        uint32_t f = 0;
        c->occ[i] = 0;
        if (obj != IGXRT_NO_RAY_HIT) { /* nv_all.shadow.comp:108 */
            if (c->scene) {
                hitstate hs;
                hs.hitT = IGXRT_NO_HIT;
                hs.u = hs.v = 0;
                hs.object = 0;
                hs.events = 0;
                trace_mixed_one(c->scene, &c->rays[i], obj, &hs);
                c->occ[i] = hs.hitT < tmax_effective(c->rays[i].tmax) ? 1u : 0u; /* trace.glsl:97 */
                f = hs.events;
            } else {
                trace_occlusion_one(c->tris, c->ntri, &c->rays[i], obj, &c->occ[i], &f);
            }
        }
        if (c->flags)
            c->flags[i] = f;
    }
}

static void shadow_mask_impl(const igxrt_triangle* tris, uint32_t ntri, const igxrt_scene_desc* scene,
                             const igxrt_ray* rays, const uint32_t* object, uint32_t width,
                             uint32_t height, uint32_t samples, uint32_t* mask, uint32_t* flags,
                             int threads);

void orc_shadow_mask(const igxrt_triangle* tris, uint32_t ntri, const igxrt_ray* rays,
                     const uint32_t* object, uint32_t width, uint32_t height, uint32_t samples,
                     uint32_t* mask, uint32_t* flags, int threads) {
    shadow_mask_impl(tris, ntri, NULL, rays, object, width, height, samples, mask, flags, threads);
}

void orc_shadow_mask_mixed(const igxrt_scene_desc* scene, const igxrt_ray* rays, const uint32_t* object,
                           uint32_t width, uint32_t height, uint32_t samples, uint32_t* mask,
                           uint32_t* flags, int threads) {
    shadow_mask_impl(scene->triangles, scene->triangle_count, scene, rays, object, width, height, samples,
                     mask, flags, threads);
}

static void shadow_mask_impl(const igxrt_triangle* tris, uint32_t ntri, const igxrt_scene_desc* scene,
                             const igxrt_ray* rays, const uint32_t* object, uint32_t width,
                             uint32_t height, uint32_t samples, uint32_t* mask, uint32_t* flags,
                             int threads) {
    const uint32_t n = width * height * samples;
    uint32_t* occ = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    shadow_ctx c = {tris, ntri, rays, object, width, height, occ, flags, scene};
    run_parallel(shadow_chunk, &c, n, 64, threads);
    const uint32_t tiles_x = (width + 15) / 16, tiles_y = (height + 1) / 2;
    memset(mask, 0, sizeof(uint32_t) * (size_t)tiles_x * tiles_y * samples);
    for (uint32_t s = 0; s < samples; ++s)
        for (uint32_t y = 0; y < height; ++y)
            for (uint32_t x = 0; x < width; ++x) {
                if (!occ[((size_t)s * height + y) * width + x])
                    continue;
                /* ballotARB(hit) over the 16x2 subgroup, stored by lane 0
                 * (nv_all.shadow.comp:128-138) */
                const uint32_t word = index_to_light(x, y, width, height, s, 4, 1, 15, 1);
                const uint32_t lane = (x & 15) | ((y & 1) << 4);
                mask[word] |= 1u << lane;
            }
    free(occ);
}

int orc_reintersect_f64(const igxrt_ray* ray, const igxrt_triangle* tri, double* t_out,
                        double* u_out, double* v_out) {
    double o[3], d[3], p0[3], e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
        o[k] = ray->org[k];
        d[k] = ray->dir[k];
        p0[k] = tri->p0[k];
        e1[k] = (double)tri->p1[k] - (double)tri->p0[k];
        e2[k] = (double)tri->p2[k] - (double)tri->p0[k];
    }
    double h[3] = {d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0],
                   d[0] * e2[1] - e2[0] * d[1]};
    double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
    double s[3] = {o[0] - p0[0], o[1] - p0[1], o[2] - p0[2]};
    double q[3] = {s[1] * e1[2] - e1[1] * s[2], s[2] * e1[0] - e1[2] * s[0],
                   s[0] * e1[1] - e1[0] * s[1]};
    double u = (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]) / a;
    double v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) / a;
    double t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) / a;
    *t_out = t;
    *u_out = u;
    *v_out = v;
    return (u >= 0 && u <= 1 && v >= 0 && u + v <= 1 && t > (double)ray->tmin) ? 1 : 0;
}

/* ------------------------------------------------------------------------ */
/* BVH traversal (the CPU baseline and fetch counter).                      */
/* ------------------------------------------------------------------------ */

#define ORC_STACK 256

typedef struct {
    v3 o, d;     /* the ray as given: the triangle test uses these */
    v3 idir;     /* 1/d, with |d| < 2^-80 raised to 2^-80 keeping the sign */
    v3 ood;      /* o * idir */
    float tmin;
    float tmin_box;
    float tmax_eff;
    uint32_t prev;
} rayprep;

static inline float safe_dir(float d) {
    return fabsf(d) < 0x1p-80f ? copysignf(0x1p-80f, d) : d;
}

static void prep_ray(const igxrt_ray* r, uint32_t prev, rayprep* p) {
    p->o = mk(r->org);
    p->d = mk(r->dir);
    p->idir.x = 1.0f / safe_dir(r->dir[0]);
    p->idir.y = 1.0f / safe_dir(r->dir[1]);
    p->idir.z = 1.0f / safe_dir(r->dir[2]);
    p->ood.x = p->o.x * p->idir.x;
    p->ood.y = p->o.y * p->idir.y;
    p->ood.z = p->o.z * p->idir.z;
    p->tmin = r->tmin;
    p->tmin_box = (r->tmin > -INFINITY) ? fmaf(-fabsf(r->tmin), 0x1p-10f, r->tmin) : -INFINITY;
    p->tmax_eff = tmax_effective(r->tmax);
    p->prev = prev;
}

/* Slab test against a padded box; identical operation sequence on the GPU. */
static inline int box_hit(const rayprep* r, float lox, float hix, float loy, float hiy,
                          float loz, float hiz, float tcull, float* tnear) {
    const float t0x = fmaf(lox, r->idir.x, -r->ood.x), t1x = fmaf(hix, r->idir.x, -r->ood.x);
    const float t0y = fmaf(loy, r->idir.y, -r->ood.y), t1y = fmaf(hiy, r->idir.y, -r->ood.y);
    const float t0z = fmaf(loz, r->idir.z, -r->ood.z), t1z = fmaf(hiz, r->idir.z, -r->ood.z);
    const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)),
                           fmaxf(fminf(t0z, t1z), r->tmin_box));
    const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)),
                           fminf(fmaxf(t0z, t1z), tcull));
    *tnear = tn;
    return tn <= tf;
}

/* rayIntersectTri's arithmetic on a primitive record (e1, e2 stored). */
static inline int rec_intersect(const rayprep* r, const igxrt_prim_record* rec, float* t_out,
                                float* u_out, float* v_out) {
    const v3 p0 = mk(rec->p0), e1 = mk(rec->e1), e2 = mk(rec->e2);
    const v3 h = cross(r->d, e2);
    const float a = dot(e1, h);
    const float f = 1 / a;
    const v3 s = sub(r->o, p0);
    const float u = f * dot(s, h);
    if (u < 0 || u > 1)
        return 0;
    const v3 q = cross(s, e1);
    const float v = f * dot(r->d, q);
    if (v < 0 || u + v > 1)
        return 0;
    *t_out = f * dot(e2, q);
    *u_out = u;
    *v_out = v;
    return 1;
}

typedef struct {
    float t, u, v;
    uint32_t prim;
    float tcull;
} best_hit;

/* Box cull limit: best t widened upward by 2^-10 of its magnitude (t can be
 * negative with a negative tmin), kept finite so the {+inf} box of an absent
 * child is never entered. */
static inline float cull_limit(float t) { return fminf(fmaf(fabsf(t), 0x1p-10f, t), FLT_MAX); }

/* Returns 1 when the record is accepted under the (t, prim) order. */
static inline int leaf_record(const rayprep* r, const igxrt_prim_record* rec, best_hit* b,
                              int anyhit) {
    float t, u, v;
    if (!rec_intersect(r, rec, &t, &u, &v))
        return 0;
    if (t <= r->tmin || rec->prim == r->prev)
        return 0;
    if (anyhit)
        return t < r->tmax_eff;
    if (t < b->t || (t == b->t && rec->prim < b->prim)) {
        b->t = t;
        b->u = u;
        b->v = v;
        b->prim = rec->prim;
        b->tcull = cull_limit(t);
        return 1;
    }
    return 0;
}

/* Traversal stack entry: a pushed child and the entry distance its box had
 * when it was pushed.  A popped entry whose distance is beyond the current
 * cull limit is dropped without fetching: its box test would now fail. */
typedef struct {
    int32_t ref;
    float tnear;
} stack_entry;

/* Pops the next live entry into *next; returns 0 when the stack runs out. */
static inline int pop_live(const stack_entry* stack, int* sp, float tcull, int32_t* next) {
    while (*sp > 0) {
        const stack_entry e = stack[--*sp];
        if (e.tnear <= tcull) {
            *next = e.ref;
            return 1;
        }
    }
    return 0;
}

static int bvh2_trace_one(const igxrt_bvh2_node* nodes, uint64_t nn,
                          const igxrt_prim_record* prims, uint64_t np, const rayprep* r,
                          int anyhit, best_hit* b, uint32_t* occluded, uint32_t* nf,
                          uint32_t* pf) {
    stack_entry stack[ORC_STACK];
    int sp = 0;
    *occluded = 0;
    if (nn == 0)
        return 0;
    int32_t next = 0;
    for (;;) {
        if (next >= 0) {
            if ((uint64_t)next >= nn)
                return -1;
            const igxrt_bvh2_node* n = &nodes[next];
            ++*nf;
            float tn0, tn1;
            const int h0 = box_hit(r, n->c0_x[0], n->c0_x[1], n->c0_y[0], n->c0_y[1],
                                   n->c0_z[0], n->c0_z[1], b->tcull, &tn0);
            const int h1 = box_hit(r, n->c1_x[0], n->c1_x[1], n->c1_y[0], n->c1_y[1],
                                   n->c1_z[0], n->c1_z[1], b->tcull, &tn1);
            if (h0 && h1) {
                const int first = tn1 < tn0 ? 1 : 0;
                if (sp >= ORC_STACK)
                    return -1;
                stack[sp].ref = n->child[1 - first];
                stack[sp].tnear = first ? tn0 : tn1;
                ++sp;
                next = n->child[first];
            } else if (h0) {
                next = n->child[0];
            } else if (h1) {
                next = n->child[1];
            } else if (!pop_live(stack, &sp, b->tcull, &next)) {
                break;
            }
        } else {
            uint64_t i = (uint64_t)(uint32_t)~next;
            for (;;) {
                if (i >= np)
                    return -1;
                const igxrt_prim_record* rec = &prims[i];
                ++*pf;
                if (leaf_record(r, rec, b, anyhit) && anyhit) {
                    *occluded = 1;
                    return 0;
                }
                if (rec->leaf_end)
                    break;
                ++i;
            }
            if (!pop_live(stack, &sp, b->tcull, &next))
                break;
        }
    }
    return 0;
}

static int bvh4_trace_one(const igxrt_bvh4_node* nodes, uint64_t nn,
                          const igxrt_prim_record* prims, uint64_t np, const rayprep* r,
                          int anyhit, best_hit* b, uint32_t* occluded, uint32_t* nf,
                          uint32_t* pf) {
    stack_entry stack[ORC_STACK];
    int sp = 0;
    *occluded = 0;
    if (nn == 0)
        return 0;
    int32_t next = 0;
    for (;;) {
        if (next >= 0) {
            if ((uint64_t)next >= nn)
                return -1;
            const igxrt_bvh4_node* n = &nodes[next];
            ++*nf;
            float tn[4];
            int slot[4];
            int m = 0;
            for (int k = 0; k < 4; ++k) {
                float t;
                if (box_hit(r, n->lo_x[k], n->hi_x[k], n->lo_y[k], n->hi_y[k], n->lo_z[k],
                            n->hi_z[k], b->tcull, &t)) {
                    /* insertion by (tnear, slot): stable for equal tnear */
                    int j = m++;
                    while (j > 0 && t < tn[j - 1]) {
                        tn[j] = tn[j - 1];
                        slot[j] = slot[j - 1];
                        --j;
                    }
                    tn[j] = t;
                    slot[j] = k;
                }
            }
            if (m == 0) {
                if (!pop_live(stack, &sp, b->tcull, &next))
                    break;
            } else {
                if (sp + m - 1 > ORC_STACK)
                    return -1;
                for (int j = m - 1; j >= 1; --j) {
                    stack[sp].ref = n->child[slot[j]];
                    stack[sp].tnear = tn[j];
                    ++sp;
                }
                next = n->child[slot[0]];
            }
        } else {
            uint64_t i = (uint64_t)(uint32_t)~next;
            for (;;) {
                if (i >= np)
                    return -1;
                const igxrt_prim_record* rec = &prims[i];
                ++*pf;
                if (leaf_record(r, rec, b, anyhit) && anyhit) {
                    *occluded = 1;
                    return 0;
                }
                if (rec->leaf_end)
                    break;
                ++i;
            }
            if (!pop_live(stack, &sp, b->tcull, &next))
                break;
        }
    }
    return 0;
}

/* BVH8 slot order key: the entry distance mapped to an order-preserving word
 * with its low 3 bits replaced by the slot, so keys are distinct and sort by
 * (distance, slot); a pushed entry keeps the distance of the key with those
 * bits cleared, which is never larger than the box's own. */
static inline uint32_t order_key(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static inline int normal_step(float m) {
    const float a = fabsf(m);
    return a >= FLT_MIN && a <= FLT_MAX;
}

/* The slab test of box_hit on given per-axis plane distances. */
static inline int slab_hit(const rayprep* r, float t0x, float t1x, float t0y, float t1y, float t0z,
                           float t1z, float tcull, float* tnear) {
    const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)),
                           fmaxf(fminf(t0z, t1z), r->tmin_box));
    const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)),
                           fminf(fmaxf(t0z, t1z), tcull));
    *tnear = tn;
    return tn <= tf;
}

static inline float key_distance(uint32_t k) {
    k &= ~7u;
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* BVH8 layout (include/igxrt.h igxrt_bvh8_node): slot boxes decoded as
 * fmaf(q, 2^exp, origin), tested with box_hit, entered nearest first. */
static int bvh8_trace_one(const igxrt_bvh8_node* nodes, uint64_t nn,
                          const igxrt_prim_record* prims, uint64_t np, const rayprep* r,
                          int anyhit, best_hit* b, uint32_t* occluded, uint32_t* nf,
                          uint32_t* pf) {
    stack_entry stack[ORC_STACK];
    int sp = 0;
    *occluded = 0;
    if (nn == 0)
        return 0;
    int32_t next = 0;
    for (;;) {
        if (next >= 0) {
            if ((uint64_t)next >= nn)
                return -1;
            const igxrt_bvh8_node* n = &nodes[next];
            ++*nf;
            const float sx = ldexpf(1.f, n->exp[0]), sy = ldexpf(1.f, n->exp[1]),
                        sz = ldexpf(1.f, n->exp[2]);
            /* ray space: plane q at fmaf(q, 2^exp / d, fmaf(origin, 1/d, -o/d))
             * while every step is a finite normal float; else world space */
            const float mx = sx * r->idir.x, my = sy * r->idir.y, mz = sz * r->idir.z;
            const float bx = fmaf(n->origin[0], r->idir.x, -r->ood.x);
            const float by = fmaf(n->origin[1], r->idir.y, -r->ood.y);
            const float bz = fmaf(n->origin[2], r->idir.z, -r->ood.z);
            const int fast = normal_step(mx) && normal_step(my) && normal_step(mz) &&
                             fabsf(bx) <= FLT_MAX && fabsf(by) <= FLT_MAX && fabsf(bz) <= FLT_MAX;
            uint32_t key[8];
            int m = 0;
            for (int c = 0; c < 8; ++c) {
                if (!(n->valid >> c & 1))
                    continue;
                float t;
                int hit;
                if (fast)
                    hit = slab_hit(r, fmaf((float)n->lo_x[c], mx, bx), fmaf((float)n->hi_x[c], mx, bx),
                                   fmaf((float)n->lo_y[c], my, by), fmaf((float)n->hi_y[c], my, by),
                                   fmaf((float)n->lo_z[c], mz, bz), fmaf((float)n->hi_z[c], mz, bz),
                                   b->tcull, &t);
                else
                    hit = box_hit(r, fmaf((float)n->lo_x[c], sx, n->origin[0]),
                                  fmaf((float)n->hi_x[c], sx, n->origin[0]),
                                  fmaf((float)n->lo_y[c], sy, n->origin[1]),
                                  fmaf((float)n->hi_y[c], sy, n->origin[1]),
                                  fmaf((float)n->lo_z[c], sz, n->origin[2]),
                                  fmaf((float)n->hi_z[c], sz, n->origin[2]), b->tcull, &t);
                if (!hit)
                    continue;
                const uint32_t k = (order_key(t) & ~7u) | (uint32_t)c;
                int j = m++;
                while (j > 0 && k < key[j - 1]) {
                    key[j] = key[j - 1];
                    --j;
                }
                key[j] = k;
            }
            if (m == 0) {
                if (!pop_live(stack, &sp, b->tcull, &next))
                    break;
            } else {
                if (sp + m - 1 > ORC_STACK)
                    return -1;
                for (int j = m - 1; j >= 1; --j) {
                    stack[sp].ref = n->child[key[j] & 7u];
                    stack[sp].tnear = key_distance(key[j]);
                    ++sp;
                }
                next = n->child[key[0] & 7u];
            }
        } else {
            uint64_t i = (uint64_t)(uint32_t)~next;
            for (;;) {
                if (i >= np)
                    return -1;
                const igxrt_prim_record* rec = &prims[i];
                ++*pf;
                if (leaf_record(r, rec, b, anyhit) && anyhit) {
                    *occluded = 1;
                    return 0;
                }
                if (rec->leaf_end)
                    break;
                ++i;
            }
            if (!pop_live(stack, &sp, b->tcull, &next))
                break;
        }
    }
    return 0;
}

typedef struct {
    uint32_t layout;
    const void* nodes;
    uint64_t nn;
    const igxrt_prim_record* prims;
    uint64_t np;
    const igxrt_ray* rays;
    const uint32_t* prev;
    uint32_t mode;
    igxrt_hit* hits;
    uint32_t* occ;
    uint32_t* nf;
    uint32_t* pf;
    _Atomic int error;
} bvh_ctx;

static void bvh_chunk(void* p, uint32_t b0, uint32_t e0) {
    bvh_ctx* c = (bvh_ctx*)p;
    for (uint32_t i = b0; i < e0; ++i) {
        rayprep r;
        prep_ray(&c->rays[i], c->prev ? c->prev[i] : IGXRT_NO_RAY_HIT, &r);
        best_hit b;
        b.t = r.tmax_eff;
        b.u = 0;
        b.v = 0;
        b.prim = 0; /* "prim < b.prim" never holds until a first hit */
        b.tcull = cull_limit(b.t);
        uint32_t occ = 0, nf = 0, pf = 0;
        int rc;
        if (c->layout == IGXRT_LAYOUT_BVH4)
            rc = bvh4_trace_one((const igxrt_bvh4_node*)c->nodes, c->nn, c->prims, c->np, &r,
                                c->mode == 1, &b, &occ, &nf, &pf);
        else if (c->layout == IGXRT_LAYOUT_BVH8)
            rc = bvh8_trace_one((const igxrt_bvh8_node*)c->nodes, c->nn, c->prims, c->np, &r,
                                c->mode == 1, &b, &occ, &nf, &pf);
        else
            rc = bvh2_trace_one((const igxrt_bvh2_node*)c->nodes, c->nn, c->prims, c->np, &r,
                                c->mode == 1, &b, &occ, &nf, &pf);
        if (rc != 0)
            atomic_store(&c->error, 1);
        if (c->mode == 1) {
            if (c->occ)
                c->occ[i] = occ;
        } else if (c->hits) {
            if (b.t < r.tmax_eff) {
                c->hits[i].t = b.t;
                c->hits[i].u = b.u;
                c->hits[i].v = b.v;
                c->hits[i].prim = b.prim;
            } else {
                c->hits[i].t = IGXRT_NO_HIT;
                c->hits[i].u = 0;
                c->hits[i].v = 0;
                c->hits[i].prim = IGXRT_NO_RAY_HIT;
            }
        }
        if (c->nf)
            c->nf[i] = nf;
        if (c->pf)
            c->pf[i] = pf;
    }
}

int orc_bvh_trace(uint32_t layout, const void* nodes, uint64_t node_count,
                  const igxrt_prim_record* prims, uint64_t prim_count, const igxrt_ray* rays,
                  const uint32_t* prev_hit, uint32_t nrays, uint32_t mode, igxrt_hit* out_hits,
                  uint32_t* out_occluded, uint32_t* node_fetches, uint32_t* prim_fetches,
                  int threads) {
    bvh_ctx c;
    c.layout = layout;
    c.nodes = nodes;
    c.nn = node_count;
    c.prims = prims;
    c.np = prim_count;
    c.rays = rays;
    c.prev = prev_hit;
    c.mode = mode;
    c.hits = out_hits;
    c.occ = out_occluded;
    c.nf = node_fetches;
    c.pf = prim_fetches;
    atomic_init(&c.error, 0);
    run_parallel(bvh_chunk, &c, nrays, 256, threads);
    return atomic_load(&c.error) ? -1 : 0;
}
