/*
 * bvh_build_oracle.c — a BVH builder of the oracle's own, for the CPU
 * reference arm of the benchmark.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference (res/shaders/trace.glsl:9-98)
 * loops over every triangle; its CPU restatement in trace_oracle.c traverses a
 * BVH so that a timed CPU run finishes.  That run must not use the engine's
 * builder, so this file builds the tree the CPU traversal walks: a binned
 * surface-area-heuristic split (16 bins per axis over the centroid bounds,
 * leaves of at most 4 triangles), single-threaded, emitted in the BVH2 node
 * and primitive-record formats of include/igxrt.h that orc_bvh_trace reads.
 *
 * Boxes are widened outward by max(2^-18 * max|coordinate|, 1e-30), so the
 * traversal's slab test (binary32 fmaf, cull limit 2^-10 above the best t)
 * never culls a triangle the reference's test accepts.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define OB_BINS 16
#define OB_LEAF 4

typedef struct {
    float lo[3], hi[3];
} obox;

static void obox_empty(obox* b) {
    for (int a = 0; a < 3; ++a) {
        b->lo[a] = INFINITY;
        b->hi[a] = -INFINITY;
    }
}

static void obox_grow(obox* b, const obox* o) {
    for (int a = 0; a < 3; ++a) {
        if (o->lo[a] < b->lo[a])
            b->lo[a] = o->lo[a];
        if (o->hi[a] > b->hi[a])
            b->hi[a] = o->hi[a];
    }
}

static double obox_area(const obox* b) {
    const double dx = (double)b->hi[0] - b->lo[0], dy = (double)b->hi[1] - b->lo[1],
                 dz = (double)b->hi[2] - b->lo[2];
    if (!(dx >= 0) || !(dy >= 0) || !(dz >= 0))
        return 0.0;
    return dx * dy + dy * dz + dz * dx;
}

typedef struct {
    const obox* boxes;   /* per triangle */
    const float* cent;   /* 3 per triangle */
    uint32_t* idx;       /* triangle order, partitioned in place */
    igxrt_bvh2_node* nodes;
    uint64_t nnodes;
    float pad;
} obuild;

/* Bounds of the triangles idx[b..e) and of their centroids. */
static void range_bounds(const obuild* s, uint32_t b, uint32_t e, obox* box, obox* cb) {
    obox_empty(box);
    obox_empty(cb);
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t t = s->idx[i];
        obox_grow(box, &s->boxes[t]);
        obox c;
        for (int a = 0; a < 3; ++a)
            c.lo[a] = c.hi[a] = s->cent[3 * t + a];
        obox_grow(cb, &c);
    }
}

/* Binned SAH split of idx[b..e): returns the split position (b < m < e). */
static uint32_t split_range(obuild* s, uint32_t b, uint32_t e, const obox* cb) {
    const uint32_t n = e - b;
    double best_cost = INFINITY;
    int best_axis = -1, best_bin = 0;
    for (int a = 0; a < 3; ++a) {
        const float lo = cb->lo[a], ext = cb->hi[a] - cb->lo[a];
        if (!(ext > 0))
            continue;
        obox bin_box[OB_BINS];
        uint32_t bin_n[OB_BINS];
        for (int k = 0; k < OB_BINS; ++k) {
            obox_empty(&bin_box[k]);
            bin_n[k] = 0;
        }
        const float scale = (float)OB_BINS / ext;
        for (uint32_t i = b; i < e; ++i) {
            const uint32_t t = s->idx[i];
            int k = (int)((s->cent[3 * t + a] - lo) * scale);
            k = k < 0 ? 0 : (k >= OB_BINS ? OB_BINS - 1 : k);
            obox_grow(&bin_box[k], &s->boxes[t]);
            ++bin_n[k];
        }
        double right_area[OB_BINS];
        uint32_t right_n[OB_BINS];
        obox acc;
        obox_empty(&acc);
        uint32_t cnt = 0;
        for (int k = OB_BINS - 1; k > 0; --k) {
            obox_grow(&acc, &bin_box[k]);
            cnt += bin_n[k];
            right_area[k] = obox_area(&acc);
            right_n[k] = cnt;
        }
        obox_empty(&acc);
        cnt = 0;
        for (int k = 0; k < OB_BINS - 1; ++k) {
            obox_grow(&acc, &bin_box[k]);
            cnt += bin_n[k];
            if (cnt == 0 || right_n[k + 1] == 0)
                continue;
            const double cost = obox_area(&acc) * cnt + right_area[k + 1] * right_n[k + 1];
            if (cost < best_cost) {
                best_cost = cost;
                best_axis = a;
                best_bin = k;
            }
        }
    }
    uint32_t m = b + n / 2;
    if (best_axis >= 0) {
        const int a = best_axis;
        const float lo = cb->lo[a], scale = (float)OB_BINS / (cb->hi[a] - cb->lo[a]);
        uint32_t i = b, j = e;
        while (i < j) {
            const uint32_t t = s->idx[i];
            int k = (int)((s->cent[3 * t + a] - lo) * scale);
            k = k < 0 ? 0 : (k >= OB_BINS ? OB_BINS - 1 : k);
            if (k <= best_bin) {
                ++i;
            } else {
                --j;
                s->idx[i] = s->idx[j];
                s->idx[j] = t;
            }
        }
        if (i > b && i < e)
            m = i;
    }
    return m; /* all centroids equal, or a one-sided split: halve the range */
}

static void padded(const obuild* s, const obox* b, float out_x[2], float out_y[2], float out_z[2]) {
    out_x[0] = b->lo[0] - s->pad;
    out_x[1] = b->hi[0] + s->pad;
    out_y[0] = b->lo[1] - s->pad;
    out_y[1] = b->hi[1] + s->pad;
    out_z[0] = b->lo[2] - s->pad;
    out_z[1] = b->hi[2] + s->pad;
}

typedef struct {
    uint32_t b, e;   /* triangle range */
    uint64_t node;   /* node whose child slot receives it */
    int slot;
    int depth;
} ojob;

/* Beyond this depth a range is halved instead of split by the heuristic, so
 * the traversal stack (ORC_STACK entries) always suffices. */
#define OB_MAX_SAH_DEPTH 48

int64_t orc_bvh_build(const igxrt_triangle* tris, uint32_t ntri, igxrt_bvh2_node* nodes,
                      igxrt_prim_record* prims) {
    if (ntri == 0)
        return 0;
    obox* boxes = (obox*)malloc(sizeof(obox) * ntri);
    float* cent = (float*)malloc(sizeof(float) * 3 * (size_t)ntri);
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * ntri);
    ojob* jobs = (ojob*)malloc(sizeof(ojob) * 2 * (size_t)ntri + 16);
    if (!boxes || !cent || !idx || !jobs) {
        free(boxes);
        free(cent);
        free(idx);
        free(jobs);
        return -1;
    }
    float maxabs = 0.f;
    for (uint32_t t = 0; t < ntri; ++t) {
        const float* p[3] = {tris[t].p0, tris[t].p1, tris[t].p2};
        for (int a = 0; a < 3; ++a) {
            float lo = p[0][a], hi = p[0][a];
            for (int v = 1; v < 3; ++v) {
                lo = p[v][a] < lo ? p[v][a] : lo;
                hi = p[v][a] > hi ? p[v][a] : hi;
            }
            boxes[t].lo[a] = lo;
            boxes[t].hi[a] = hi;
            cent[3 * t + a] = 0.5f * lo + 0.5f * hi;
            maxabs = fabsf(lo) > maxabs ? fabsf(lo) : maxabs;
            maxabs = fabsf(hi) > maxabs ? fabsf(hi) : maxabs;
        }
        idx[t] = t;
    }
    obuild s = {boxes, cent, idx, nodes, 0, fmaxf(maxabs * 0x1p-18f, 1e-30f)};

    /* node 0 holds the root range in slot 0 (slot 1 absent) when it is a
     * single leaf; otherwise node 0 is the root's split */
    uint32_t nprim = 0;
    size_t njobs = 0;
    obox box, cb;
    range_bounds(&s, 0, ntri, &box, &cb);
    memset(&nodes[0], 0, sizeof(igxrt_bvh2_node));
    s.nnodes = 1;
    if (ntri <= OB_LEAF) {
        padded(&s, &box, nodes[0].c0_x, nodes[0].c0_y, nodes[0].c0_z);
        nodes[0].c1_x[0] = nodes[0].c1_x[1] = INFINITY;
        nodes[0].c1_y[0] = nodes[0].c1_y[1] = INFINITY;
        nodes[0].c1_z[0] = nodes[0].c1_z[1] = INFINITY;
        nodes[0].child[1] = -1; /* never entered: its box is empty */
        jobs[njobs++] = (ojob){0, ntri, 0, 0, 1};
    } else {
        const uint32_t m = split_range(&s, 0, ntri, &cb);
        jobs[njobs++] = (ojob){m, ntri, 0, 1, 1};
        jobs[njobs++] = (ojob){0, m, 0, 0, 1};
    }
    while (njobs) {
        const ojob j = jobs[--njobs];
        igxrt_bvh2_node* parent = &nodes[j.node];
        range_bounds(&s, j.b, j.e, &box, &cb);
        if (j.slot == 0)
            padded(&s, &box, parent->c0_x, parent->c0_y, parent->c0_z);
        else
            padded(&s, &box, parent->c1_x, parent->c1_y, parent->c1_z);
        if (j.e - j.b <= OB_LEAF) {
            parent->child[j.slot] = ~(int32_t)nprim;
            for (uint32_t i = j.b; i < j.e; ++i) {
                const igxrt_triangle* t = &tris[idx[i]];
                igxrt_prim_record* r = &prims[nprim++];
                for (int a = 0; a < 3; ++a) {
                    r->p0[a] = t->p0[a];
                    r->e1[a] = t->p1[a] - t->p0[a]; /* primitive.glsl:245-246 */
                    r->e2[a] = t->p2[a] - t->p0[a];
                }
                r->prim = idx[i];
                r->leaf_end = i + 1 == j.e;
                r->pad = 0;
            }
            continue;
        }
        const uint64_t me = s.nnodes++;
        memset(&nodes[me], 0, sizeof(igxrt_bvh2_node));
        parent->child[j.slot] = (int32_t)me;
        const uint32_t m = j.depth < OB_MAX_SAH_DEPTH ? split_range(&s, j.b, j.e, &cb)
                                                      : j.b + (j.e - j.b) / 2;
        jobs[njobs++] = (ojob){m, j.e, me, 1, j.depth + 1};
        jobs[njobs++] = (ojob){j.b, m, me, 0, j.depth + 1};
    }
    free(boxes);
    free(cent);
    free(idx);
    free(jobs);
    return (int64_t)s.nnodes;
}
