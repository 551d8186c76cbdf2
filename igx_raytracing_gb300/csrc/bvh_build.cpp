// bvh_build.cpp — host BVH builder, validator and (de)serialiser.
//
// The reference has no acceleration structure: traceGeometry and
// traceOcclusion (res/shaders/trace.glsl:9-98) test every primitive.  This
// builder produces the BVH the CUDA kernels traverse instead:
//   * binned SAH over triangle centroids (32 bins by default), leaves of at
//     most `max_leaf_size` triangles, a median split below depth
//     kMaxDepth - 24 so the depth stays bounded;
//   * the BVH2 layout (64-byte nodes with both child boxes) and a BVH4 layout
//     (128-byte nodes) collapsed from the same binary tree, sharing one array
//     of 48-byte primitive records in leaf order;
//   * every box widened outward by pad_abs = 2^-18 * max|coordinate| so the
//     kernels' binary32 slab test never culls a box whose triangle the
//     reference's test would accept (rounding of the slab distances is below
//     2^-23 * max|coordinate| for ray origins within that magnitude).
// Host code is compiled with -ffp-contract=off so the tree is bit-identical on
// every host architecture.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>

#include "internal.h"

namespace igxrt {

std::string format(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return std::string(buf);
}

namespace {

constexpr float kInf = INFINITY;

// The {+inf, +inf} slab of an absent child.
bool slot_empty(float lo, float hi) { return lo == kInf && hi == kInf; }

struct Aabb {
    float lo[3], hi[3];
    void reset() {
        for (int a = 0; a < 3; ++a) {
            lo[a] = kInf;
            hi[a] = -kInf;
        }
    }
    void grow(const Aabb& b) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow_point(const float* p) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    // Half surface area; 0 for an empty box.
    float half_area() const {
        if (!(hi[0] >= lo[0]))
            return 0.f;
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
};

struct BNode {
    Aabb box;
    uint32_t left = 0, right = 0;
    uint32_t first = 0, count = 0;  // count > 0: leaf over refs[first, first+count)
    bool leaf() const { return count > 0; }
};

struct Builder {
    const igxrt_scene_desc* d = nullptr;  // primitives: triangles, spheres, cubes
    uint32_t n = 0;
    uint32_t max_leaf = 8;
    uint32_t bins = 32;
    float cn = 1.f, ct = 1.f;
    std::vector<Aabb> tb;
    std::vector<float> cen;  // 3 per triangle
    std::vector<uint32_t> refs;
    std::vector<BNode> nodes;
    std::atomic<uint32_t> node_count{0};
    std::atomic<int> spare_threads{0};

    uint32_t build(uint32_t begin, uint32_t end, uint32_t depth);
    uint32_t split_median(uint32_t begin, uint32_t end, const Aabb& cb);
};

uint32_t Builder::split_median(uint32_t begin, uint32_t end, const Aabb& cb) {
    int axis = 0;
    float best = -1.f;
    for (int a = 0; a < 3; ++a) {
        const float e = cb.hi[a] - cb.lo[a];
        if (e > best) {
            best = e;
            axis = a;
        }
    }
    const uint32_t mid = begin + (end - begin) / 2;
    const float* c = cen.data();
    std::nth_element(refs.begin() + begin, refs.begin() + mid, refs.begin() + end,
                     [c, axis](uint32_t x, uint32_t y) {
                         const float cx = c[3 * x + axis], cy = c[3 * y + axis];
                         return cx < cy || (cx == cy && x < y);
                     });
    return mid;
}

uint32_t Builder::build(uint32_t begin, uint32_t end, uint32_t depth) {
    const uint32_t id = node_count.fetch_add(1);
    BNode& nd = nodes[id];
    const uint32_t cnt = end - begin;
    Aabb box, cb;
    box.reset();
    cb.reset();
    for (uint32_t i = begin; i < end; ++i) {
        const uint32_t r = refs[i];
        box.grow(tb[r]);
        cb.grow_point(&cen[3 * r]);
    }
    nd.box = box;
    auto make_leaf = [&]() {
        nd.first = begin;
        nd.count = cnt;
        return id;
    };
    if (cnt == 1)
        return make_leaf();

    uint32_t mid = begin;
    if (depth + 24 >= kMaxDepth) {
        if (cnt <= max_leaf)
            return make_leaf();
        mid = split_median(begin, end, cb);
    } else {
        float best_cost = kInf;
        int best_axis = -1;
        uint32_t best_bin = 0;
        std::vector<uint32_t> bcount(bins);
        std::vector<Aabb> bbox(bins);
        std::vector<float> right_area(bins);
        std::vector<uint32_t> right_count(bins);
        for (int a = 0; a < 3; ++a) {
            const float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.f))
                continue;
            const float scale = (float)bins / ext;
            const float cmin = cb.lo[a];
            std::fill(bcount.begin(), bcount.end(), 0u);
            for (auto& b : bbox)
                b.reset();
            for (uint32_t i = begin; i < end; ++i) {
                const uint32_t r = refs[i];
                int b = (int)((cen[3 * r + a] - cmin) * scale);
                b = std::min(std::max(b, 0), (int)bins - 1);
                ++bcount[b];
                bbox[b].grow(tb[r]);
            }
            Aabb acc;
            acc.reset();
            uint32_t nacc = 0;
            for (int b = (int)bins - 1; b > 0; --b) {
                acc.grow(bbox[b]);
                nacc += bcount[b];
                right_area[b] = acc.half_area();
                right_count[b] = nacc;
            }
            acc.reset();
            nacc = 0;
            for (uint32_t b = 0; b + 1 < bins; ++b) {
                acc.grow(bbox[b]);
                nacc += bcount[b];
                const uint32_t nr = right_count[b + 1];
                if (nacc == 0 || nr == 0)
                    continue;
                const float cost = acc.half_area() * (float)nacc + right_area[b + 1] * (float)nr;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_bin = b;
                }
            }
        }
        if (best_axis < 0) {
            // All centroids coincide: no SAH plane separates them.
            if (cnt <= max_leaf)
                return make_leaf();
            mid = begin + cnt / 2;
        } else {
            const float parent_area = box.half_area();
            const float split_cost =
                parent_area > 0.f ? cn + ct * best_cost / parent_area : cn + ct * (float)cnt;
            const float leaf_cost = ct * (float)cnt;
            if (cnt <= max_leaf && leaf_cost <= split_cost)
                return make_leaf();
            const float scale = (float)bins / (cb.hi[best_axis] - cb.lo[best_axis]);
            const float cmin = cb.lo[best_axis];
            const float* c = cen.data();
            const int ax = best_axis;
            const uint32_t bb = best_bin, nb = bins;
            auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](uint32_t r) {
                int b = (int)((c[3 * r + ax] - cmin) * scale);
                b = std::min(std::max(b, 0), (int)nb - 1);
                return (uint32_t)b <= bb;
            });
            mid = (uint32_t)(it - refs.begin());
            if (mid == begin || mid == end)
                mid = split_median(begin, end, cb);
        }
    }

    uint32_t l = 0, r = 0;
    bool spawned = false;
    std::thread worker;
    if (cnt >= 65536) {
        int s = spare_threads.load();
        while (s > 0 && !spare_threads.compare_exchange_weak(s, s - 1)) {
        }
        if (s > 0) {
            spawned = true;
            worker = std::thread([&]() {
                l = build(begin, mid, depth + 1);
                spare_threads.fetch_add(1);
            });
        }
    }
    if (!spawned)
        l = build(begin, mid, depth + 1);
    r = build(mid, end, depth + 1);
    if (spawned)
        worker.join();
    nd.left = l;
    nd.right = r;
    return id;
}

struct Layout {
    const Builder& b;
    igxrt_bvh& out;
    float pad;
    std::vector<uint32_t> leaf_rec;  // build node -> first primitive record
    uint32_t max_depth = 0;
    double sah_nodes = 0, sah_tris = 0;

    void set_box(float* lo_hi_x, float* lo_hi_y, float* lo_hi_z, const Aabb& a) const {
        lo_hi_x[0] = a.lo[0] - pad;
        lo_hi_x[1] = a.hi[0] + pad;
        lo_hi_y[0] = a.lo[1] - pad;
        lo_hi_y[1] = a.hi[1] + pad;
        lo_hi_z[0] = a.lo[2] - pad;
        lo_hi_z[1] = a.hi[2] + pad;
    }

    int32_t emit_leaf(uint32_t id) {
        const BNode& nd = b.nodes[id];
        const uint32_t first = (uint32_t)out.prims.size();
        leaf_rec[id] = first;
        const uint32_t nt = b.d->triangle_count, ns = b.d->sphere_count;
        for (uint32_t k = 0; k < nd.count; ++k) {
            const uint32_t t = b.refs[nd.first + k];  // global object id
            igxrt_prim_record rec{};
            if (t < nt) {
                const igxrt_triangle& tri = b.d->triangles[t];
                for (int a = 0; a < 3; ++a) {
                    rec.p0[a] = tri.p0[a];
                    rec.e1[a] = tri.p1[a] - tri.p0[a];
                    rec.e2[a] = tri.p2[a] - tri.p0[a];
                }
                rec.pad = kPrimTriangle;
            } else if (t < nt + ns) {
                const float* s = b.d->spheres + 4 * (size_t)(t - nt);
                for (int a = 0; a < 3; ++a)
                    rec.p0[a] = s[a];
                rec.e1[0] = s[3];
                rec.pad = kPrimSphere;
            } else {
                const igxrt_cube& c = b.d->cubes[t - nt - ns];
                const float start[3] = {c.xy0[0], c.xy0[1], c.z0_x1[0]};
                const float end[3] = {c.z0_x1[1], c.yz1[0], c.yz1[1]};
                for (int a = 0; a < 3; ++a) {
                    rec.p0[a] = start[a];
                    rec.e1[a] = end[a];
                }
                rec.pad = kPrimCube;
            }
            rec.prim = t;
            rec.leaf_end = (k + 1 == nd.count) ? 1u : 0u;
            out.prims.push_back(rec);
        }
        return ~(int32_t)first;
    }

    int32_t emit2(uint32_t id, uint32_t depth) {
        const BNode& nd = b.nodes[id];
        max_depth = std::max(max_depth, depth);
        const uint32_t idx = (uint32_t)out.nodes2.size();
        out.nodes2.push_back(igxrt_bvh2_node{});
        const uint32_t kids[2] = {nd.left, nd.right};
        int32_t refs[2];
        for (int c = 0; c < 2; ++c) {
            const BNode& k = b.nodes[kids[c]];
            refs[c] = k.leaf() ? emit_leaf(kids[c]) : emit2(kids[c], depth + 1);
        }
        igxrt_bvh2_node& o = out.nodes2[idx];
        set_box(o.c0_x, o.c0_y, o.c0_z, b.nodes[kids[0]].box);
        set_box(o.c1_x, o.c1_y, o.c1_z, b.nodes[kids[1]].box);
        o.child[0] = refs[0];
        o.child[1] = refs[1];
        o.pad[0] = o.pad[1] = 0;
        return (int32_t)idx;
    }

    int32_t emit4(uint32_t id) {
        std::vector<uint32_t> kids = {b.nodes[id].left, b.nodes[id].right};
        while (kids.size() < 4) {
            int pick = -1;
            float best = -1.f;
            for (size_t k = 0; k < kids.size(); ++k) {
                const BNode& c = b.nodes[kids[k]];
                if (!c.leaf() && c.box.half_area() > best) {
                    best = c.box.half_area();
                    pick = (int)k;
                }
            }
            if (pick < 0)
                break;
            const BNode& c = b.nodes[kids[pick]];
            const uint32_t l = c.left, r = c.right;
            kids[pick] = l;
            kids.insert(kids.begin() + pick + 1, r);
        }
        const uint32_t idx = (uint32_t)out.nodes4.size();
        out.nodes4.push_back(igxrt_bvh4_node{});
        int32_t refs[4] = {0, 0, 0, 0};
        for (size_t k = 0; k < kids.size(); ++k) {
            const BNode& c = b.nodes[kids[k]];
            refs[k] = c.leaf() ? ~(int32_t)leaf_rec[kids[k]] : emit4(kids[k]);
        }
        igxrt_bvh4_node& o = out.nodes4[idx];
        for (int k = 0; k < 4; ++k) {
            if ((size_t)k < kids.size()) {
                const Aabb& a = b.nodes[kids[k]].box;
                o.lo_x[k] = a.lo[0] - pad;
                o.hi_x[k] = a.hi[0] + pad;
                o.lo_y[k] = a.lo[1] - pad;
                o.hi_y[k] = a.hi[1] + pad;
                o.lo_z[k] = a.lo[2] - pad;
                o.hi_z[k] = a.hi[2] + pad;
                o.child[k] = refs[k];
            } else {
                o.lo_x[k] = o.hi_x[k] = kInf;
                o.lo_y[k] = o.hi_y[k] = kInf;
                o.lo_z[k] = o.hi_z[k] = kInf;
                o.child[k] = 0;
            }
            o.pad[k] = 0;
        }
        return (int32_t)idx;
    }

    void sah(uint32_t id, float root_area) {
        const BNode& nd = b.nodes[id];
        const double rel = root_area > 0.f ? (double)nd.box.half_area() / root_area : 1.0;
        if (nd.leaf()) {
            sah_tris += rel * nd.count;
            return;
        }
        sah_nodes += rel;
        sah(nd.left, root_area);
        sah(nd.right, root_area);
    }
};

void empty_slot2(float* x, float* y, float* z) {
    x[0] = x[1] = y[0] = y[1] = z[0] = z[1] = kInf;
}

// Largest traversal stack any ray can need: along a root-to-leaf path each
// node pushes (entered children - 1) entries, at most (non-empty slots - 1).
uint32_t stack_bound2(const std::vector<igxrt_bvh2_node>& n, int32_t i) {
    const igxrt_bvh2_node& x = n[i];
    const bool e1 = x.c1_x[0] == kInf && x.c1_x[1] == kInf;
    uint32_t deepest = 0;
    for (int c = 0; c < (e1 ? 1 : 2); ++c)
        if (x.child[c] >= 0)
            deepest = std::max(deepest, stack_bound2(n, x.child[c]));
    return deepest + (e1 ? 0u : 1u);
}

uint32_t stack_bound8(const std::vector<igxrt_bvh8_node>& n, int32_t i) {
    const igxrt_bvh8_node& x = n[i];
    uint32_t deepest = 0, used = 0;
    for (int c = 0; c < 8; ++c) {
        if (!(x.valid >> c & 1))
            continue;
        ++used;
        if (x.child[c] >= 0)
            deepest = std::max(deepest, stack_bound8(n, x.child[c]));
    }
    return deepest + (used ? used - 1 : 0);
}

// BVH8 from the BVH2 arrays: a node takes its BVH2 node's slots and opens the
// interior slot of largest area until eight slots are used; interior slots
// become BVH8 nodes (preorder), leaf slots keep their record ranges.  Every
// slot remembers its BVH2 source so the refit can re-quantize it.
struct Bvh8Emitter {
    igxrt_bvh& b;

    static float slot_area(const igxrt_bvh2_node& m, int c) {
        const float* x = c ? m.c1_x : m.c0_x;
        const float* y = c ? m.c1_y : m.c0_y;
        const float* z = c ? m.c1_z : m.c0_z;
        const float dx = x[1] - x[0], dy = y[1] - y[0], dz = z[1] - z[0];
        return dx * dy + dy * dz + dz * dx;
    }

    uint32_t emit(uint32_t node2) {
        struct Kid {
            int32_t ref;
            uint32_t src;
            float area;
        };
        Kid kids[8];
        int used = 0;
        auto add_slots = [&](uint32_t k, int at) {
            const igxrt_bvh2_node& m = b.nodes2[k];
            Kid got[2];
            int n = 0;
            for (int c = 0; c < 2; ++c) {
                const float* x = c ? m.c1_x : m.c0_x;
                if (slot_empty(x[0], x[1]))
                    continue;
                got[n++] = Kid{m.child[c], 2 * k + (uint32_t)c, slot_area(m, c)};
            }
            // replace kids[at] (or append when at == used) by the n slots
            const int tail = at < used ? at + 1 : used;
            for (int s = used - 1; s >= tail; --s)
                kids[s + n - (at < used ? 1 : 0)] = kids[s];
            for (int s = 0; s < n; ++s)
                kids[at + s] = got[s];
            used += n - (at < used ? 1 : 0);
        };
        add_slots(node2, 0);
        while (used < 8) {
            int pick = -1;
            float best = -1.f;
            for (int s = 0; s < used; ++s)
                if (kids[s].ref >= 0 && kids[s].area > best) {
                    best = kids[s].area;
                    pick = s;
                }
            if (pick < 0)
                break;
            add_slots((uint32_t)kids[pick].ref, pick);
        }
        const uint32_t idx = (uint32_t)b.nodes8.size();
        b.nodes8.push_back(igxrt_bvh8_node{});
        b.src8.resize(b.src8.size() + 8, kNoSource);
        int32_t child[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int s = 0; s < used; ++s)
            child[s] = kids[s].ref >= 0 ? (int32_t)emit((uint32_t)kids[s].ref) : kids[s].ref;
        igxrt_bvh8_node& o = b.nodes8[idx];
        for (int s = 0; s < used; ++s) {
            o.valid |= (uint8_t)(1u << s);
            o.child[s] = child[s];
            b.src8[8 * (size_t)idx + s] = kids[s].src;
        }
        bvh8_quantize_node(b.nodes2.data(), &b.src8[8 * (size_t)idx], o);
        return idx;
    }
};

// Adds the BVH8 layout to a built tree, or leaves it out (bvh8_nodes = 0)
// when its traversal stack would exceed the kernels' capacity.
void add_bvh8(igxrt_bvh& b) {
    b.nodes8.clear();
    b.src8.clear();
    b.info.bvh8_nodes = 0;
    b.info.max_stack[IGXRT_LAYOUT_BVH8] = 0;
    if (b.nodes2.empty())
        return;
    Bvh8Emitter{b}.emit(0);
    const uint32_t bound = stack_bound8(b.nodes8, 0);
    if (bound > kStackCapacity) {
        b.nodes8.clear();
        b.src8.clear();
        return;
    }
    b.info.bvh8_nodes = (uint32_t)b.nodes8.size();
    b.info.max_stack[IGXRT_LAYOUT_BVH8] = bound;
}

uint32_t stack_bound4(const std::vector<igxrt_bvh4_node>& n, int32_t i) {
    const igxrt_bvh4_node& x = n[i];
    uint32_t deepest = 0, used = 0;
    for (int c = 0; c < 4; ++c) {
        if (x.lo_x[c] == kInf && x.hi_x[c] == kInf)
            continue;
        ++used;
        if (x.child[c] >= 0)
            deepest = std::max(deepest, stack_bound4(n, x.child[c]));
    }
    return deepest + (used ? used - 1 : 0);
}

}  // namespace

igxrt_status build_bvh(const igxrt_triangle* tris, uint32_t count, const igxrt_build_options* opts,
                       igxrt_bvh& out, std::string& err) {
    igxrt_scene_desc d{};
    d.triangles = tris;
    d.triangle_count = count;
    return build_bvh_mixed(d, opts, out, err);
}

igxrt_status build_bvh_mixed(const igxrt_scene_desc& d, const igxrt_build_options* opts,
                             igxrt_bvh& out, std::string& err) {
    out = igxrt_bvh{};
    if ((d.triangle_count && !d.triangles) || (d.sphere_count && !d.spheres) ||
        (d.cube_count && !d.cubes) || (d.plane_count && !d.planes)) {
        err = "a primitive buffer with a non-zero count is NULL";
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    const uint64_t total = (uint64_t)d.triangle_count + d.sphere_count + d.cube_count;
    if (total + d.plane_count >= 0x7fffffffu) {
        err = "too many primitives";
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    const uint32_t count = (uint32_t)total;  // primitives in the tree
    Builder b;
    b.d = &d;
    b.n = count;
    if (opts) {
        if (opts->max_leaf_size)
            b.max_leaf = opts->max_leaf_size;
        if (opts->sah_bins)
            b.bins = opts->sah_bins;
        if (opts->node_cost > 0)
            b.cn = opts->node_cost;
        if (opts->tri_cost > 0)
            b.ct = opts->tri_cost;
    }
    if (b.max_leaf < 1 || b.max_leaf > 16) {
        err = format("max_leaf_size %u outside 1..16", b.max_leaf);
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    if (b.bins < 2 || b.bins > 256) {
        err = format("sah_bins %u outside 2..256", b.bins);
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    unsigned hw = std::thread::hardware_concurrency();
    unsigned threads = (opts && opts->threads) ? opts->threads : (hw ? hw : 1);
    b.spare_threads = (int)threads - 1;

    const uint32_t nt = d.triangle_count, ns = d.sphere_count, nc = d.cube_count;
    out.tris.assign(d.triangles, d.triangles + nt);
    out.spheres.assign(d.spheres, d.spheres + 4 * (size_t)ns);
    out.cubes.assign(d.cubes, d.cubes + nc);
    out.planes.assign(d.planes, d.planes + 4 * (size_t)d.plane_count);
    for (float v : out.planes)
        if (!std::isfinite(v)) {
            err = "a plane has a non-finite coefficient";
            out = igxrt_bvh{};
            return IGXRT_ERROR_INVALID_ARGUMENT;
        }
    Aabb scene;
    scene.reset();
    float maxabs = 0.f;
    b.tb.resize(count);
    b.cen.resize(3 * (size_t)count);
    b.refs.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        float v[3][3];
        int nv;
        if (i < nt) {
            const igxrt_triangle& t = d.triangles[i];
            for (int c = 0; c < 3; ++c) {
                v[0][c] = t.p0[c];
                v[1][c] = t.p1[c];
                v[2][c] = t.p2[c];
            }
            nv = 3;
        } else if (i < nt + ns) {
            // the sphere's box: centre -/+ |radius| (the test squares the radius)
            const float* s = d.spheres + 4 * (size_t)(i - nt);
            const float r = std::fabs(s[3]);
            for (int c = 0; c < 3; ++c) {  // a non-finite radius fails the check below
                v[0][c] = s[c] - r;
                v[1][c] = s[c] + r;
            }
            nv = 2;
        } else {
            const igxrt_cube& cb = d.cubes[i - nt - ns];
            const float start[3] = {cb.xy0[0], cb.xy0[1], cb.z0_x1[0]};
            const float end[3] = {cb.z0_x1[1], cb.yz1[0], cb.yz1[1]};
            for (int c = 0; c < 3; ++c) {
                v[0][c] = start[c];
                v[1][c] = end[c];
            }
            nv = 2;
        }
        Aabb a;
        a.reset();
        for (int k = 0; k < nv; ++k) {
            for (int c = 0; c < 3; ++c) {
                if (!std::isfinite(v[k][c])) {
                    err = format("primitive %u has a non-finite coordinate", i);
                    out = igxrt_bvh{};
                    return IGXRT_ERROR_INVALID_ARGUMENT;
                }
                maxabs = std::max(maxabs, std::fabs(v[k][c]));
            }
            a.grow_point(v[k]);
        }
        b.tb[i] = a;
        for (int c = 0; c < 3; ++c)
            b.cen[3 * (size_t)i + c] = (a.lo[c] + a.hi[c]) * 0.5f;
        b.refs[i] = i;
        scene.grow(a);
    }

    igxrt_bvh_info& info = out.info;
    info.triangle_count = nt;
    info.sphere_count = ns;
    info.cube_count = nc;
    info.plane_count = d.plane_count;
    info.max_leaf_size = b.max_leaf;
    const float pad = std::max(maxabs * 0x1p-18f, 1e-30f);
    info.pad_abs = pad;
    for (int a = 0; a < 3; ++a) {
        info.bounds[a] = count ? scene.lo[a] : 0.f;
        info.bounds[3 + a] = count ? scene.hi[a] : 0.f;
    }
    if (count == 0)
        return IGXRT_OK;

    b.nodes.resize(2 * (size_t)count);
    const uint32_t root = b.build(0, count, 0);

    Layout lay{b, out, pad, std::vector<uint32_t>(b.nodes.size(), 0xffffffffu)};
    out.prims.reserve(count);
    const BNode& rn = b.nodes[root];
    if (rn.leaf()) {
        // A one-leaf scene still needs a root node: the leaf sits in slot 0.
        igxrt_bvh2_node n2{};
        const int32_t ref = lay.emit_leaf(root);
        lay.set_box(n2.c0_x, n2.c0_y, n2.c0_z, rn.box);
        empty_slot2(n2.c1_x, n2.c1_y, n2.c1_z);
        n2.child[0] = ref;
        n2.child[1] = 0;
        out.nodes2.push_back(n2);
        igxrt_bvh4_node n4{};
        for (int k = 0; k < 4; ++k) {
            n4.lo_x[k] = n4.hi_x[k] = n4.lo_y[k] = n4.hi_y[k] = n4.lo_z[k] = n4.hi_z[k] = kInf;
            n4.child[k] = 0;
        }
        n4.lo_x[0] = rn.box.lo[0] - pad;
        n4.hi_x[0] = rn.box.hi[0] + pad;
        n4.lo_y[0] = rn.box.lo[1] - pad;
        n4.hi_y[0] = rn.box.hi[1] + pad;
        n4.lo_z[0] = rn.box.lo[2] - pad;
        n4.hi_z[0] = rn.box.hi[2] + pad;
        n4.child[0] = ref;
        out.nodes4.push_back(n4);
        lay.max_depth = 1;
        info.leaf_count = 1;
    } else {
        out.nodes2.reserve(count);
        lay.emit2(root, 1);
        lay.emit4(root);
        info.leaf_count = 0;
        for (const auto& p : out.prims)
            info.leaf_count += p.leaf_end;
    }
    lay.sah(root, rn.box.half_area());
    info.sah_cost = (float)(b.cn * lay.sah_nodes + b.ct * lay.sah_tris);
    info.max_depth = lay.max_depth;
    info.max_stack[IGXRT_LAYOUT_BVH2] = stack_bound2(out.nodes2, 0);
    info.max_stack[IGXRT_LAYOUT_BVH4] = stack_bound4(out.nodes4, 0);
    info.bvh2_nodes = (uint32_t)out.nodes2.size();
    info.bvh4_nodes = (uint32_t)out.nodes4.size();
    add_bvh8(out);
    info.device_bytes = sizeof(igxrt_bvh2_node) * out.nodes2.size() +
                        sizeof(igxrt_bvh4_node) * out.nodes4.size() +
                        sizeof(igxrt_bvh8_node) * out.nodes8.size() + sizeof(uint32_t) * out.src8.size() +
                        sizeof(igxrt_prim_record) * out.prims.size() +
                        sizeof(igxrt_triangle) * out.tris.size() +
                        sizeof(float) * out.planes.size();
    return IGXRT_OK;
}

// ------------------------------------------------------------------------
// Refit (host): new primitive positions, same topology
// ------------------------------------------------------------------------

namespace {

// Bounds of object `id` in a scene description by the builder's rule (the
// points it bounds: triangle vertices, sphere centre -/+ |radius|, cube
// corners); `finite` and `maxabs` cover the same points.
Aabb object_bounds(const igxrt_scene_desc& d, uint32_t id, bool& finite, float& maxabs) {
    const uint32_t nt = d.triangle_count, ns = d.sphere_count;
    float v[3][3];
    int nv;
    if (id < nt) {
        const igxrt_triangle& t = d.triangles[id];
        for (int c = 0; c < 3; ++c) {
            v[0][c] = t.p0[c];
            v[1][c] = t.p1[c];
            v[2][c] = t.p2[c];
        }
        nv = 3;
    } else if (id < nt + ns) {
        const float* s = d.spheres + 4 * (size_t)(id - nt);
        const float r = std::fabs(s[3]);
        for (int c = 0; c < 3; ++c) {
            v[0][c] = s[c] - r;
            v[1][c] = s[c] + r;
        }
        nv = 2;
    } else {
        const igxrt_cube& cb = d.cubes[id - nt - ns];
        const float start[3] = {cb.xy0[0], cb.xy0[1], cb.z0_x1[0]};
        const float end[3] = {cb.z0_x1[1], cb.yz1[0], cb.yz1[1]};
        for (int c = 0; c < 3; ++c) {
            v[0][c] = start[c];
            v[1][c] = end[c];
        }
        nv = 2;
    }
    Aabb a;
    a.reset();
    finite = true;
    for (int k = 0; k < nv; ++k) {
        for (int c = 0; c < 3; ++c) {
            finite = finite && std::isfinite(v[k][c]);
            maxabs = std::max(maxabs, std::fabs(v[k][c]));
        }
        a.grow_point(v[k]);
    }
    return a;
}

}  // namespace

igxrt_status refit_bvh(igxrt_bvh& b, const igxrt_scene_desc& d, std::string& err) {
    if (d.triangle_count != b.tris.size() || d.sphere_count != b.spheres.size() / 4 ||
        d.cube_count != b.cubes.size() || d.plane_count != b.planes.size() / 4) {
        err = "refit needs the primitive counts of the build";
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    if ((d.triangle_count && !d.triangles) || (d.sphere_count && !d.spheres) ||
        (d.cube_count && !d.cubes) || (d.plane_count && !d.planes)) {
        err = "a primitive buffer with a non-zero count is NULL";
        return IGXRT_ERROR_INVALID_ARGUMENT;
    }
    const uint32_t n = (uint32_t)b.prims.size();
    std::vector<Aabb> bounds(n);
    float maxabs = 0.f;
    for (uint32_t id = 0; id < n; ++id) {
        bool finite;
        bounds[id] = object_bounds(d, id, finite, maxabs);
        if (!finite) {
            err = format("primitive %u has a non-finite coordinate", id);
            return IGXRT_ERROR_INVALID_ARGUMENT;
        }
    }
    for (uint32_t i = 0; i < d.plane_count * 4; ++i)
        if (!std::isfinite(d.planes[i])) {
            err = format("plane %u has a non-finite coefficient", i / 4);
            return IGXRT_ERROR_INVALID_ARGUMENT;
        }
    const float pad = std::max(maxabs * 0x1p-18f, 1e-30f);
    b.tris.assign(d.triangles, d.triangles + d.triangle_count);
    b.spheres.assign(d.spheres, d.spheres + 4 * (size_t)d.sphere_count);
    b.cubes.assign(d.cubes, d.cubes + d.cube_count);
    b.planes.assign(d.planes, d.planes + 4 * (size_t)d.plane_count);
    const uint32_t nt = d.triangle_count, ns = d.sphere_count;
    for (auto& r : b.prims) {
        const uint32_t id = r.prim;
        if (id < nt) {
            const igxrt_triangle& t = d.triangles[id];
            for (int a = 0; a < 3; ++a) {
                r.p0[a] = t.p0[a];
                r.e1[a] = t.p1[a] - t.p0[a];
                r.e2[a] = t.p2[a] - t.p0[a];
            }
        } else if (id < nt + ns) {
            const float* s = d.spheres + 4 * (size_t)(id - nt);
            for (int a = 0; a < 3; ++a)
                r.p0[a] = s[a];
            r.e1[0] = s[3];
        } else {
            const igxrt_cube& c = d.cubes[id - nt - ns];
            const float start[3] = {c.xy0[0], c.xy0[1], c.z0_x1[0]};
            const float end[3] = {c.z0_x1[1], c.yz1[0], c.yz1[1]};
            for (int a = 0; a < 3; ++a) {
                r.p0[a] = start[a];
                r.e1[a] = end[a];
            }
        }
    }
    auto leaf_box = [&](int32_t ref) {
        Aabb a;
        a.reset();
        for (uint32_t i = (uint32_t)~ref;; ++i) {
            a.grow(bounds[b.prims[i].prim]);
            if (b.prims[i].leaf_end)
                break;
        }
        return a;
    };
    auto padded = [pad](const Aabb& a, float* lo, float* hi) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = a.lo[k] - pad;
            hi[k] = a.hi[k] + pad;
        }
    };
    // children before parents: reversed depth-first order from the root (the
    // host builder's arrays are preorder already, GPU-built ones are not)
    auto bottom_up = [](size_t count, auto&& kids) {
        std::vector<uint32_t> order, stack;
        order.reserve(count);
        if (count)
            stack.push_back(0);
        while (!stack.empty() && order.size() < count) {
            const uint32_t i = stack.back();
            stack.pop_back();
            order.push_back(i);
            kids(i, stack);
        }
        std::reverse(order.begin(), order.end());
        return order;
    };
    const std::vector<uint32_t> order2 = bottom_up(b.nodes2.size(), [&](uint32_t i, std::vector<uint32_t>& st) {
        const igxrt_bvh2_node& nd = b.nodes2[i];
        for (int c = 0; c < 2; ++c) {
            const float* x = c ? nd.c1_x : nd.c0_x;
            if (!slot_empty(x[0], x[1]) && nd.child[c] >= 0 && (size_t)nd.child[c] < b.nodes2.size())
                st.push_back((uint32_t)nd.child[c]);
        }
    });
    const std::vector<uint32_t> order4 = bottom_up(b.nodes4.size(), [&](uint32_t i, std::vector<uint32_t>& st) {
        const igxrt_bvh4_node& nd = b.nodes4[i];
        for (int c = 0; c < 4; ++c)
            if (!slot_empty(nd.lo_x[c], nd.hi_x[c]) && nd.child[c] >= 0 && (size_t)nd.child[c] < b.nodes4.size())
                st.push_back((uint32_t)nd.child[c]);
    });
    for (const uint32_t i : order2) {
        igxrt_bvh2_node& nd = b.nodes2[i];
        for (int c = 0; c < 2; ++c) {
            float* x = c ? nd.c1_x : nd.c0_x;
            float* y = c ? nd.c1_y : nd.c0_y;
            float* z = c ? nd.c1_z : nd.c0_z;
            if (slot_empty(x[0], x[1]))
                continue;
            float lo[3], hi[3];
            if (nd.child[c] < 0) {
                padded(leaf_box(nd.child[c]), lo, hi);
            } else {
                const igxrt_bvh2_node& m = b.nodes2[nd.child[c]];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = kInf;
                    hi[k] = -kInf;
                }
                for (int g = 0; g < 2; ++g) {
                    const float* gx = g ? m.c1_x : m.c0_x;
                    const float* gy = g ? m.c1_y : m.c0_y;
                    const float* gz = g ? m.c1_z : m.c0_z;
                    if (slot_empty(gx[0], gx[1]))
                        continue;
                    lo[0] = std::min(lo[0], gx[0]);
                    hi[0] = std::max(hi[0], gx[1]);
                    lo[1] = std::min(lo[1], gy[0]);
                    hi[1] = std::max(hi[1], gy[1]);
                    lo[2] = std::min(lo[2], gz[0]);
                    hi[2] = std::max(hi[2], gz[1]);
                }
            }
            x[0] = lo[0];
            x[1] = hi[0];
            y[0] = lo[1];
            y[1] = hi[1];
            z[0] = lo[2];
            z[1] = hi[2];
        }
    }
    for (const uint32_t i : order4) {
        igxrt_bvh4_node& nd = b.nodes4[i];
        for (int c = 0; c < 4; ++c) {
            if (slot_empty(nd.lo_x[c], nd.hi_x[c]))
                continue;
            float lo[3], hi[3];
            if (nd.child[c] < 0) {
                padded(leaf_box(nd.child[c]), lo, hi);
            } else {
                const igxrt_bvh4_node& m = b.nodes4[nd.child[c]];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = kInf;
                    hi[k] = -kInf;
                }
                for (int g = 0; g < 4; ++g) {
                    if (slot_empty(m.lo_x[g], m.hi_x[g]))
                        continue;
                    lo[0] = std::min(lo[0], m.lo_x[g]);
                    hi[0] = std::max(hi[0], m.hi_x[g]);
                    lo[1] = std::min(lo[1], m.lo_y[g]);
                    hi[1] = std::max(hi[1], m.hi_y[g]);
                    lo[2] = std::min(lo[2], m.lo_z[g]);
                    hi[2] = std::max(hi[2], m.hi_z[g]);
                }
            }
            nd.lo_x[c] = lo[0];
            nd.hi_x[c] = hi[0];
            nd.lo_y[c] = lo[1];
            nd.hi_y[c] = hi[1];
            nd.lo_z[c] = lo[2];
            nd.hi_z[c] = hi[2];
        }
    }
    // BVH8: re-quantized from the refit BVH2 boxes of its slots
    for (size_t i = 0; i < b.nodes8.size(); ++i)
        bvh8_quantize_node(b.nodes2.data(), &b.src8[8 * i], b.nodes8[i]);
    Aabb scene;
    scene.reset();
    for (const Aabb& a : bounds)
        scene.grow(a);
    b.info.pad_abs = pad;
    for (int a = 0; a < 3; ++a) {
        b.info.bounds[a] = n ? scene.lo[a] : 0.f;
        b.info.bounds[3 + a] = n ? scene.hi[a] : 0.f;
    }
    return IGXRT_OK;
}

// ------------------------------------------------------------------------
// Validation
// ------------------------------------------------------------------------

namespace {

bool box_empty(float lo, float hi) { return slot_empty(lo, hi); }

struct Checker {
    const igxrt_bvh& b;
    std::string& msg;
    std::vector<uint8_t> rec_seen, tri_seen, node_seen;

    bool fail(const std::string& m) {
        msg = m;
        return false;
    }

    bool inside(const float* p, const float lo[3], const float hi[3]) const {
        for (int a = 0; a < 3; ++a)
            if (!(p[a] >= lo[a] && p[a] <= hi[a]))
                return false;
        return true;
    }

    bool leaf(int32_t ref, const float lo[3], const float hi[3]) {
        uint64_t i = (uint32_t)~ref;
        for (uint32_t k = 0;; ++k, ++i) {
            if (i >= b.prims.size())
                return fail(format("leaf record %llu out of range", (unsigned long long)i));
            if (k >= 16)
                return fail("leaf longer than 16 records");
            if (rec_seen[i])
                return fail(format("primitive record %llu reached twice", (unsigned long long)i));
            rec_seen[i] = 1;
            const igxrt_prim_record& r = b.prims[i];
            const size_t nt = b.tris.size(), ns = b.spheres.size() / 4, nc = b.cubes.size();
            if (r.prim >= nt + ns + nc)
                return fail(format("record %llu names object %u", (unsigned long long)i, r.prim));
            const uint32_t want = r.prim < nt ? kPrimTriangle : r.prim < nt + ns ? kPrimSphere : kPrimCube;
            if (r.pad != want)
                return fail(format("record %llu has type %u, object %u needs %u",
                                   (unsigned long long)i, r.pad, r.prim, want));
            if (want == kPrimTriangle) {
                const igxrt_triangle& t = b.tris[r.prim];
                for (int a = 0; a < 3; ++a) {
                    const float e1 = t.p1[a] - t.p0[a], e2 = t.p2[a] - t.p0[a];
                    if (memcmp(&r.p0[a], &t.p0[a], 4) || memcmp(&r.e1[a], &e1, 4) ||
                        memcmp(&r.e2[a], &e2, 4))
                        return fail(format("record %llu does not match triangle %u",
                                           (unsigned long long)i, r.prim));
                }
                if (!inside(t.p0, lo, hi) || !inside(t.p1, lo, hi) || !inside(t.p2, lo, hi))
                    return fail(format("triangle %u outside its leaf box", r.prim));
            } else if (want == kPrimSphere) {
                const float* s = &b.spheres[4 * (r.prim - nt)];
                if (memcmp(r.p0, s, 12) || memcmp(&r.e1[0], &s[3], 4))
                    return fail(format("record %llu does not match sphere %u", (unsigned long long)i, r.prim));
                const float rad = std::fabs(s[3]);
                const float c0[3] = {s[0] - rad, s[1] - rad, s[2] - rad};
                const float c1[3] = {s[0] + rad, s[1] + rad, s[2] + rad};
                if (!inside(c0, lo, hi) || !inside(c1, lo, hi))
                    return fail(format("sphere %u outside its leaf box", r.prim));
            } else {
                const igxrt_cube& c = b.cubes[r.prim - nt - ns];
                const float start[3] = {c.xy0[0], c.xy0[1], c.z0_x1[0]};
                const float end[3] = {c.z0_x1[1], c.yz1[0], c.yz1[1]};
                if (memcmp(r.p0, start, 12) || memcmp(r.e1, end, 12))
                    return fail(format("record %llu does not match cube %u", (unsigned long long)i, r.prim));
                if (!inside(start, lo, hi) || !inside(end, lo, hi))
                    return fail(format("cube %u outside its leaf box", r.prim));
            }
            if (r.leaf_end)
                break;
        }
        return true;
    }

    // BVH8: every slot's decoded box (as the kernels decode it) must hold the
    // bounds of everything below it; `content` returns those bounds.
    bool node8(const igxrt_scene_desc& d, int32_t node, uint32_t depth, Aabb& content) {
        if (node < 0 || (size_t)node >= b.nodes8.size())
            return fail(format("BVH8 node index %d out of range", node));
        if (node_seen[node])
            return fail(format("BVH8 node %d reached twice", node));
        node_seen[node] = 1;
        if (depth > kMaxDepth)
            return fail(format("BVH8 depth %u exceeds %u", depth, kMaxDepth));
        const igxrt_bvh8_node& n = b.nodes8[node];
        if (!n.valid)
            return fail(format("BVH8 node %d has no slot", node));
        const uint8_t* q[3][2] = {{n.lo_x, n.hi_x}, {n.lo_y, n.hi_y}, {n.lo_z, n.hi_z}};
        for (int a = 0; a < 3; ++a)
            if (n.exp[a] < -126 || !std::isfinite(n.origin[a]))
                return fail(format("BVH8 node %d has a bad grid", node));
        content.reset();
        for (int c = 0; c < 8; ++c) {
            if (!(n.valid >> c & 1))
                continue;
            if (b.src8[8 * (size_t)node + c] >= 2 * b.nodes2.size())
                return fail(format("BVH8 node %d slot %d has no BVH2 source", node, c));
            float lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
                const float s = ldexpf(1.f, n.exp[a]);
                lo[a] = fmaf((float)q[a][0][c], s, n.origin[a]);
                hi[a] = fmaf((float)q[a][1][c], s, n.origin[a]);
            }
            Aabb sub;
            sub.reset();
            if (n.child[c] < 0) {
                if (!leaf(n.child[c], lo, hi))
                    return false;
                for (uint32_t i = (uint32_t)~n.child[c];; ++i) {
                    bool finite;
                    float unused = 0.f;
                    sub.grow(object_bounds(d, b.prims[i].prim, finite, unused));
                    if (b.prims[i].leaf_end)
                        break;
                }
            } else {
                if (!node8(d, n.child[c], depth + 1, sub))
                    return false;
                for (int a = 0; a < 3; ++a)
                    if (!(sub.lo[a] >= lo[a] && sub.hi[a] <= hi[a]))
                        return fail(format("BVH8 node %d slot %d does not hold its subtree", node, c));
            }
            content.grow(sub);
        }
        return true;
    }
};

}  // namespace

igxrt_status validate_bvh(const igxrt_bvh& b, std::string& msg) {
    // objects in the tree: triangles, spheres, cubes (planes stay outside)
    if (b.spheres.size() % 4 || b.planes.size() % 4) {
        msg = "sphere or plane buffer is not a whole number of vec4s";
        return IGXRT_ERROR_INVALID_BVH;
    }
    const size_t nt = b.tris.size() + b.spheres.size() / 4 + b.cubes.size();
    if (b.prims.size() != nt) {
        msg = format("%zu primitive records for %zu objects", b.prims.size(), nt);
        return IGXRT_ERROR_INVALID_BVH;
    }
    if (nt == 0) {
        if (!b.nodes2.empty() || !b.nodes4.empty()) {
            msg = "empty scene with nodes";
            return IGXRT_ERROR_INVALID_BVH;
        }
        return IGXRT_OK;
    }
    if (b.nodes2.empty() || b.nodes4.empty()) {
        msg = "non-empty scene without nodes";
        return IGXRT_ERROR_INVALID_BVH;
    }
    for (uint32_t l = 0; l < IGXRT_LAYOUT_COUNT; ++l)
        if (b.info.max_stack[l] > kStackCapacity) {
            msg = format("layout %u needs a %u-entry stack (limit %u)", l, b.info.max_stack[l],
                         kStackCapacity);
            return IGXRT_ERROR_INVALID_BVH;
        }
    for (int layout = 0; layout < 2; ++layout) {
        Checker ck{b, msg, std::vector<uint8_t>(nt, 0), std::vector<uint8_t>(nt, 0), {}};
        const size_t nn = layout == 0 ? b.nodes2.size() : b.nodes4.size();
        ck.node_seen.assign(nn, 0);
        struct Item {
            int32_t node;
            uint32_t depth;
        };
        std::vector<Item> stack = {{0, 1}};
        while (!stack.empty()) {
            const Item it = stack.back();
            stack.pop_back();
            if (it.node < 0 || (size_t)it.node >= nn) {
                msg = format("node index %d out of range", it.node);
                return IGXRT_ERROR_INVALID_BVH;
            }
            if (ck.node_seen[it.node]) {
                msg = format("node %d reached twice", it.node);
                return IGXRT_ERROR_INVALID_BVH;
            }
            ck.node_seen[it.node] = 1;
            if (it.depth > kMaxDepth) {
                msg = format("depth %u exceeds %u", it.depth, kMaxDepth);
                return IGXRT_ERROR_INVALID_BVH;
            }
            const int slots = layout == 0 ? 2 : 4;
            for (int c = 0; c < slots; ++c) {
                float lo[3], hi[3];
                int32_t ref;
                if (layout == 0) {
                    const igxrt_bvh2_node& n = b.nodes2[it.node];
                    const float* x = c ? n.c1_x : n.c0_x;
                    const float* y = c ? n.c1_y : n.c0_y;
                    const float* z = c ? n.c1_z : n.c0_z;
                    lo[0] = x[0]; hi[0] = x[1];
                    lo[1] = y[0]; hi[1] = y[1];
                    lo[2] = z[0]; hi[2] = z[1];
                    ref = n.child[c];
                } else {
                    const igxrt_bvh4_node& n = b.nodes4[it.node];
                    lo[0] = n.lo_x[c]; hi[0] = n.hi_x[c];
                    lo[1] = n.lo_y[c]; hi[1] = n.hi_y[c];
                    lo[2] = n.lo_z[c]; hi[2] = n.hi_z[c];
                    ref = n.child[c];
                }
                if (box_empty(lo[0], hi[0]) && box_empty(lo[1], hi[1]) && box_empty(lo[2], hi[2]))
                    continue;
                if (ref < 0) {
                    if (!ck.leaf(ref, lo, hi))
                        return IGXRT_ERROR_INVALID_BVH;
                } else {
                    // Interior child: its own child boxes must lie inside this box.
                    if ((size_t)ref >= nn) {
                        msg = format("child index %d out of range", ref);
                        return IGXRT_ERROR_INVALID_BVH;
                    }
                    const int sub = layout == 0 ? 2 : 4;
                    for (int g = 0; g < sub; ++g) {
                        float glo[3], ghi[3];
                        if (layout == 0) {
                            const igxrt_bvh2_node& m = b.nodes2[ref];
                            const float* x = g ? m.c1_x : m.c0_x;
                            const float* y = g ? m.c1_y : m.c0_y;
                            const float* z = g ? m.c1_z : m.c0_z;
                            glo[0] = x[0]; ghi[0] = x[1];
                            glo[1] = y[0]; ghi[1] = y[1];
                            glo[2] = z[0]; ghi[2] = z[1];
                        } else {
                            const igxrt_bvh4_node& m = b.nodes4[ref];
                            glo[0] = m.lo_x[g]; ghi[0] = m.hi_x[g];
                            glo[1] = m.lo_y[g]; ghi[1] = m.hi_y[g];
                            glo[2] = m.lo_z[g]; ghi[2] = m.hi_z[g];
                        }
                        if (box_empty(glo[0], ghi[0]))
                            continue;
                        for (int a = 0; a < 3; ++a)
                            if (!(glo[a] >= lo[a] && ghi[a] <= hi[a])) {
                                msg = format("node %d child box escapes its parent box", ref);
                                return IGXRT_ERROR_INVALID_BVH;
                            }
                    }
                    stack.push_back({ref, it.depth + 1});
                }
            }
        }
        for (size_t i = 0; i < nn; ++i)
            if (!ck.node_seen[i]) {
                msg = format("node %zu unreachable", i);
                return IGXRT_ERROR_INVALID_BVH;
            }
        for (size_t i = 0; i < nt; ++i) {
            if (!ck.rec_seen[i]) {
                msg = format("primitive record %zu unreachable", i);
                return IGXRT_ERROR_INVALID_BVH;
            }
        }
        std::vector<uint8_t> tri_seen(nt, 0);
        for (const auto& r : b.prims) {
            if (tri_seen[r.prim]) {
                msg = format("triangle %u in two leaves", r.prim);
                return IGXRT_ERROR_INVALID_BVH;
            }
            tri_seen[r.prim] = 1;
        }
    }
    // BVH8 (optional: GPU builds and very deep trees have none)
    if (b.info.bvh8_nodes != b.nodes8.size() || b.src8.size() != 8 * b.nodes8.size()) {
        msg = "BVH8 arrays and info disagree";
        return IGXRT_ERROR_INVALID_BVH;
    }
    if (!b.nodes8.empty()) {
        Checker ck{b, msg, std::vector<uint8_t>(nt, 0), {}, std::vector<uint8_t>(b.nodes8.size(), 0)};
        igxrt_scene_desc d{};
        d.triangles = b.tris.data();
        d.triangle_count = (uint32_t)b.tris.size();
        d.spheres = b.spheres.data();
        d.sphere_count = (uint32_t)(b.spheres.size() / 4);
        d.cubes = b.cubes.data();
        d.cube_count = (uint32_t)b.cubes.size();
        Aabb all;
        if (!ck.node8(d, 0, 1, all))
            return IGXRT_ERROR_INVALID_BVH;
        for (size_t i = 0; i < b.nodes8.size(); ++i)
            if (!ck.node_seen[i]) {
                msg = format("BVH8 node %zu unreachable", i);
                return IGXRT_ERROR_INVALID_BVH;
            }
        for (size_t i = 0; i < nt; ++i)
            if (!ck.rec_seen[i]) {
                msg = format("primitive record %zu unreachable in BVH8", i);
                return IGXRT_ERROR_INVALID_BVH;
            }
    }
    return IGXRT_OK;
}

}  // namespace igxrt

// ------------------------------------------------------------------------
// C ABI: host BVH objects
// ------------------------------------------------------------------------

using namespace igxrt;

namespace {

struct FileHeader {
    char magic[8];
    uint32_t version;
    uint32_t abi;
    uint64_t tris, nodes2, nodes4, prims;
    uint64_t spheres, cubes, planes;
    uint64_t nodes8;  // followed by 8 BVH2 sources per BVH8 node
    igxrt_bvh_info info;
};
constexpr uint32_t kFileVersion = 3;

constexpr char kMagic[8] = {'I', 'G', 'X', 'R', 'T', 'B', 'V', 'H'};

}  // namespace

extern "C" {

igxrt_status igxrt_bvh_build(const igxrt_triangle* tris, uint32_t count,
                             const igxrt_build_options* opts, igxrt_bvh** out) {
    if (!out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_bvh* b = new (std::nothrow) igxrt_bvh();
    if (!b)
        return IGXRT_ERROR_OUT_OF_MEMORY;
    std::string err;
    igxrt_status st;
    try {
        st = build_bvh(tris, count, opts, *b, err);
    } catch (const std::bad_alloc&) {
        st = IGXRT_ERROR_OUT_OF_MEMORY;
    }
    if (st != IGXRT_OK) {
        delete b;
        return st;
    }
    *out = b;
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_build_mixed(const igxrt_scene_desc* desc, const igxrt_build_options* opts,
                                   igxrt_bvh** out) {
    if (!out || !desc)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    igxrt_bvh* b = new (std::nothrow) igxrt_bvh();
    if (!b)
        return IGXRT_ERROR_OUT_OF_MEMORY;
    std::string err;
    igxrt_status st;
    try {
        st = build_bvh_mixed(*desc, opts, *b, err);
    } catch (const std::bad_alloc&) {
        st = IGXRT_ERROR_OUT_OF_MEMORY;
    }
    if (st != IGXRT_OK) {
        delete b;
        return st;
    }
    *out = b;
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_destroy(igxrt_bvh* bvh) {
    delete bvh;
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_refit(igxrt_bvh* bvh, const igxrt_scene_desc* desc) {
    if (!bvh || !desc)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::string err;
    try {
        igxrt_bvh next = *bvh;  // all or nothing: a rejected description changes nothing
        const igxrt_status st = refit_bvh(next, *desc, err);
        if (st != IGXRT_OK)
            return st;
        *bvh = std::move(next);
    } catch (const std::bad_alloc&) {
        return IGXRT_ERROR_OUT_OF_MEMORY;
    }
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_get_info(const igxrt_bvh* bvh, igxrt_bvh_info* info) {
    if (!bvh || !info)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *info = bvh->info;
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_get_data(const igxrt_bvh* bvh, uint32_t layout, const void** nodes,
                                uint64_t* node_count, const igxrt_prim_record** prims,
                                uint64_t* prim_count) {
    if (!bvh || layout >= IGXRT_LAYOUT_COUNT)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    if (nodes)
        *nodes = layout == IGXRT_LAYOUT_BVH2   ? (const void*)bvh->nodes2.data()
                 : layout == IGXRT_LAYOUT_BVH4 ? (const void*)bvh->nodes4.data()
                                               : (const void*)bvh->nodes8.data();
    if (node_count)
        *node_count = layout == IGXRT_LAYOUT_BVH2   ? bvh->nodes2.size()
                      : layout == IGXRT_LAYOUT_BVH4 ? bvh->nodes4.size()
                                                    : bvh->nodes8.size();
    if (prims)
        *prims = bvh->prims.data();
    if (prim_count)
        *prim_count = bvh->prims.size();
    return IGXRT_OK;
}

igxrt_status igxrt_bvh_validate(const igxrt_bvh* bvh, char* msg, size_t msg_len) {
    if (!bvh)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    std::string m;
    const igxrt_status st = validate_bvh(*bvh, m);
    if (msg && msg_len) {
        snprintf(msg, msg_len, "%s", st == IGXRT_OK ? "ok" : m.c_str());
    }
    return st;
}

igxrt_status igxrt_bvh_save(const igxrt_bvh* bvh, const char* path) {
    if (!bvh || !path)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "wb");
    if (!f)
        return IGXRT_ERROR_IO;
    FileHeader h{};
    memcpy(h.magic, kMagic, 8);
    h.version = kFileVersion;
    h.abi = IGXRT_ABI_VERSION;
    h.tris = bvh->tris.size();
    h.nodes2 = bvh->nodes2.size();
    h.nodes4 = bvh->nodes4.size();
    h.prims = bvh->prims.size();
    h.spheres = bvh->spheres.size() / 4;
    h.cubes = bvh->cubes.size();
    h.planes = bvh->planes.size() / 4;
    h.nodes8 = bvh->nodes8.size();
    h.info = bvh->info;
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    ok = ok && fwrite(bvh->tris.data(), sizeof(igxrt_triangle), h.tris, f) == h.tris;
    ok = ok && fwrite(bvh->nodes2.data(), sizeof(igxrt_bvh2_node), h.nodes2, f) == h.nodes2;
    ok = ok && fwrite(bvh->nodes4.data(), sizeof(igxrt_bvh4_node), h.nodes4, f) == h.nodes4;
    ok = ok && fwrite(bvh->prims.data(), sizeof(igxrt_prim_record), h.prims, f) == h.prims;
    ok = ok && fwrite(bvh->spheres.data(), 16, h.spheres, f) == h.spheres;
    ok = ok && fwrite(bvh->cubes.data(), sizeof(igxrt_cube), h.cubes, f) == h.cubes;
    ok = ok && fwrite(bvh->planes.data(), 16, h.planes, f) == h.planes;
    ok = ok && fwrite(bvh->nodes8.data(), sizeof(igxrt_bvh8_node), h.nodes8, f) == h.nodes8;
    ok = ok && fwrite(bvh->src8.data(), 32, h.nodes8, f) == h.nodes8;
    ok = (fclose(f) == 0) && ok;
    return ok ? IGXRT_OK : IGXRT_ERROR_IO;
}

igxrt_status igxrt_bvh_load(const char* path, igxrt_bvh** out) {
    if (!path || !out)
        return IGXRT_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = fopen(path, "rb");
    if (!f)
        return IGXRT_ERROR_IO;
    FileHeader h{};
    igxrt_bvh* b = nullptr;
    igxrt_status st = IGXRT_ERROR_IO;
    do {
        if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, kMagic, 8) || h.version != kFileVersion)
            break;
        const uint64_t objects = h.tris + h.spheres + h.cubes;
        if (h.tris >= 0x7fffffffu || h.spheres >= 0x7fffffffu || h.cubes >= 0x7fffffffu ||
            h.planes >= 0x7fffffffu || objects + h.planes >= 0x7fffffffu || h.prims != objects ||
            h.nodes2 > 2 * objects + 1 || h.nodes4 > 2 * objects + 1 || h.nodes8 > 2 * objects + 1)
            break;
        b = new (std::nothrow) igxrt_bvh();
        if (!b) {
            st = IGXRT_ERROR_OUT_OF_MEMORY;
            break;
        }
        b->tris.resize(h.tris);
        b->nodes2.resize(h.nodes2);
        b->nodes4.resize(h.nodes4);
        b->prims.resize(h.prims);
        b->spheres.resize(4 * h.spheres);
        b->cubes.resize(h.cubes);
        b->planes.resize(4 * h.planes);
        b->nodes8.resize(h.nodes8);
        b->src8.resize(8 * h.nodes8);
        if (fread(b->tris.data(), sizeof(igxrt_triangle), h.tris, f) != h.tris ||
            fread(b->nodes2.data(), sizeof(igxrt_bvh2_node), h.nodes2, f) != h.nodes2 ||
            fread(b->nodes4.data(), sizeof(igxrt_bvh4_node), h.nodes4, f) != h.nodes4 ||
            fread(b->prims.data(), sizeof(igxrt_prim_record), h.prims, f) != h.prims ||
            fread(b->spheres.data(), 16, h.spheres, f) != h.spheres ||
            fread(b->cubes.data(), sizeof(igxrt_cube), h.cubes, f) != h.cubes ||
            fread(b->planes.data(), 16, h.planes, f) != h.planes ||
            fread(b->nodes8.data(), sizeof(igxrt_bvh8_node), h.nodes8, f) != h.nodes8 ||
            fread(b->src8.data(), 32, h.nodes8, f) != h.nodes8)
            break;
        b->info = h.info;
        std::string m;
        st = validate_bvh(*b, m);
    } while (false);
    fclose(f);
    if (st != IGXRT_OK) {
        delete b;
        return st;
    }
    *out = b;
    return IGXRT_OK;
}

}  // extern "C"
