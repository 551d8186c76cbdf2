"""Refit of moved geometry: igxrt_bvh_refit on the host, igxrt_scene_refit on
the GPU.

The reference re-uploads moving spheres every frame and traces them with its
linear loop (test/scene/niels_scene.cpp:61-70, res/shaders/trace.glsl:22-46);
with a BVH the boxes must follow the geometry.  Checks:
  * refit with unchanged geometry reproduces the build bit for bit;
  * refit boxes equal a numpy restatement of the builder's rule (object bounds,
    leaf union padded by max(2^-18 * max|coordinate|, 1e-30), interior union);
  * traversal of a refit tree equals the brute-force oracle on the moved
    geometry;
  * the GPU refit equals the host refit bit for bit (nodes of every layout,
    records), through host staging and through CUDA tensors.
"""
import math

import numpy as np
import pytest

from conftest import NO_HIT, assert_hits_equal, bits
from igx_raytracing_gb300 import BVH, IgxrtError, scenes
from igx_raytracing_gb300._capi import CUBE_DTYPE, LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8, TRIANGLE_DTYPE
from oracle import pyoracle


def moved_triangles(tris, frame):
    """A smooth displacement (keeps the tree sensible, changes every box)."""
    out = tris.copy()
    for f in ("p0", "p1", "p2"):
        p = out[f].astype(np.float64)
        d = np.stack([np.sin(3.1 * p[:, 1] + frame), np.cos(2.3 * p[:, 2] - frame),
                      np.sin(1.7 * p[:, 0] + 0.5 * frame)], 1)
        out[f] = (p + 0.03 * d + 0.01 * frame).astype(np.float32)
    return out


def moved_mixed(sc, frame):
    rng = np.random.default_rng(100 + frame)
    out = dict(sc)
    out["tris"] = moved_triangles(sc["tris"], frame)
    s = sc["spheres"].copy()
    s[:, :3] += rng.uniform(-0.02, 0.02, (len(s), 3)).astype(np.float32)
    s[:, 3] *= rng.uniform(0.8, 1.2, len(s)).astype(np.float32)
    out["spheres"] = s
    c = sc["cubes"].copy()
    shift = rng.uniform(-0.02, 0.02, (len(c), 3)).astype(np.float32)
    c["xy0"] += shift[:, :2]
    c["z0_x1"][:, 0] += shift[:, 2]
    c["z0_x1"][:, 1] += shift[:, 0]
    c["yz1"] += shift[:, 1:]
    out["cubes"] = c
    out["planes"] = sc["planes"] * np.float32(1.01)
    return out


def random_mixed(seed, nt=2000, ns=300, nc=200, npl=2):
    rng = np.random.default_rng(seed)
    tris = scenes.random_triangles(nt, 6100 + seed, mu=math.log(0.05))
    spheres = np.concatenate([rng.uniform(0, 1, (ns, 3)), rng.uniform(0.005, 0.05, (ns, 1))], 1)
    lo = rng.uniform(0, 1, (nc, 3))
    hi = lo + rng.uniform(0.01, 0.08, (nc, 3))
    cubes = np.zeros(nc, CUBE_DTYPE)
    cubes["xy0"] = lo[:, :2]
    cubes["z0_x1"] = np.stack([lo[:, 2], hi[:, 0]], 1)
    cubes["yz1"] = hi[:, 1:]
    planes = np.concatenate([rng.normal(size=(npl, 3)), rng.uniform(-2.5, -1.5, (npl, 1))], 1)
    return dict(tris=tris, spheres=spheres.astype(np.float32), cubes=cubes,
                planes=planes.astype(np.float32))


# --- numpy restatement of the builder's box rule ---------------------------

def object_bounds(tris=None, spheres=None, cubes=None):
    lo, hi = [], []
    if tris is not None and len(tris):
        v = np.stack([tris["p0"], tris["p1"], tris["p2"]], 1)
        lo.append(v.min(1))
        hi.append(v.max(1))
    if spheres is not None and len(spheres):
        r = np.abs(spheres[:, 3:4])
        lo.append(spheres[:, :3] - r)
        hi.append(spheres[:, :3] + r)
    if cubes is not None and len(cubes):
        start = np.stack([cubes["xy0"][:, 0], cubes["xy0"][:, 1], cubes["z0_x1"][:, 0]], 1)
        end = np.stack([cubes["z0_x1"][:, 1], cubes["yz1"][:, 0], cubes["yz1"][:, 1]], 1)
        lo.append(np.minimum(start, end))
        hi.append(np.maximum(start, end))
    return np.concatenate(lo).astype(np.float32), np.concatenate(hi).astype(np.float32)


def expected_boxes(layout, nodes, prims, lo, hi):
    """Slot boxes of every node, children before parents (preorder layout)."""
    pad = np.float32(max(np.float32(max(np.abs(lo).max(), np.abs(hi).max()) * np.float32(2.0 ** -18)),
                         np.float32(1e-30)))
    slots = 2 if layout == LAYOUT_BVH2 else 4
    out = np.zeros((len(nodes), slots, 2, 3), np.float32)  # [node, slot, lo/hi, axis]

    def slot_box(node, c):
        if layout == LAYOUT_BVH2:
            k = "c0" if c == 0 else "c1"
            return np.array([[node[k + "_x"][0], node[k + "_y"][0], node[k + "_z"][0]],
                             [node[k + "_x"][1], node[k + "_y"][1], node[k + "_z"][1]]], np.float32)
        return np.array([[node["lo_x"][c], node["lo_y"][c], node["lo_z"][c]],
                         [node["hi_x"][c], node["hi_y"][c], node["hi_z"][c]]], np.float32)

    empty = np.zeros((len(nodes), slots), bool)
    for i in range(len(nodes)):
        for c in range(slots):
            b = slot_box(nodes[i], c)
            empty[i, c] = b[0, 0] == np.inf and b[1, 0] == np.inf
    for i in range(len(nodes) - 1, -1, -1):
        for c in range(slots):
            if empty[i, c]:
                out[i, c] = np.inf
                continue
            ref = int(nodes[i]["child"][c])
            if ref < 0:
                first = ~ref
                last = first
                while not prims["leaf_end"][last]:
                    last += 1
                ids = prims["prim"][first:last + 1]
                out[i, c, 0] = lo[ids].min(0) - pad
                out[i, c, 1] = hi[ids].max(0) + pad
            else:
                used = ~empty[ref]
                out[i, c, 0] = out[ref, used, 0].min(0)
                out[i, c, 1] = out[ref, used, 1].max(0)
    return out, pad


def boxes_of(layout, nodes):
    if layout == LAYOUT_BVH2:
        b = np.zeros((len(nodes), 2, 2, 3), np.float32)
        for c, k in enumerate(("c0", "c1")):
            for a, ax in enumerate("xyz"):
                b[:, c, 0, a] = nodes[f"{k}_{ax}"][:, 0]
                b[:, c, 1, a] = nodes[f"{k}_{ax}"][:, 1]
        return b
    b = np.zeros((len(nodes), 4, 2, 3), np.float32)
    for a, ax in enumerate("xyz"):
        b[:, :, 0, a] = nodes[f"lo_{ax}"]
        b[:, :, 1, a] = nodes[f"hi_{ax}"]
    return b


def assert_same_arrays(a, b):
    assert a.dtype == b.dtype and a.shape == b.shape
    assert a.tobytes() == b.tobytes()


def assert_bvh_equal(x: BVH, y: BVH):
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8):
        nx, px = x.arrays(layout)
        ny, py = y.arrays(layout)
        assert_same_arrays(nx, ny)
        assert_same_arrays(px, py)


# --- host refit --------------------------------------------------------------

@pytest.mark.parametrize("kind", ["heightfield", "random", "mixed"])
def test_refit_unchanged_geometry_reproduces_build(kind):
    if kind == "mixed":
        sc = random_mixed(1)
        b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        c = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        c.refit(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    else:
        tris = (scenes.heightfield(40, 30, seed=3) if kind == "heightfield"
                else scenes.random_triangles(5000, 17, mu=math.log(0.03)))
        b = BVH.build(tris)
        c = BVH.build(tris)
        c.refit(tris)
    assert_bvh_equal(b, c)
    assert b.info == c.info


@pytest.mark.parametrize("layout", [LAYOUT_BVH2, LAYOUT_BVH4])
def test_refit_boxes_follow_the_builder_rule(layout):
    tris = scenes.random_triangles(3000, 23, mu=math.log(0.04))
    b = BVH.build(tris)
    moved = moved_triangles(tris, 1.0)
    b.refit(moved)
    b.validate()
    nodes, prims = b.arrays(layout)
    lo, hi = object_bounds(moved)
    want, pad = expected_boxes(layout, nodes, prims, lo, hi)
    assert bits(np.float32(b.info["pad_abs"])) == bits(pad)
    assert np.array_equal(bits(boxes_of(layout, nodes)), bits(want))
    tri = moved[prims["prim"]]
    assert np.array_equal(bits(prims["p0"]), bits(tri["p0"]))
    assert np.array_equal(bits(prims["e1"]), bits(tri["p1"] - tri["p0"]))
    assert np.array_equal(bits(prims["e2"]), bits(tri["p2"] - tri["p0"]))
    assert np.allclose(b.info["bounds"], np.concatenate([lo.min(0), hi.max(0)]))


def test_refit_mixed_boxes_follow_the_builder_rule():
    sc = random_mixed(2)
    b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    mv = moved_mixed(sc, 1)
    b.refit(mv["tris"], mv["spheres"], mv["cubes"], mv["planes"])
    b.validate()
    lo, hi = object_bounds(mv["tris"], mv["spheres"], mv["cubes"])
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4):
        nodes, prims = b.arrays(layout)
        want, _ = expected_boxes(layout, nodes, prims, lo, hi)
        assert np.array_equal(bits(boxes_of(layout, nodes)), bits(want))
    sph = prims["pad"] == 1
    ids = prims["prim"][sph] - len(mv["tris"])
    assert np.array_equal(bits(prims["p0"][sph]), bits(mv["spheres"][ids, :3]))
    assert np.array_equal(bits(prims["e1"][sph][:, 0]), bits(mv["spheres"][ids, 3]))


def test_refit_traversal_matches_brute_force():
    tris = scenes.random_triangles(4000, 29, mu=math.log(0.04))
    b = BVH.build(tris)
    rays = scenes.incoherent_rays(3000, 31, tmax=float(NO_HIT))
    for frame in (0.5, 2.0):
        moved = moved_triangles(tris, frame)
        b.refit(moved)
        expect, flags = pyoracle.trace_geometry(moved, rays)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        for layout in (LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8):
            nodes, prims = b.arrays(layout)
            got = pyoracle.bvh_trace(layout, nodes, prims, rays)
            assert_hits_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok],
                              expect["v"][ok], f"frame {frame} layout {layout}")


def test_refit_rejects_bad_input_and_keeps_the_tree():
    tris = scenes.random_triangles(500, 37)
    b = BVH.build(tris)
    ref = BVH.build(tris)
    with pytest.raises(IgxrtError):
        b.refit(tris[:-1])  # another primitive count
    bad = tris.copy()
    bad["p1"][7, 2] = np.nan
    with pytest.raises(IgxrtError):
        b.refit(bad)
    bad = tris.copy()
    bad["p2"][3, 0] = np.inf
    with pytest.raises(IgxrtError):
        b.refit(bad)
    assert_bvh_equal(b, ref)


@pytest.mark.parametrize("what", ["sphere_centre", "sphere_radius", "cube", "plane"])
def test_refit_rejects_non_finite_mixed(what):
    sc = random_mixed(3, nt=200, ns=50, nc=40)
    b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    ref = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    mv = moved_mixed(sc, 1)
    if what == "sphere_centre":
        mv["spheres"][4, 1] = np.nan
    elif what == "sphere_radius":
        mv["spheres"][9, 3] = np.inf
    elif what == "cube":  # one NaN corner coordinate leaves the min/max finite
        mv["cubes"]["z0_x1"][5, 1] = np.nan
    else:
        mv["planes"][1, 3] = np.nan
    with pytest.raises(IgxrtError):
        b.refit(mv["tris"], mv["spheres"], mv["cubes"], mv["planes"])
    assert_bvh_equal(b, ref)


# --- GPU refit ---------------------------------------------------------------

def triangle_tensor(tris):
    import torch

    return torch.from_numpy(np.ascontiguousarray(tris).view(np.float32).reshape(-1, 12).copy()).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [LAYOUT_BVH2, LAYOUT_BVH4])
def test_scene_read_bvh_equals_upload(ctx, layout):
    tris = scenes.random_triangles(2000, 41)
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    n, p = scene.read_bvh(layout)
    bn, bp = b.arrays(layout)
    assert_same_arrays(n, bn)
    assert_same_arrays(p, bp)


@pytest.mark.gpu
@pytest.mark.parametrize("device_buffers", [False, True])
@pytest.mark.parametrize("n", [1, 7, 3000, 200000])
def test_gpu_refit_equals_host_refit(ctx, n, device_buffers):
    tris = scenes.random_triangles(n, 43 + n, mu=math.log(0.02))
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    for frame in (1.0, 2.5):  # twice: the arrival counters are reset per refit
        moved = moved_triangles(tris, frame)
        b.refit(moved)
        scene.refit(triangle_tensor(moved) if device_buffers else moved)
        assert_bvh_arrays_equal(scene, b)
        assert bits(np.float32(scene.info["pad_abs"])) == bits(np.float32(b.info["pad_abs"]))
        assert np.array_equal(np.float32(scene.info["bounds"]), np.float32(b.info["bounds"]))


def assert_bvh_arrays_equal(scene, b):
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8):
        sn, sp = scene.read_bvh(layout)
        bn, bp = b.arrays(layout)
        assert_same_arrays(sn, bn)
        assert_same_arrays(sp, bp)


@pytest.mark.gpu
def test_gpu_refit_traces_match_oracle(ctx):
    tris = scenes.random_triangles(20000, 47, mu=math.log(0.02))
    scene = ctx.create_scene(tris)
    rays = scenes.incoherent_rays(20000, 53, tmax=float(NO_HIT))
    saved = ctx.launch_params
    for frame in (0.5, 1.5, 3.0):
        moved = moved_triangles(tris, frame)
        scene.refit(moved)
        expect, flags = pyoracle.trace_geometry(moved, rays)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        sh = rays.copy()
        sh["tmax"] = np.float32(0.3)
        occ, oflags = pyoracle.trace_occlusion(moved, sh)
        ook = (oflags & pyoracle.EVENT_NAN_T) == 0
        for layout in (LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8):
            ctx.set_launch_params(layout=layout)
            got = scene.trace_geometry(rays)
            assert_hits_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok],
                              expect["v"][ok], f"frame {frame} layout {layout}")
            assert np.array_equal(scene.trace_occlusion(sh)[ook], occ[ook])
    ctx.set_launch_params(**saved)


@pytest.mark.gpu
def test_gpu_refit_mixed(ctx):
    from test_mixed import assert_mixed_equal

    sc = random_mixed(5)
    b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    scene = ctx.create_scene(bvh=b)
    rays = scenes.incoherent_rays(6000, 59, tmax=float(NO_HIT))
    for frame in (1, 2):
        mv = moved_mixed(sc, frame)
        b.refit(mv["tris"], mv["spheres"], mv["cubes"], mv["planes"])
        if frame == 1:
            scene.refit(mv["tris"], mv["spheres"], mv["cubes"], mv["planes"])
        else:
            import torch

            scene.refit(triangle_tensor(mv["tris"]), torch.from_numpy(mv["spheres"]).cuda(),
                        torch.from_numpy(mv["cubes"].view(np.float32).reshape(-1, 6).copy()).cuda(),
                        torch.from_numpy(mv["planes"]).cuda())
        assert_bvh_arrays_equal(scene, b)
        expect, flags = pyoracle.trace_geometry_mixed(rays, None, **mv)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        got = scene.trace_geometry(rays)
        assert_mixed_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok],
                           expect["v"][ok], len(mv["tris"]), len(mv["spheres"]))


@pytest.mark.gpu
def test_gpu_refit_rejects_bad_input_and_keeps_the_scene(ctx):
    tris = scenes.random_triangles(3000, 61)
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    bad = moved_triangles(tris, 1.0)
    bad["p0"][1234, 1] = np.inf
    with pytest.raises(IgxrtError):
        scene.refit(bad)
    with pytest.raises(IgxrtError):
        scene.refit(triangle_tensor(bad))
    with pytest.raises(IgxrtError):
        scene.refit(tris[:100])
    assert_bvh_arrays_equal(scene, b)
    rays = scenes.incoherent_rays(2000, 67, tmax=float(NO_HIT))
    expect, flags = pyoracle.trace_geometry(tris, rays)
    ok = (flags & pyoracle.EVENT_NAN_T) == 0
    got = scene.trace_geometry(rays)
    assert_hits_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok], expect["v"][ok])
    assert TRIANGLE_DTYPE.itemsize == 48


@pytest.mark.gpu
@pytest.mark.parametrize("what", ["sphere_radius", "cube", "plane"])
def test_gpu_refit_rejects_non_finite_mixed(ctx, what):
    sc = random_mixed(6, nt=300, ns=60, nc=50)
    b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    scene = ctx.create_scene(bvh=b)
    mv = moved_mixed(sc, 2)
    if what == "sphere_radius":
        mv["spheres"][9, 3] = np.nan
    elif what == "cube":
        mv["cubes"]["xy0"][5, 0] = np.nan
    else:
        mv["planes"][0, 2] = np.inf
    with pytest.raises(IgxrtError):
        scene.refit(mv["tris"], mv["spheres"], mv["cubes"], mv["planes"])
    assert_bvh_arrays_equal(scene, b)
