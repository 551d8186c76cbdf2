"""GPU BVH build (igxrt_scene_create_gpu, a linear BVH) and scene download.

The reference has no acceleration structure; its result is the linear loop's
(res/shaders/trace.glsl:9-98).  A GPU-built tree has other splits than the
host SAH build but the same node formats, records and padding, so every query
must still equal the brute-force oracle bit for bit, the CPU traversal of the
downloaded tree must equal the GPU's (hits and per-ray fetch counts), and the
refit must reproduce the build when nothing moved.
"""
import math
import os

import numpy as np
import pytest

from conftest import NO_HIT, assert_hits_equal
from igx_raytracing_gb300 import BVH, IgxrtError, scenes
from igx_raytracing_gb300._capi import LAYOUT_BVH2, LAYOUT_BVH4
from oracle import pyoracle
from test_refit import moved_triangles, random_mixed, triangle_tensor

pytestmark = pytest.mark.gpu


def oracle_check(scene, tris, rays, what):
    expect, flags = pyoracle.trace_geometry(tris, rays)
    ok = (flags & pyoracle.EVENT_NAN_T) == 0
    got = scene.trace_geometry(rays)
    assert_hits_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok], expect["v"][ok], what,
                      rays=rays[ok], tris=tris)
    sh = rays.copy()
    sh["tmax"] = np.float32(0.25)
    occ, oflags = pyoracle.trace_occlusion(tris, sh)
    ook = (oflags & pyoracle.EVENT_NAN_T) == 0
    assert np.array_equal(scene.trace_occlusion(sh)[ook], occ[ook]), what


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 1000, 30000])
@pytest.mark.parametrize("leaf", [1, 2, 4])
def test_gpu_build_traces_match_oracle(ctx, n, leaf):
    tris = scenes.random_triangles(n, 70 + n, mu=math.log(0.02 if n > 100 else 0.2))
    scene = ctx.create_scene_gpu(tris, max_leaf_size=leaf)
    info = scene.info
    assert info["triangle_count"] == n and info["max_leaf_size"] == leaf
    rays = scenes.incoherent_rays(4000, 71, tmax=float(NO_HIT))
    saved = ctx.launch_params
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4):
        ctx.set_launch_params(layout=layout)
        oracle_check(scene, tris, rays, f"n {n} leaf {leaf} layout {layout}")
    ctx.set_launch_params(**saved)


def test_gpu_build_heightfield_primary_rays(ctx):
    tris = scenes.heightfield(64, 32, seed=scenes.seed_for(1))
    scene = ctx.create_scene_gpu(tris)
    rays = scenes.pinhole_rays(128, 128, eye=(0.5, -1.0, 0.5), target=(0.5, 0.5, 0.0))
    oracle_check(scene, tris, rays, "heightfield")


def test_gpu_build_download_matches_cpu_traversal(ctx, tmp_path):
    tris = scenes.random_triangles(20000, 73, mu=math.log(0.02))
    scene = ctx.create_scene_gpu(tris)
    bvh = scene.download()  # validated by the library
    bvh.validate()
    info = bvh.info
    assert info == scene.info
    assert info["max_stack"][0] <= 128 and info["max_depth"] >= 1
    rays = scenes.incoherent_rays(5000, 74, tmax=float(NO_HIT))
    saved = ctx.launch_params
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4):
        nodes, prims = bvh.arrays(layout)
        n2, p2 = scene.read_bvh(layout)
        assert nodes.tobytes() == n2.tobytes() and prims.tobytes() == p2.tobytes()
        cpu, nf, pf = pyoracle.bvh_trace(layout, nodes, prims, rays, counts=True)
        ctx.set_launch_params(layout=layout)
        got = scene.trace_geometry(rays)
        assert_hits_equal(got, cpu["prim"], cpu["t"], cpu["u"], cpu["v"], f"layout {layout}")
        gnf, gpf = ctx.count_fetches(scene, rays, layout=layout)
        assert np.array_equal(gnf, nf) and np.array_equal(gpf, pf)
    ctx.set_launch_params(**saved)
    # warm start: save, load, upload, same answers
    path = os.path.join(tmp_path, "gpu.bvh")
    bvh.save(path)
    again = ctx.create_scene(bvh=BVH.load(path))
    assert np.array_equal(again.trace_geometry(rays).view(np.uint32), scene.trace_geometry(rays).view(np.uint32))


def test_gpu_build_refit(ctx):
    tris = scenes.random_triangles(20000, 75, mu=math.log(0.02))
    scene = ctx.create_scene_gpu(tris)
    before = [scene.read_bvh(layout) for layout in (LAYOUT_BVH2, LAYOUT_BVH4)]
    scene.refit(tris)  # nothing moved: the boxes are the build's
    for layout, (nodes, prims) in zip((LAYOUT_BVH2, LAYOUT_BVH4), before):
        n, p = scene.read_bvh(layout)
        assert n.tobytes() == nodes.tobytes() and p.tobytes() == prims.tobytes()
    host = scene.download()
    moved = moved_triangles(tris, 1.5)
    host.refit(moved)  # the host refit walks a non-preorder tree too
    scene.refit(triangle_tensor(moved))
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4):
        n, p = scene.read_bvh(layout)
        hn, hp = host.arrays(layout)
        assert n.tobytes() == hn.tobytes() and p.tobytes() == hp.tobytes()
    rays = scenes.incoherent_rays(4000, 76, tmax=float(NO_HIT))
    oracle_check(scene, moved, rays, "gpu build after refit")


def test_gpu_build_device_tensors_equal_host_arrays(ctx):
    tris = scenes.random_triangles(5000, 77, mu=math.log(0.03))
    a = ctx.create_scene_gpu(tris)
    b = ctx.create_scene_gpu(triangle_tensor(tris))
    rays = scenes.incoherent_rays(3000, 78, tmax=float(NO_HIT))
    n_a, p_a = a.read_bvh(LAYOUT_BVH2)
    n_b, p_b = b.read_bvh(LAYOUT_BVH2)
    assert n_a.tobytes() == n_b.tobytes() and p_a.tobytes() == p_b.tobytes()  # BVH2 is deterministic
    assert np.array_equal(a.trace_geometry(rays).view(np.uint32), b.trace_geometry(rays).view(np.uint32))


def test_gpu_build_mixed(ctx):
    from test_mixed import assert_mixed_equal, mixed_rays

    sc = random_mixed(9)
    scene = ctx.create_scene_gpu(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    scene.download()
    rays = mixed_rays(9, 6000, sc)
    saved = ctx.launch_params
    for layout in (LAYOUT_BVH2, LAYOUT_BVH4):
        ctx.set_launch_params(layout=layout)
        expect, flags = pyoracle.trace_geometry_mixed(rays, None, **sc)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        got = scene.trace_geometry(rays)
        assert_mixed_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok], expect["v"][ok],
                           len(sc["tris"]), len(sc["spheres"]))
    ctx.set_launch_params(**saved)


def test_gpu_build_rejects_non_finite_and_handles_empty(ctx):
    tris = scenes.random_triangles(3000, 79)
    bad = tris.copy()
    bad["p1"][100, 0] = np.nan
    with pytest.raises(IgxrtError):
        ctx.create_scene_gpu(bad)
    with pytest.raises(IgxrtError):
        ctx.create_scene_gpu(triangle_tensor(bad))
    empty = ctx.create_scene_gpu(tris[:0])
    assert empty.info["bvh2_nodes"] == 0
    rays = scenes.incoherent_rays(100, 80, tmax=float(NO_HIT))
    assert (empty.trace_geometry(rays)["prim"] == 0xFFFFFFFF).all()
    ok = ctx.create_scene_gpu(tris)  # the context still works
    oracle_check(ok, tris, rays, "after a rejected build")


def test_gpu_build_has_no_bvh8(ctx):
    """GPU builds emit BVH2 and BVH4 only; the compressed BVH8 layout is a
    host-build layout, and tracing it on a GPU-built scene is refused."""
    tris = scenes.random_triangles(2000, 81)
    scene = ctx.create_scene_gpu(tris)
    assert scene.info["bvh8_nodes"] == 0
    saved = ctx.launch_params
    ctx.set_launch_params(layout=2)
    try:
        with pytest.raises(IgxrtError):
            scene.trace_geometry(scenes.incoherent_rays(64, 82))
    finally:
        ctx.set_launch_params(**saved)
