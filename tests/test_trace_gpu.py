"""GPU parity: the CUDA kernels against the reference-pinned golden fixtures,
the brute-force oracle and the CPU BVH traversal, through the C ABI."""
import math

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, NO_HIT, assert_hits_equal, bits, closest_rays, load_golden,
                      nan_free, occlusion_rays)
from igx_raytracing_gb300 import BVH, IgxrtError, LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8, scenes
from igx_raytracing_gb300._capi import HIT_DTYPE, TRIANGLE_DTYPE
from oracle import pyoracle

pytestmark = pytest.mark.gpu
LAYOUTS = [LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8]


@pytest.fixture
def params(ctx):
    saved = ctx.launch_params
    yield ctx
    ctx.set_launch_params(**saved)


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("layout", LAYOUTS)
def test_golden_closest_host_memory(params, case, layout):
    ctx = params
    ctx.set_launch_params(layout=layout)
    g = load_golden(case)
    scene = ctx.create_scene(g["tris"])
    got = scene.trace_geometry(closest_rays(g), g["prev"])
    ok = nan_free(g)
    assert_hits_equal(got[ok], g["hit_prim"][ok], g["hit_t"][ok], g["hit_u"][ok], g["hit_v"][ok],
                      case, rays=closest_rays(g)[ok], tris=g["tris"])
    occ = scene.trace_occlusion(occlusion_rays(g), g["prev"])
    ok = nan_free(g, "occlusion")
    assert np.array_equal(occ[ok], g["occluded"][ok])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_device_memory(ctx, case):
    import torch

    g = load_golden(case)
    scene = ctx.create_scene(g["tris"])
    rays = torch.from_numpy(closest_rays(g).view(np.float32).reshape(-1, 8).copy()).cuda()
    prev = torch.from_numpy(g["prev"].view(np.int32).copy()).cuda()
    out = scene.trace_geometry(rays, prev)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(HIT_DTYPE).reshape(-1)
    ok = nan_free(g)
    assert_hits_equal(got[ok], g["hit_prim"][ok], g["hit_t"][ok], g["hit_u"][ok], g["hit_v"][ok],
                      case)
    orays = torch.from_numpy(occlusion_rays(g).view(np.float32).reshape(-1, 8).copy()).cuda()
    occ = scene.trace_occlusion(orays, prev)
    torch.cuda.synchronize()
    ok = nan_free(g, "occlusion")
    assert np.array_equal(occ.cpu().numpy().view(np.uint32)[ok], g["occluded"][ok])
    ctx.sync()


def test_small_workload_all_rays_vs_brute_force(ctx):
    tris, rays = scenes.workload_small()
    expect, flags = pyoracle.trace_geometry(tris, rays)
    assert not flags.any()
    scene = ctx.create_scene(tris)
    got = scene.trace_geometry(rays)
    assert_hits_equal(got, expect["prim"], expect["t"], expect["u"], expect["v"], "heightfield",
                      rays=rays, tris=tris)


@pytest.mark.parametrize("block,depth,packet", [(32, 0, 32), (64, 8, 64), (128, 16, 64),
                                                (256, 32, 128), (128, 64, 4096), (256, 0, 32)])
@pytest.mark.parametrize("layout", LAYOUTS)
def test_launch_shapes_agree(params, block, depth, packet, layout):
    ctx = params
    tris = scenes.random_triangles(30000, 77, mu=math.log(0.01))
    rays = scenes.incoherent_rays(20000, 78)
    b = BVH.build(tris)
    nodes, prims = b.arrays(layout)
    expect = pyoracle.bvh_trace(layout, nodes, prims, rays)
    scene = ctx.create_scene(bvh=b)
    ctx.set_launch_params(block_size=block, stack_depth=depth, packet_size=packet, layout=layout)
    got = scene.trace_geometry(rays)
    assert_hits_equal(got, expect["prim"], expect["t"], expect["u"], expect["v"], "shape",
                      rays=rays, tris=tris)
    sh = rays.copy()
    sh["tmax"] = 0.05
    assert np.array_equal(scene.trace_occlusion(sh),
                          pyoracle.bvh_trace(layout, nodes, prims, sh, mode=1))


def test_fetch_counts_match_cpu_traversal(ctx):
    tris = scenes.random_triangles(50000, 91, mu=math.log(0.008))
    rays = scenes.incoherent_rays(30000, 92)
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    for layout in LAYOUTS:
        nodes, prims = b.arrays(layout)
        for mode in (0, 1):
            rr = rays.copy()
            if mode == 1:
                rr["tmax"] = 0.1
            _, nf, pf = pyoracle.bvh_trace(layout, nodes, prims, rr, mode=mode, counts=True)
            gnf, gpf = ctx.count_fetches(scene, rr, mode=mode, layout=layout)
            assert np.array_equal(gnf, nf) and np.array_equal(gpf, pf)


def test_empty_scene_and_zero_rays(ctx):
    scene = ctx.create_scene(np.zeros(0, TRIANGLE_DTYPE))
    rays = scenes.incoherent_rays(1000, 3)
    got = scene.trace_geometry(rays)
    assert (got["prim"] == 0xFFFFFFFF).all() and (bits(got["t"]) == bits(np.float32(NO_HIT))).all()
    assert not scene.trace_occlusion(rays).any()
    tris, _ = scenes.workload_small()
    s2 = ctx.create_scene(tris)
    assert len(s2.trace_geometry(rays[:0])) == 0


def test_single_triangle_scene(ctx):
    tris = scenes.random_triangles(1, 4, mu=math.log(0.5))
    rays = scenes.incoherent_rays(5000, 5)
    expect, _ = pyoracle.trace_geometry(tris, rays)
    got = ctx.create_scene(tris).trace_geometry(rays)
    assert_hits_equal(got, expect["prim"], expect["t"], expect["u"], expect["v"], "one")


def test_interval_semantics(ctx):
    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    base = scene.trace_geometry(rays)
    hit = base["prim"] != 0xFFFFFFFF
    # any-hit with tmax == closest t is not occluded by that hit; just above it is
    r = rays[hit].copy()
    r["tmax"] = base["t"][hit]
    assert not scene.trace_occlusion(r).any()
    r["tmax"] = np.nextafter(base["t"][hit], np.float32(np.inf))
    assert scene.trace_occlusion(r).all()
    # tmin beyond the first hit finds the next surface or nothing, as the oracle does
    r2 = rays[hit].copy()
    r2["tmin"] = base["t"][hit]
    expect, _ = pyoracle.trace_geometry(tris, r2)
    assert_hits_equal(scene.trace_geometry(r2), expect["prim"], expect["t"], expect["u"],
                      expect["v"], "tmin")
    # NaN and +inf tmax behave as noHit
    r3 = rays.copy()
    r3["tmax"] = np.nan
    assert np.array_equal(scene.trace_geometry(r3)["prim"], base["prim"])
    r3["tmax"] = np.inf
    assert np.array_equal(scene.trace_geometry(r3)["prim"], base["prim"])


def test_host_pointer_without_flag_is_rejected(ctx, engine_lib):
    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    out = np.zeros(len(rays), HIT_DTYPE)
    st = engine_lib.igxrt_trace_closest(ctx.handle, scene.handle, rays.ctypes.data, None,
                                        len(rays), out.ctypes.data, 0, None)
    assert st == 1
    assert b"IGXRT_TRACE_HOST_MEMORY" in engine_lib.igxrt_last_error(ctx.handle)
    with pytest.raises(IgxrtError):
        ctx.set_launch_params(block_size=48)


def test_determinism_and_permutation_invariance(ctx):
    tris = scenes.random_triangles(100000, 61)
    rays = scenes.incoherent_rays(200000, 62)
    scene = ctx.create_scene(tris)
    a = scene.trace_geometry(rays)
    b = scene.trace_geometry(rays)
    assert a.tobytes() == b.tobytes()
    perm = np.random.default_rng(0).permutation(len(rays))
    c = scene.trace_geometry(rays[perm])
    assert a[perm].tobytes() == c.tobytes()


def host_copy(a, memory):
    """a as pageable numpy memory, or in pinned host memory."""
    if memory != "pinned":
        return a.copy()
    import torch

    raw = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    buf = torch.empty(raw.size, dtype=torch.uint8).pin_memory().numpy()
    buf[:] = raw
    return buf.view(a.dtype).reshape(a.shape)


@pytest.mark.parametrize("memory", ["pageable", "pinned", "staged"])
@pytest.mark.parametrize("layout", LAYOUTS)
def test_host_array_routes_match_the_cpu_traversal(params, layout, memory):
    """Host arrays the kernels can address (pinned, or pageable on a device
    that reads host page tables) are read and written in place; with
    IGXRT_TRACE_STAGED they go through device buffers.  Every route gives the
    CPU traversal's hits, occlusion words and fetch counts."""
    ctx = params
    tris = scenes.random_triangles(20000, 93, mu=math.log(0.01))
    rays = host_copy(scenes.incoherent_rays(300_000, 94), memory)
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    nodes, prims = b.arrays(layout)
    ctx.set_launch_params(layout=layout)
    ctx.stage_host_arrays = memory == "staged"
    try:
        hits = host_copy(np.zeros(len(rays), dtype=HIT_DTYPE), memory)
        ctx.trace_closest(scene, rays, out=hits)
        expect, nf, pf = pyoracle.bvh_trace(layout, nodes, prims, rays, mode=0, counts=True)
        assert hits.tobytes() == expect.tobytes()
        gnf, gpf = ctx.count_fetches(scene, rays, mode=0, layout=layout)
        assert np.array_equal(gnf, nf) and np.array_equal(gpf, pf)
        sh = rays.copy()
        sh["tmax"] = 0.2
        sh = host_copy(sh, memory)
        prev = host_copy(hits["prim"].copy(), memory)
        occ = host_copy(np.zeros(len(rays), dtype=np.uint32), memory)
        ctx.trace_any(scene, sh, prev, out=occ)
        assert np.array_equal(occ, pyoracle.bvh_trace(layout, nodes, prims, sh, prev=prev, mode=1))
        assert occ.any() and not occ.all()
    finally:
        ctx.stage_host_arrays = False


def test_staged_flag_needs_the_host_flag(ctx, engine_lib):
    import ctypes as C

    tris = scenes.random_triangles(100, 95)
    scene = ctx.create_scene(tris)
    rays = scenes.incoherent_rays(64, 96)
    out = np.zeros(64, dtype=HIT_DTYPE)
    st = engine_lib.igxrt_trace_closest(ctx.handle, scene.handle, rays.ctypes.data, None, 64,
                                        out.ctypes.data, 2, C.c_void_p(0))
    assert st == 1
    assert b"IGXRT_TRACE_STAGED" in engine_lib.igxrt_last_error(ctx.handle)
