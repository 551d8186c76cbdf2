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
                                                (256, 32, 128), (128, 64, 4096), (256, 0, 32),
                                                (128, 2, 32), (128, 16, 8), (64, 16, 24)])
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
    with pytest.raises(IgxrtError):
        ctx.set_launch_params(packet_size=12)  # not a multiple of 8


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


def _quad_scene():
    """Triangles 0 and 1: a 4x4 quad at z = 1; behind it, at z = 2, a grid of
    small triangles.  Rays toward +z hit triangle 0 or 1 unless prev_hit
    excludes it."""
    back = scenes.heightfield(32, 32, scenes.seed_for(3, 1))
    back["p0"][:, 2] = 2.0
    back["p1"][:, 2] = 2.0
    back["p2"][:, 2] = 2.0
    quad = np.zeros(2, dtype=TRIANGLE_DTYPE)
    quad["p0"] = [(-1.5, -1.5, 1.0), (2.5, 2.5, 1.0)]
    quad["p1"] = [(2.5, -1.5, 1.0), (-1.5, 2.5, 1.0)]
    quad["p2"] = [(-1.5, 2.5, 1.0), (2.5, -1.5, 1.0)]
    return np.concatenate([quad, back])


def _up_rays(n, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, dtype=scenes.RAY_DTYPE)
    rays["org"][:, :2] = rng.uniform(0.05, 0.95, (n, 2))
    rays["dir"] = (0.0, 0.0, 1.0)
    rays["tmax"] = np.float32(3.4028235e38)
    return rays


def test_a_launch_sees_the_writes_of_the_trace_before_it(ctx):
    """Trace launches may start while the kernel before them drains; without
    IGXRT_TRACE_INDEPENDENT the kernel waits for that kernel's writes before
    reading its inputs.  Here the second trace's prev_hit is the first one's
    output (0 or 1 per ray), which decides almost every closest hit."""
    import torch

    tris = _quad_scene()
    scene = ctx.create_scene(tris)
    n = 600_000
    a_rays = _up_rays(n, 5)
    a_rays["tmax"] = np.where(np.arange(n) % 3 == 0, 0.5, 1.5).astype(np.float32)  # occluded iff tmax > 1
    b_rays = _up_rays(n, 6)
    d_a = torch.from_numpy(a_rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_b = torch.from_numpy(b_rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    for rep in range(3):
        occ = torch.full((n,), -1, dtype=torch.int32, device="cuda")  # stale: no exclusion
        hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        ctx.trace_any(scene, d_a, out=occ)
        ctx.trace_closest(scene, d_b, occ, out=hits)
        torch.cuda.synchronize()
        prev = occ.cpu().numpy().view(np.uint32)
        assert set(np.unique(prev)) == {0, 1}
        got = hits.cpu().numpy().view(HIT_DTYPE).reshape(-1)
        expect = scene.trace_geometry(b_rays, prev)
        assert got.tobytes() == expect.tobytes()
        assert (got["prim"] >= 2).sum() > n // 3  # the exclusions mattered


def test_independent_launches_and_queue_slot_reuse(ctx):
    """IGXRT_TRACE_INDEPENDENT launches give the results of the same calls
    made one at a time; 4,200 back-to-back launches wrap the context's ring of
    4,096 queue slots, each left zeroed by its previous launch's last warp."""
    import torch

    tris = _quad_scene()
    scene = ctx.create_scene(tris)
    rays = _up_rays(4096, 7)
    rays["tmax"] = np.where(np.arange(4096) % 2 == 0, 0.5, 1.5).astype(np.float32)
    expect_hits = scene.trace_geometry(rays)
    expect_occ = scene.trace_occlusion(rays)
    d_r = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    outs_h = [torch.empty((64, 4), dtype=torch.float32, device="cuda") for _ in range(64)]
    outs_o = [torch.empty(64, dtype=torch.int32, device="cuda") for _ in range(64)]
    for k in range(4200):
        j = (k // 2) % 64  # every slice gets both queries, many times over
        sl = slice(64 * j, 64 * (j + 1))
        if k % 2 == 0:
            ctx.trace_closest(scene, d_r[sl], out=outs_h[j], independent=True)
        else:
            ctx.trace_any(scene, d_r[sl], out=outs_o[j], independent=True)
    torch.cuda.synchronize()
    ctx.sync()
    got_h = torch.cat(outs_h).cpu().numpy().view(HIT_DTYPE).reshape(-1)
    got_o = torch.cat(outs_o).cpu().numpy().view(np.uint32)
    assert got_h.tobytes() == expect_hits.tobytes()
    assert np.array_equal(got_o, expect_occ)
    assert expect_occ.any() and not expect_occ.all()


def test_pinned_tensors_take_the_stream_ordered_path(ctx):
    """Pinned CPU tensors are addressable by the kernels: the call queues the
    launch on the stream (no host synchronization) and the kernel reads the
    rays and writes the results in host memory; after a stream
    synchronization they equal the host-memory call's."""
    import torch

    tris = scenes.random_triangles(20000, 97, mu=math.log(0.01))
    rays = scenes.incoherent_rays(200_000, 98)
    rays["tmax"] = np.where(np.arange(len(rays)) % 2 == 0, 0.3, 3.0e38).astype(np.float32)
    scene = ctx.create_scene(tris)
    h_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    hits = ctx.trace_closest(scene, h_rays)
    assert hits.is_pinned() and not hits.is_cuda
    prev = torch.from_numpy(np.arange(len(rays), dtype=np.int32) % 20000).pin_memory()
    occ = ctx.trace_any(scene, h_rays, prev, independent=True)
    torch.cuda.synchronize()
    assert hits.numpy().view(HIT_DTYPE).reshape(-1).tobytes() == scene.trace_geometry(rays).tobytes()
    expect = scene.trace_occlusion(rays, prev.numpy().view(np.uint32))
    assert np.array_equal(occ.numpy().view(np.uint32), expect)
    assert expect.any() and not expect.all()
