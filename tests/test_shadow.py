"""The fused shadow pass (nv_all.shadow.comp as one kernel) against the
oracle's restatement: brute-force traceOcclusion per pixel and sample,
ballot-packed at indexToLight (light.glsl:221-229)."""
import numpy as np
import pytest

from igx_raytracing_gb300 import NO_RAY_HIT, RAY_DTYPE, scenes
from oracle import pyoracle


def shadow_setup(width=37, height=23, samples=3, seed=0):
    """Primary hits of a heightfield, then per pixel and sample a shadow ray
    toward a jittered point light (tmax = its distance)."""
    tris = scenes.heightfield(64, 32, scenes.seed_for(1, 40 + seed))
    prim = scenes.pinhole_rays(width, height, eye=(0.5, -1.0, 0.5), target=(0.5, 0.5, 0.0))
    hits, _ = pyoracle.trace_geometry(tris, prim)
    obj = hits["prim"].copy()
    rng = np.random.default_rng(seed)
    o = prim["org"].astype(np.float64) + hits["t"][:, None].astype(np.float64) * prim["dir"]
    o[obj == NO_RAY_HIT] = 0.0
    rays = np.zeros(width * height * samples, dtype=RAY_DTYPE)
    for s in range(samples):
        light = np.array([0.5, 0.5, 2.0]) + rng.uniform(-0.8, 0.8, 3)
        d = light - o
        dist = np.linalg.norm(d, axis=1)
        dist[dist == 0] = 1.0
        sl = slice(s * width * height, (s + 1) * width * height)
        rays["org"][sl] = o.astype(np.float32)
        rays["dir"][sl] = (d / dist[:, None]).astype(np.float32)
        rays["tmax"][sl] = dist.astype(np.float32)
    return tris, rays, obj


def test_oracle_packing_layout():
    # one occluded pixel per tile position: bit and word positions of the
    # reference's NVIDIA layout (16x2 tiles, word = tile.x + tile.y*tiles.x + s*tiles)
    tris = np.zeros(1, dtype=scenes.TRIANGLE_DTYPE)
    tris["p0"], tris["p1"], tris["p2"] = (-10, -10, 1), (30, -10, 1), (-10, 30, 1)
    w, h, s = 18, 3, 2
    rays = np.zeros(w * h * s, dtype=RAY_DTYPE)
    rays["dir"] = (0, 0, 1)
    rays["tmax"] = 0.5  # the triangle at z = 1 is beyond: nothing occluded
    obj = np.full(w * h, 7, dtype=np.uint32)  # a primary object that is not the occluder
    pick = [(0, 0, 0), (15, 1, 0), (16, 0, 0), (17, 2, 1), (3, 2, 1)]
    for x, y, smp in pick:
        rays["tmax"][(smp * h + y) * w + x] = 2.0
    mask, _ = pyoracle.shadow_mask(tris, rays, obj, w, h, s)
    tiles_x, tiles_y = 2, 2
    assert len(mask) == tiles_x * tiles_y * s
    expect = np.zeros_like(mask)
    for x, y, smp in pick:
        expect[(x >> 4) + (y >> 1) * tiles_x + smp * tiles_x * tiles_y] |= 1 << ((x & 15) | ((y & 1) << 4))
    assert np.array_equal(mask, expect)
    obj[:] = NO_RAY_HIT  # no primary hit: no rays, all words zero
    mask, _ = pyoracle.shadow_mask(tris, rays, obj, w, h, s)
    assert not mask.any()


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("dims", [(37, 23, 3), (16, 2, 1), (1, 1, 2), (64, 40, 2)])
def test_shadow_mask_matches_oracle(ctx, layout, dims):
    w, h, s = dims
    tris, rays, obj = shadow_setup(w, h, s, seed=w + h)
    expect, flags = pyoracle.shadow_mask(tris, rays, obj, w, h, s)
    assert not (flags & pyoracle.EVENT_NAN_T).any()
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    scene = ctx.create_scene(tris)
    got = ctx.trace_shadow_mask(scene, rays, obj, w, h, s)
    ctx.set_launch_params(**saved)
    assert np.array_equal(got, expect)
    if w * h >= 500:
        assert expect.any()  # the larger setups do shadow some pixels


@pytest.mark.gpu
def test_shadow_mask_device_memory(ctx):
    import torch

    w, h, s = 40, 30, 2
    tris, rays, obj = shadow_setup(w, h, s, seed=3)
    expect, _ = pyoracle.shadow_mask(tris, rays, obj, w, h, s)
    scene = ctx.create_scene(tris)
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_obj = torch.from_numpy(obj.view(np.int32).copy()).cuda()
    got = ctx.trace_shadow_mask(scene, d_rays, d_obj, w, h, s)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy().view(np.uint32), expect)


@pytest.mark.gpu
@pytest.mark.parametrize("memory", ["pageable", "pinned", "staged"])
def test_shadow_mask_host_routes_match_device_pass(ctx, memory):
    """Host arrays the kernels can address are read in place by the
    compaction (which gathers the traced rays into device memory) and the
    mask is stored in place; staged arrays go through device buffers.  The
    words equal the device-memory pass, which the tests above pin to the
    oracle; two samples make the object index wrap."""
    import torch

    w, h, s = 300, 200, 2
    tris = scenes.heightfield(64, 32, scenes.seed_for(1, 77))
    prim = scenes.pinhole_rays(w, h, eye=(0.5, -1.0, 0.5), target=(0.5, 0.5, 0.0))
    scene = ctx.create_scene(tris)
    hits = scene.trace_geometry(prim)
    obj = hits["prim"].copy()
    o = prim["org"] + hits["t"][:, None] * prim["dir"]
    o[obj == NO_RAY_HIT] = 0.0
    rays = np.zeros(w * h * s, dtype=RAY_DTYPE)
    for k, light in enumerate(([0.2, 0.3, 1.5], [0.8, 0.6, 1.2])):
        d = np.asarray(light, np.float32) - o
        dist = np.linalg.norm(d, axis=1).astype(np.float32)
        dist[dist == 0] = 1.0
        sl = slice(k * w * h, (k + 1) * w * h)
        rays["org"][sl] = o
        rays["dir"][sl] = d / dist[:, None]
        rays["tmax"][sl] = dist
    words = ((w + 15) // 16) * ((h + 1) // 2) * s
    if memory == "pinned":
        h_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory().numpy()
        h_rays = h_rays.view(RAY_DTYPE).reshape(-1)
        h_obj = torch.from_numpy(obj.view(np.int32).copy()).pin_memory().numpy().view(np.uint32)
        out = torch.zeros(words, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    else:
        h_rays, h_obj, out = rays, obj, np.zeros(words, dtype=np.uint32)
    ctx.stage_host_arrays = memory == "staged"
    try:
        got = ctx.trace_shadow_mask(scene, h_rays, h_obj, w, h, s, out=out)
    finally:
        ctx.stage_host_arrays = False
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_obj = torch.from_numpy(obj.view(np.int32).copy()).cuda()
    expect = ctx.trace_shadow_mask(scene, d_rays, d_obj, w, h, s)
    torch.cuda.synchronize()
    assert np.array_equal(got, expect.cpu().numpy().view(np.uint32))
    assert got.any() and (obj == NO_RAY_HIT).any()
