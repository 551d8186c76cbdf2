"""The fused primary pass (raygen.comp as one kernel): ray generation,
closest hit and the shader's output encodings.

CPU: the oracle's decodeSpheremap / encodeNormal / interpolate restatement
against the reference's own code (golden `normals`).  GPU: the kernel's two
images against the oracle's, bit for bit."""
import numpy as np
import pytest

from conftest import bits, load_golden
from igx_raytracing_gb300 import scenes
from oracle import pyoracle


def test_decode_encode_match_reference():
    g = load_golden("normals")
    assert np.array_equal(bits(pyoracle.decode_spheremap(g["dec_in"])), bits(g["dec_out"]))
    assert np.array_equal(pyoracle.encode_normal(g["enc_in"]), g["enc_out"])


def test_object_normal_matches_reference():
    # trace.glsl:50-57: interpolate(decodeSpheremap(n0..n2), uv) of the hit triangle,
    # computed with float32 operations in the shader's order
    g = load_golden("normals")
    hit = g["hit_prim"] != 0xFFFFFFFF
    t = g["tris"][g["hit_prim"][hit]]
    n0, n1, n2 = (pyoracle.decode_spheremap(t[f]) for f in ("n0", "n1", "n2"))
    u = g["hit_u"][hit][:, None].astype(np.float32)
    v = g["hit_v"][hit][:, None].astype(np.float32)
    w = (np.float32(1) - u) - v
    n = (u * n1 + v * n2) + w * n0
    assert n.dtype == np.float32
    assert np.array_equal(bits(n), bits(g["object_normal"][hit]))


def normals_scene():
    g = load_golden("normals")
    return g["tris"]


def test_oracle_gbuffer_encodes_hits_and_misses():
    tris = normals_scene()
    cam = scenes.camera_record(24, 16, eye=(0.5, -1.0, 0.5), target=(0.5, 0.5, 0.5))
    do, uv, flags = pyoracle.gbuffer(tris, cam, uv_fill=-7.0)
    obj = do[..., 3].view(np.uint32)
    hit = obj != 0xFFFFFFFF
    assert hit.any() and (~hit).any()
    assert (uv[~hit] == -7.0).all()  # the shader writes uv_normal on hits only
    assert not flags.any()


@pytest.mark.gpu
@pytest.mark.parametrize("route", ["host", "device"])
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("dims,jitter", [((61, 37), (0.5, 0.5)), ((8, 4), (0.0, 0.0)),
                                         ((130, 67), (0.123, 0.877))])
def test_gbuffer_matches_oracle(ctx, layout, dims, jitter, route):
    """Host images (written in place) and device images, on images whose
    last tile row and column lie partly outside."""
    w, h = dims
    tris = normals_scene()
    cam = scenes.camera_record(w, h, eye=(0.5, -1.2, 0.6), target=(0.5, 0.5, 0.45), jitter=jitter)
    e_do, e_uv, flags = pyoracle.gbuffer(tris, cam, uv_fill=-3.0)
    assert not flags.any()
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    scene = ctx.create_scene(tris)
    uv = np.full((h, w, 4), -3.0, dtype=np.float32)
    if route == "device":
        import torch

        d_do = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        d_uv = torch.from_numpy(uv).cuda()
        ctx.trace_gbuffer(scene, cam, d_do, d_uv)
        torch.cuda.synchronize()
        g_do, g_uv = d_do.cpu().numpy(), d_uv.cpu().numpy()
    else:
        g_do, g_uv = ctx.trace_gbuffer(scene, cam, uv_normal=uv)
    ctx.set_launch_params(**saved)
    assert np.array_equal(bits(g_do), bits(e_do))
    assert np.array_equal(bits(g_uv), bits(e_uv))


@pytest.mark.gpu
def test_gbuffer_device_memory(ctx):
    import torch

    tris = normals_scene()
    w, h = 64, 48
    cam = scenes.camera_record(w, h, eye=(0.5, 0.5, -1.5), target=(0.5, 0.5, 0.5), up=(0, 1, 0))
    e_do, e_uv, _ = pyoracle.gbuffer(tris, cam, uv_fill=0.0)
    scene = ctx.create_scene(tris)
    d_do = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    d_uv = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.trace_gbuffer(scene, cam, d_do, d_uv)
    torch.cuda.synchronize()
    assert np.array_equal(bits(d_do.cpu().numpy()), bits(e_do))
    assert np.array_equal(bits(d_uv.cpu().numpy()), bits(e_uv))


@pytest.mark.gpu
def test_camera_rays_split_the_gbuffer_pass(ctx):
    """igxrt_camera_rays + igxrt_trace_closest reproduce the fused pass's
    dir_object image bit for bit (hits: dir * t and the object id; misses:
    the direction and noRayHit)."""
    tris = normals_scene()
    w, h = 67, 41
    cam = scenes.camera_record(w, h, eye=(0.5, -1.2, 0.6), target=(0.5, 0.5, 0.45), jitter=(0.3, 0.7))
    scene = ctx.create_scene(tris)
    g_do, _ = ctx.trace_gbuffer(scene, cam)
    rays = ctx.camera_rays(cam)
    assert (rays["org"] == rays["org"][0]).all() and (rays["tmin"] == 0).all()
    hits = ctx.trace_closest(scene, rays)
    d = rays["dir"].astype(np.float32)
    hit = hits["prim"] != 0xFFFFFFFF
    expect = np.zeros((w * h, 4), np.float32)
    expect[:, :3] = np.where(hit[:, None], d * hits["t"][:, None].astype(np.float32), d)
    expect[:, 3] = hits["prim"].view(np.float32)
    assert np.array_equal(bits(g_do.reshape(-1, 4)), bits(expect))


@pytest.mark.gpu
@pytest.mark.parametrize("memory", ["pageable", "pinned", "staged"])
def test_gbuffer_host_routes_match_oracle(ctx, memory):
    """Host images the kernel can address are written in place, so a miss
    leaves the caller's uv_normal untouched without an upload; staged images
    carry it through the device.  Both equal the oracle, on a ragged image
    (the last tile row and column half outside it)."""
    w, h = 613, 389
    tris = normals_scene()
    cam = scenes.camera_record(w, h, eye=(0.5, -1.2, 0.6), target=(0.5, 0.5, 0.45), jitter=(0.25, 0.75))
    e_do, e_uv, flags = pyoracle.gbuffer(tris, cam, uv_fill=-3.0)
    assert not flags.any()
    scene = ctx.create_scene(tris)
    if memory == "pinned":
        import torch

        g_do = torch.zeros((h, w, 4), dtype=torch.float32).pin_memory().numpy()
        g_uv = torch.full((h, w, 4), -3.0, dtype=torch.float32).pin_memory().numpy()
    else:
        g_do = np.zeros((h, w, 4), dtype=np.float32)
        g_uv = np.full((h, w, 4), -3.0, dtype=np.float32)
    ctx.stage_host_arrays = memory == "staged"
    try:
        ctx.trace_gbuffer(scene, cam, g_do, g_uv)
        rays = ctx.camera_rays(cam)
    finally:
        ctx.stage_host_arrays = False
    assert np.array_equal(bits(g_do), bits(e_do))
    assert np.array_equal(bits(g_uv), bits(e_uv))
    hit = g_do[..., 3].view(np.uint32) != 0xFFFFFFFF
    assert hit.any() and (~hit).any()
    assert rays.tobytes() == ctx.camera_rays(cam).tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("route", ["host", "device"])
def test_gbuffer_empty_scene_misses_everywhere(ctx, route):
    """A scene without primitives: every pixel a miss ({dir, noRayHit}), the
    caller's uv_normal untouched, in both forms."""
    w, h = 37, 21
    cam = scenes.camera_record(w, h, eye=(0.5, -1.2, 0.6), target=(0.5, 0.5, 0.45))
    e_do, e_uv, _ = pyoracle.gbuffer(np.zeros(0, dtype=normals_scene().dtype), cam, uv_fill=-3.0)
    scene = ctx.create_scene(np.zeros(0, dtype=normals_scene().dtype))
    uv = np.full((h, w, 4), -3.0, dtype=np.float32)
    if route == "device":
        import torch

        d_do = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        d_uv = torch.from_numpy(uv).cuda()
        ctx.trace_gbuffer(scene, cam, d_do, d_uv)
        torch.cuda.synchronize()
        g_do, g_uv = d_do.cpu().numpy(), d_uv.cpu().numpy()
    else:
        g_do, g_uv = ctx.trace_gbuffer(scene, cam, uv_normal=uv)
    assert (g_do[..., 3].view(np.uint32) == 0xFFFFFFFF).all()
    assert np.array_equal(bits(g_do), bits(e_do))
    assert (g_uv == -3.0).all() and np.array_equal(bits(g_uv), bits(e_uv))
