"""Mixed scenes (triangles, spheres, cubes, planes: the reference's four
primitive types, res/shaders/defines.glsl:1-4) through every pass: the
G-buffer (raygen.comp), the shadow mask (nv_all.shadow.comp), batches and the
server, against the oracle and, for the G-buffer, against the reference's own
traceGeometry (golden `niels_gbuffer`, NielsScene's primitives,
test/scene/niels_scene.cpp:10-52).

For a sphere, cube or plane hit the G-buffer's object normal is the hit's
geometry normal (trace.glsl:59-63), written through encodeNormal
(raygen.comp:46-51).  Everything is compared bit for bit."""
import math

import numpy as np
import pytest

from conftest import bits, load_golden
from igx_raytracing_gb300 import NO_RAY_HIT, RAY_DTYPE, Server, scenes
from oracle import pyoracle
from test_mixed import random_mixed


def golden_gbuffer():
    g = load_golden("niels_gbuffer")
    sc = dict(tris=g["tris"], spheres=g["spheres"], cubes=g["cubes"], planes=g["planes"])
    return g, sc


def test_oracle_mixed_gbuffer_matches_reference_golden():
    g, sc = golden_gbuffer()
    do, uv, flags = pyoracle.gbuffer_mixed(g["camera"], **sc, uv_fill=0.0)
    assert not flags.any()
    assert np.array_equal(bits(do), bits(g["dir_object"]))
    assert np.array_equal(bits(uv), bits(g["uv_normal"]))
    # every kind of object is seen, and some pixels miss
    obj = do[..., 3].view(np.uint32)
    n = np.cumsum([len(sc[k]) for k in ("tris", "spheres", "cubes", "planes")])
    kinds = np.searchsorted(n, obj[obj != NO_RAY_HIT], "right")
    assert set(kinds.tolist()) == {0, 1, 2, 3} and (obj == NO_RAY_HIT).any()


def mixed_camera(w, h, jitter=(0.5, 0.5)):
    return scenes.camera_record(w, h, eye=(0.5, -1.2, 0.6), target=(0.5, 0.5, 0.45), jitter=jitter)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_gbuffer_mixed_matches_reference_golden(ctx, layout):
    g, sc = golden_gbuffer()
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    try:
        scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        uv = np.zeros_like(g["uv_normal"])
        got_do, got_uv = ctx.trace_gbuffer(scene, g["camera"], uv_normal=uv)
    finally:
        ctx.set_launch_params(**saved)
    assert np.array_equal(bits(got_do), bits(g["dir_object"]))
    assert np.array_equal(bits(got_uv), bits(g["uv_normal"]))


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("seed,dims", [(11, (97, 61)), (12, (40, 24))])
def test_gbuffer_mixed_matches_oracle(ctx, layout, seed, dims):
    w, h = dims
    sc = random_mixed(seed)
    cam = mixed_camera(w, h, jitter=(0.3, 0.6))
    e_do, e_uv, flags = pyoracle.gbuffer_mixed(cam, **sc, uv_fill=-5.0)
    ok = ((flags & pyoracle.EVENT_NAN_T) == 0).reshape(h, w)
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    try:
        scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        got_do, got_uv = ctx.trace_gbuffer(scene, cam, uv_normal=np.full((h, w, 4), -5.0, np.float32))
    finally:
        ctx.set_launch_params(**saved)
    assert np.array_equal(bits(got_do)[ok], bits(e_do)[ok])
    assert np.array_equal(bits(got_uv)[ok], bits(e_uv)[ok])
    obj = e_do[..., 3].view(np.uint32)
    assert (obj[ok] >= len(sc["tris"])).any() and (obj[ok] < len(sc["tris"])).any()


def shadow_setup_mixed(sc, w, h, samples, seed):
    """Primary objects from the oracle's mixed G-buffer, then per pixel and
    sample a shadow ray toward a jittered point light (tmax = its distance),
    starting at the primary hit (eye + dirObject.xyz, nv_all.shadow.comp:84)."""
    cam = mixed_camera(w, h)
    do, _, flags = pyoracle.gbuffer_mixed(cam, **sc)
    obj = do[..., 3].view(np.uint32).reshape(-1).copy()
    eye = np.asarray(cam["eye"][0], np.float32)
    o = (eye[None, :] + do[..., :3].reshape(-1, 3)).astype(np.float32)
    rng = np.random.default_rng(seed)
    rays = np.zeros(w * h * samples, dtype=RAY_DTYPE)
    for s in range(samples):
        light = np.array([0.5, 0.5, 2.0]) + rng.uniform(-0.8, 0.8, 3)
        d = light - o.astype(np.float64)
        dist = np.linalg.norm(d, axis=1)
        dist[dist == 0] = 1.0
        sl = slice(s * w * h, (s + 1) * w * h)
        rays["org"][sl] = o
        rays["dir"][sl] = (d / dist[:, None]).astype(np.float32)
        rays["tmax"][sl] = dist.astype(np.float32)
    return rays, obj


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("dims", [(53, 29, 2), (16, 2, 1)])
def test_shadow_mask_mixed_matches_oracle(ctx, layout, dims):
    w, h, s = dims
    sc = random_mixed(21 + w)
    rays, obj = shadow_setup_mixed(sc, w, h, s, seed=w)
    expect, flags = pyoracle.shadow_mask_mixed(rays, obj, w, h, s, **sc)
    assert not (flags & pyoracle.EVENT_NAN_T).any()
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    try:
        scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        got = ctx.trace_shadow_mask(scene, rays, obj, w, h, s)
    finally:
        ctx.set_launch_params(**saved)
    assert np.array_equal(got, expect)
    if w * h >= 500:
        assert expect.any()


def _mixed_items(seed):
    """Two mixed scenes and one triangle-only scene, closest and any-hit
    queries, with and without prev_hit."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(3):
        sc = random_mixed(seed * 10 + k) if k < 2 else dict(
            tris=scenes.random_triangles(4000, 9100 + seed, mu=math.log(0.03)), spheres=None, cubes=None,
            planes=None)
        n = int(rng.integers(2000, 9000))
        rays = scenes.incoherent_rays(n, 9200 + seed * 10 + k, tmax=float(3.4028235e38))
        mode = k % 2
        if mode:
            rays["tmax"] = rng.uniform(0.02, 0.8, n).astype(np.float32)
        nobj = sum(len(v) for v in sc.values() if v is not None)
        prev = rng.integers(0, nobj, n).astype(np.uint32) if k != 1 else None
        out.append((sc, rays, prev, mode))
    return out


def _oracle(sc, rays, prev, mode):
    if mode == 0:
        return pyoracle.trace_geometry_mixed(rays, prev, **sc)
    return pyoracle.trace_occlusion_mixed(rays, prev, **sc)


def _equal(got, expect, mode, ok):
    if mode == 0:
        assert np.array_equal(got["prim"][ok], expect["prim"][ok])
        for f in ("t", "u", "v"):
            assert np.array_equal(bits(got[f])[ok], bits(expect[f])[ok]), f
    else:
        assert np.array_equal(np.asarray(got).view(np.uint32)[ok], expect[ok])


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_batch_with_mixed_scenes_matches_oracle(ctx, layout):
    import torch

    from igx_raytracing_gb300 import HIT_DTYPE

    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    try:
        items, expect = [], []
        for sc, rays, prev, mode in _mixed_items(layout):
            scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
            d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
            d_prev = None if prev is None else torch.from_numpy(prev.view(np.int32).copy()).cuda()
            out = (torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda") if mode == 0
                   else torch.zeros(len(rays), dtype=torch.int32, device="cuda"))
            items.append((scene, d_rays, d_prev, out, mode))
            expect.append(_oracle(sc, rays, prev, mode))
        batch = ctx.create_batch(items)
        for _ in range(2):  # a graph replay gives the same words
            batch.launch()
            torch.cuda.synchronize()
            for (scene, _, _, out, mode), (e, flags) in zip(items, expect):
                got = out.cpu().numpy()
                got = got.view(HIT_DTYPE).reshape(-1) if mode == 0 else got
                _equal(got, e, mode, (flags & pyoracle.EVENT_NAN_T) == 0)
        batch.close()
    finally:
        ctx.set_launch_params(**saved)


@pytest.mark.gpu
def test_server_serves_mixed_scenes_like_the_oracle(ctx):
    work = _mixed_items(7)
    srv = Server(ctx, streams=2, slice_rays=1024, max_batch_rays=6000)
    ids, scenes_ = [], []
    for sc, *_ in work:
        s = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
        scenes_.append(s)
        ids.append(srv.add_scene(s))
    tickets = [srv.submit(ids[k], rays, prev, mode) for k, (sc, rays, prev, mode) in enumerate(work)]
    outs = [srv.wait(t, timeout=60.0)["out"] for t in tickets]
    srv.close()
    for (sc, rays, prev, mode), got in zip(work, outs):
        e, flags = _oracle(sc, rays, prev, mode)
        _equal(got, e, mode, (flags & pyoracle.EVENT_NAN_T) == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_plain_queries_on_mixed_scenes_many_seeds(ctx, layout):
    """The plain calls on the same kind of items, several seeds: rays that a
    plane decides when they start free their lane early, and such a lane must
    not carry that decision into the ray it helps in the launch's tail."""
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    try:
        for seed in range(5, 11):
            for sc, rays, prev, mode in _mixed_items(seed):
                scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
                got = scene.trace_geometry(rays, prev) if mode == 0 else scene.trace_occlusion(rays, prev)
                e, flags = _oracle(sc, rays, prev, mode)
                _equal(got, e, mode, (flags & pyoracle.EVENT_NAN_T) == 0)
                scene.close()
    finally:
        ctx.set_launch_params(**saved)
