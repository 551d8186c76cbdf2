"""Batched multi-scene launches and the autotuner (GPU).

A batch must return, item for item, exactly what the plain kernel returns for
that item alone: the batched kernel only changes which warp traces a ray.
"""
import math
import os

import numpy as np
import pytest

from conftest import bits
from igx_raytracing_gb300 import IgxrtError, scenes

pytestmark = pytest.mark.gpu


def _items(ctx, seed=0, nscenes=9, with_empty=True):
    import torch

    rng = np.random.default_rng(seed)
    items, plain = [], []
    for s in range(nscenes):
        ntri = int(rng.integers(200, 40000))
        tris = scenes.random_triangles(ntri, 7000 + seed * 100 + s, mu=math.log(0.02))
        scene = ctx.create_scene(tris)
        nray = int(rng.integers(1, 30000)) if not (with_empty and s == 3) else 0
        rays = scenes.batch_rays(s, nray) if nray else scenes.incoherent_rays(0, 1)
        mode = s % 2
        if mode == 1:
            rays["tmax"] = rng.uniform(0.01, 0.5, len(rays)).astype(np.float32)
        prev = None
        if s % 3 == 0 and nray:
            prev = rng.integers(0, ntri, nray).astype(np.uint32)
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        d_prev = None if prev is None else torch.from_numpy(prev.view(np.int32).copy()).cuda()
        out = (torch.full((nray, 4), -1.0, dtype=torch.float32, device="cuda") if mode == 0
               else torch.full((nray,), 7, dtype=torch.int32, device="cuda"))
        items.append((scene, d_rays, d_prev, out, mode))
        plain.append(scene.trace_geometry(rays, prev) if mode == 0 else scene.trace_occlusion(rays, prev))
    return items, plain


def _check(items, plain):
    import torch

    torch.cuda.synchronize()
    for (scene, d_rays, d_prev, out, mode), expect in zip(items, plain):
        got = out.cpu().numpy()
        if mode == 0:
            got = got.view(np.uint32).reshape(-1, 4)
            assert np.array_equal(got[:, 3], expect["prim"])
            assert np.array_equal(got[:, 0], bits(expect["t"]))
            assert np.array_equal(got[:, 1], bits(expect["u"]))
            assert np.array_equal(got[:, 2], bits(expect["v"]))
        else:
            assert np.array_equal(got.view(np.uint32), expect)


@pytest.fixture
def params(ctx):
    saved = ctx.launch_params
    yield ctx
    ctx.set_launch_params(**saved)


@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("packet,refill", [(8, 8), (16, 4), (32, 1), (64, 8), (256, 32)])
def test_trace_batch_matches_plain(params, layout, packet, refill):
    ctx = params
    ctx.set_launch_params(layout=layout, packet_size=packet, refill_lanes=refill)
    items, plain = _items(ctx, seed=layout * 10 + packet)
    ctx.trace_batch(items)
    _check(items, plain)
    ctx.sync()


def test_graph_batch_replays_identically(ctx):
    import torch

    items, plain = _items(ctx, seed=5)
    batch = ctx.create_batch(items)
    for _ in range(3):
        for _, _, _, out, _ in items:
            out.fill_(0)
        batch.launch()
        _check(items, plain)
    batch.close()
    # an explicit parameter set, BVH4
    batch = ctx.create_batch(items, params={"layout": 1, "packet_size": 128, "block_size": 256,
                                            "stack_depth": 8, "refill_lanes": 4})
    batch.launch()
    _check(items, plain)
    batch.close()
    torch.cuda.synchronize()
    ctx.sync()


def test_batch_rejects_host_arrays(ctx, engine_lib):
    from igx_raytracing_gb300 import _capi

    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    out = np.zeros((len(rays), 4), np.float32)
    arr = (_capi.BatchItem * 1)()
    arr[0].scene = scene.handle.value
    arr[0].rays = rays.ctypes.data
    arr[0].out = out.ctypes.data
    arr[0].count = len(rays)
    arr[0].mode = 0
    assert engine_lib.igxrt_trace_batch(ctx.handle, arr, 1, None) == 1
    assert b"device memory" in engine_lib.igxrt_last_error(ctx.handle)


def test_autotune_and_cache(ctx, tmp_path):
    items, plain = _items(ctx, seed=9, nscenes=6, with_empty=False)
    cache = os.path.join(tmp_path, "tune.txt")
    p, ms = ctx.autotune(items, reps=2, cache_path=cache, class_key="unit-test")
    assert ms > 0 and p["layout"] in (0, 1, 2) and p["packet_size"] in (8, 16, 32, 64, 128, 256)
    text = open(cache).read()
    assert "unit-test" in text
    p2, ms2 = ctx.autotune(items, reps=2, cache_path=cache, class_key="unit-test")
    assert p2 == p and abs(ms2 - ms) < 1e-3  # served from the cache
    p3, _ = ctx.autotune(items, reps=1, layouts=[1], force=True)
    assert p3["layout"] == 1
    # the tuned parameters give the same results
    batch = ctx.create_batch(items, params=p)
    batch.launch()
    _check(items, plain)
    batch.close()
    with pytest.raises(IgxrtError):
        ctx.autotune([])


def test_autotune_plain_launches(ctx, tmp_path):
    """IGXRT_TUNE_PLAIN times one plain launch per item; its pick traces the
    items through the plain calls with the same results, and it is cached
    under its own key."""
    import torch

    items, plain = _items(ctx, seed=10, nscenes=4, with_empty=False)
    cache = os.path.join(tmp_path, "tune.txt")
    p, ms = ctx.autotune(items, reps=2, cache_path=cache, class_key="unit-test", plain=True)
    assert ms > 0 and p["layout"] in (0, 1, 2) and p["block_size"] in (64, 128, 256)
    pb, _ = ctx.autotune(items, reps=2, cache_path=cache, class_key="unit-test")
    lines = open(cache).read().splitlines()
    assert any("unit-test|plain" in l for l in lines) and any(l.split("\t")[0].endswith("unit-test") for l in lines)
    before = dict(ctx.launch_params)
    ctx.set_launch_params(**p)
    try:
        for scene, rays, prev, out, mode in items:
            out.zero_()
            if mode == 0:
                ctx.trace_closest(scene, rays, prev, out=out)
            else:
                ctx.trace_any(scene, rays, prev, out=out)
        torch.cuda.synchronize()
        _check(items, plain)
    finally:
        ctx.set_launch_params(**before)
