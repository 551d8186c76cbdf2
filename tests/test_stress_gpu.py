"""Randomized parity stress: random scenes, rays and launch shapes against the
oracle's traversal of the same tree, bit for bit.

Every launch ends with its warps' queues drained, so every case runs the tail
work sharing (helpers, merges, stack hand-offs across the shared/local
boundary) and the queue-slot reset; the batch case mixes closest-hit and
any-hit rays of several scenes in one launch."""
import math

import numpy as np
import pytest

from igx_raytracing_gb300 import BVH, scenes
from igx_raytracing_gb300._capi import HIT_DTYPE
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    n_tris = int(rng.integers(500, 40000))
    kind = seed % 3
    if kind == 0:
        tris = scenes.random_triangles(n_tris, 2000 + seed, mu=math.log(rng.uniform(0.002, 0.05)))
    elif kind == 1:
        tris = scenes.heightfield(int(rng.integers(8, 96)), int(rng.integers(8, 96)), 3000 + seed)
    else:  # a mix: a heightfield floor with random triangles above it
        tris = np.concatenate([scenes.heightfield(40, 40, 3000 + seed),
                               scenes.random_triangles(n_tris, 2000 + seed, mu=math.log(0.01))])
    n_rays = int(rng.integers(1, 120000))
    rays = scenes.incoherent_rays(n_rays, 4000 + seed)
    coherent = rng.random(n_rays) < 0.5  # half of them from one eye toward the scene
    rays["org"][coherent] = (0.5, 0.5, -1.0)
    d = rng.normal(size=(int(coherent.sum()), 3)) * 0.2 + (0.0, 0.0, 1.0)
    rays["dir"][coherent] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays["tmin"] = np.where(rng.random(n_rays) < 0.2, rng.uniform(0.0, 0.5, n_rays), 0.0).astype(np.float32)
    rays["tmax"] = np.where(rng.random(n_rays) < 0.3, rng.uniform(0.1, 2.0, n_rays),
                            3.4028235e38).astype(np.float32)
    prev = np.where(rng.random(n_rays) < 0.3, rng.integers(0, len(tris), n_rays), 0xFFFFFFFF).astype(np.uint32)
    params = dict(block_size=int(rng.choice([32, 64, 128, 256])),
                  stack_depth=int(rng.choice([0, 1, 2, 4, 8, 16])),
                  packet_size=int(rng.choice([8, 16, 24, 32, 64, 96, 256])),
                  refill_lanes=int(rng.choice([1, 4, 8, 16, 32])),
                  phase_break=int(rng.choice([1, 2, 3, 7, 32])),
                  layout=int(rng.integers(0, 3)))
    return tris, rays, prev, params


@pytest.mark.parametrize("seed", range(12))
def test_random_scenes_rays_and_launch_shapes(ctx, seed):
    tris, rays, prev, params = _case(seed)
    saved = ctx.launch_params
    b = BVH.build(tris)
    scene = ctx.create_scene(bvh=b)
    nodes, prims = b.arrays(params["layout"])
    try:
        ctx.set_launch_params(**params)
        hits = scene.trace_geometry(rays, prev)
        occ = scene.trace_occlusion(rays, prev)
    finally:
        ctx.set_launch_params(**saved)
    expect_h = pyoracle.bvh_trace(params["layout"], nodes, prims, rays, prev=prev, mode=0)
    expect_o = pyoracle.bvh_trace(params["layout"], nodes, prims, rays, prev=prev, mode=1)
    assert hits.tobytes() == expect_h.tobytes(), params
    assert np.array_equal(occ, expect_o), params


def test_random_batch_of_scenes_and_modes(ctx):
    """One persistent launch over items of different scenes, sizes and query
    modes (warps then hold closest-hit and any-hit rays together)."""
    import torch

    items, expect = [], []
    for k in range(10):
        tris, rays, prev, _ = _case(100 + k)
        b = BVH.build(tris)
        scene = ctx.create_scene(bvh=b)
        nodes, prims = b.arrays(0)
        mode = k % 2
        d_r = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        d_p = torch.from_numpy(prev.view(np.int32).copy()).cuda()
        out = (torch.empty((len(rays), 4), dtype=torch.float32, device="cuda") if mode == 0
               else torch.empty(len(rays), dtype=torch.int32, device="cuda"))
        items.append((scene, d_r, d_p, out, mode))
        expect.append(pyoracle.bvh_trace(0, nodes, prims, rays, prev=prev, mode=mode))
    ctx.trace_batch(items)
    torch.cuda.synchronize()
    for (scene, d_r, d_p, out, mode), e in zip(items, expect):
        got = out.cpu().numpy()
        if mode == 0:
            assert got.view(HIT_DTYPE).reshape(-1).tobytes() == e.tobytes()
        else:
            assert np.array_equal(got.view(np.uint32), e)
