"""igxrt_trace_closest_static: the closest-hit query for callers that may not
allocate device memory while they trace (a render loop under another
allocator's memory budget, or one that cannot absorb an allocation's
synchronisation).  It stages through a fixed 16 MiB device array instead of a
cudaMalloc'd buffer.  Its results must equal igxrt_trace_closest's, call after
call, and it must refuse batches beyond IGXRT_STATIC_MAX_RAYS.

This file is collected last so that a failure here does not hide the rest of
the suite; it also passes when run on its own in a fresh process.
"""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import bits
from igx_raytracing_gb300 import _capi, scenes
from igx_raytracing_gb300._capi import HIT_DTYPE

pytestmark = pytest.mark.gpu


def _static(lib, ctx, scene, rays, prev=None):
    out = np.zeros(len(rays), HIT_DTYPE)
    st = lib.igxrt_trace_closest_static(
        ctx.handle, scene.handle, rays.ctypes.data,
        None if prev is None else prev.ctypes.data, len(rays), out.ctypes.data, None)
    return st, out


def _same(a, b):
    assert np.array_equal(a["prim"], b["prim"])
    for f in ("t", "u", "v"):
        assert np.array_equal(bits(a[f]), bits(b[f]))


def test_static_entry_matches_regular_entry_on_consecutive_calls(ctx, engine_lib):
    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    expect = scene.trace_geometry(rays)  # igxrt_trace_closest, host arrays

    st, got = _static(engine_lib, ctx, scene, rays)
    assert st == 0, engine_lib.igxrt_last_error(ctx.handle)
    _same(got, expect)
    # a second call reuses the array: its counter must restart from zero
    st, got2 = _static(engine_lib, ctx, scene, rays)
    assert st == 0
    _same(got2, expect)

    # a different scene, prev_hit and ray count on the next call
    rt = scenes.random_triangles(40000, 555, mu=math.log(0.01))
    rr = scenes.incoherent_rays(150000, 556)
    prev = np.random.default_rng(1).integers(0, 40000, len(rr)).astype(np.uint32)
    s2 = ctx.create_scene(rt)
    expect2 = s2.trace_geometry(rr, prev)
    st, got3 = _static(engine_lib, ctx, s2, rr, prev)
    assert st == 0
    _same(got3, expect2)
    st, got4 = _static(engine_lib, ctx, scene, rays[:1000])
    assert st == 0
    _same(got4, expect[:1000])


def _scene_cases(ctx):
    """A triangle scene from the host builder (every layout), a mixed scene
    (spheres, cubes and planes beside the triangles) and a GPU-built scene
    (BVH2 and BVH4 only)."""
    tris = scenes.random_triangles(30000, 561, mu=math.log(0.01))
    mixed = scenes.workload_mixed(20000, 2000, 2000, 4)
    return [
        ("host", ctx.create_scene(tris), (0, 1, 2)),
        ("mixed", ctx.create_scene_mixed(mixed["tris"], mixed["spheres"], mixed["cubes"], mixed["planes"]),
         (0, 1, 2)),
        ("gpu", ctx.create_scene_gpu(tris), (0, 1)),
    ]


@pytest.mark.parametrize("case", ["host", "mixed", "gpu"])
def test_static_entry_matches_regular_entry_per_scene_kind_and_layout(ctx, engine_lib, case):
    name, scene, layouts = next(c for c in _scene_cases(ctx) if c[0] == case)
    rays = scenes.incoherent_rays(60000, 562)
    prev = np.random.default_rng(563).integers(0, 30000, len(rays)).astype(np.uint32)
    saved = ctx.launch_params
    try:
        for layout in layouts:
            ctx.set_launch_params(layout=layout)
            expect = scene.trace_geometry(rays, prev)
            for _ in range(2):  # two calls in a row share the array
                st, got = _static(engine_lib, ctx, scene, rays, prev)
                assert st == 0, engine_lib.igxrt_last_error(ctx.handle)
                _same(got, expect)
    finally:
        ctx.set_launch_params(**saved)


def test_static_entry_refuses_a_layout_the_scene_lacks(ctx, engine_lib):
    tris = scenes.random_triangles(5000, 564)
    scene = ctx.create_scene_gpu(tris)  # GPU-built trees have no BVH8 layout
    rays = scenes.incoherent_rays(1000, 565)
    saved = ctx.launch_params
    try:
        ctx.set_launch_params(layout=2)
        st, _ = _static(engine_lib, ctx, scene, rays)
        assert st == 8  # IGXRT_ERROR_UNSUPPORTED, nothing launched
        assert b"layout" in engine_lib.igxrt_last_error(ctx.handle)
    finally:
        ctx.set_launch_params(**saved)


def test_static_entry_allocates_no_device_memory(ctx, engine_lib):
    import torch

    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    st, _ = _static(engine_lib, ctx, scene, rays)  # first call: address lookup, module load
    assert st == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for n in (len(rays), 7, _capi.STATIC_MAX_RAYS):
        r = rays if n <= len(rays) else np.resize(rays, n)
        st, _ = _static(engine_lib, ctx, scene, np.ascontiguousarray(r[:n]))
        assert st == 0
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_static_entry_rejects_oversized_batches(ctx, engine_lib):
    tris, rays = scenes.workload_small()
    scene = ctx.create_scene(tris)
    n = _capi.STATIC_MAX_RAYS + 1
    big = np.resize(rays, n)
    st, _ = _static(engine_lib, ctx, scene, np.ascontiguousarray(big))
    assert st == 1  # IGXRT_ERROR_INVALID_ARGUMENT, nothing launched
    msg = engine_lib.igxrt_last_error(ctx.handle).decode()
    assert "IGXRT_STATIC_MAX_RAYS" in msg and str(_capi.STATIC_MAX_RAYS) in msg
    # the array is still usable afterwards
    st, got = _static(engine_lib, ctx, scene, rays[:4096].copy())
    assert st == 0
    _same(got, scene.trace_geometry(rays[:4096]))
