"""Host BVH builder (engine) + CPU traversal (oracle), no GPU needed.

The CPU traversal visits the engine's exported BVH in the kernels' order; it
must equal the brute-force linear loop bit for bit, in both node layouts.
"""
import math
import os

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, assert_hits_equal, closest_rays, load_golden, nan_free,
                      occlusion_rays)
from igx_raytracing_gb300 import BVH, IgxrtError, LAYOUT_BVH2, LAYOUT_BVH4, scenes
from igx_raytracing_gb300._capi import TRIANGLE_DTYPE
from oracle import pyoracle

LAYOUTS = [LAYOUT_BVH2, LAYOUT_BVH4]


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("leaf", [1, 4, 8, 16])
def test_cpu_bvh_matches_golden(case, layout, leaf):
    g = load_golden(case)
    b = BVH.build(g["tris"], max_leaf_size=leaf)
    b.validate()
    nodes, prims = b.arrays(layout)
    got = pyoracle.bvh_trace(layout, nodes, prims, closest_rays(g), g["prev"])
    ok = nan_free(g)
    assert_hits_equal(got[ok], g["hit_prim"][ok], g["hit_t"][ok], g["hit_u"][ok], g["hit_v"][ok],
                      case)
    occ = pyoracle.bvh_trace(layout, nodes, prims, occlusion_rays(g), g["prev"], mode=1)
    ok = nan_free(g, "occlusion")
    assert np.array_equal(occ[ok], g["occluded"][ok])


def test_nan_rays_are_rare_and_only_in_plane_cases():
    for case in GOLDEN_CASES:
        g = load_golden(case)
        bad = ~nan_free(g)
        if case != "edge_cases":
            assert not bad.any(), case
        else:  # the three rays that lie in a triangle's plane by construction
            assert 1 <= bad.sum() <= 12


@pytest.mark.parametrize("layout", LAYOUTS)
def test_cpu_bvh_matches_brute_force_random(layout):
    tris = scenes.random_triangles(20000, 4242, mu=math.log(0.01))
    rays = scenes.incoherent_rays(4000, 4343)
    b = BVH.build(tris)
    b.validate()
    nodes, prims = b.arrays(layout)
    expect, flags = pyoracle.trace_geometry(tris, rays)
    assert not (flags & pyoracle.EVENT_NAN_T).any()
    got = pyoracle.bvh_trace(layout, nodes, prims, rays)
    assert_hits_equal(got, expect["prim"], expect["t"], expect["u"], expect["v"], "random")


def test_sphere_rays_match_brute_force():
    # a small displaced sphere seen from outside: many rays graze silhouettes
    tris = scenes.displaced_sphere(64, 32, 0.02, 31)
    rays = scenes.pinhole_rays(96, 64, eye=(0.0, -3.0, 0.0), target=(0.0, 0.0, 0.0))
    expect, flags = pyoracle.trace_geometry(tris, rays)
    b = BVH.build(tris)
    for layout in LAYOUTS:
        nodes, prims = b.arrays(layout)
        got = pyoracle.bvh_trace(layout, nodes, prims, rays)
        ok = flags & pyoracle.EVENT_NAN_T == 0
        assert_hits_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok],
                          expect["v"][ok], "sphere")


def test_empty_and_tiny_scenes():
    for n in (0, 1, 2, 3):
        tris = scenes.random_triangles(n, 5, mu=math.log(0.3)) if n else np.zeros(0, TRIANGLE_DTYPE)
        b = BVH.build(tris)
        b.validate()
        info = b.info
        assert info["triangle_count"] == n
        rays = scenes.incoherent_rays(500, 6)
        expect, _ = pyoracle.trace_geometry(tris, rays)
        for layout in LAYOUTS:
            nodes, prims = b.arrays(layout)
            got = pyoracle.bvh_trace(layout, nodes, prims, rays)
            assert np.array_equal(got["prim"], expect["prim"])


def test_coincident_centroids_and_depth_bound():
    # 300 copies of one triangle: no SAH plane separates them
    tris = np.repeat(scenes.random_triangles(1, 7, mu=math.log(0.2)), 300)
    b = BVH.build(tris, max_leaf_size=4)
    b.validate()
    rays = scenes.incoherent_rays(300, 8)
    expect, _ = pyoracle.trace_geometry(tris, rays)
    nodes, prims = b.arrays(LAYOUT_BVH2)
    got = pyoracle.bvh_trace(LAYOUT_BVH2, nodes, prims, rays)
    assert np.array_equal(got["prim"], expect["prim"])  # ties: lowest copy index
    # geometrically shrinking triangles nest deeply
    k = np.arange(400)
    v0 = np.stack([0.5 ** (k / 8.0), np.zeros_like(k, dtype=float), np.zeros_like(k, dtype=float)], 1)
    tr = np.zeros(len(k), TRIANGLE_DTYPE)
    tr["p0"], tr["p1"], tr["p2"] = v0, v0 + [0, 1e-3, 0], v0 + [0, 0, 1e-3]
    b2 = BVH.build(tr, max_leaf_size=1)
    b2.validate()
    info = b2.info
    assert info["max_depth"] <= 80 and max(info["max_stack"]) <= 128


def test_invalid_inputs_rejected():
    tris = scenes.random_triangles(10, 1)
    bad = tris.copy()
    bad[3]["p1"][1] = np.nan
    with pytest.raises(IgxrtError):
        BVH.build(bad)
    bad["p1"][3][1] = np.inf
    with pytest.raises(IgxrtError):
        BVH.build(bad)
    for leaf in (17, 100):
        with pytest.raises(IgxrtError):
            BVH.build(tris, max_leaf_size=leaf)
    with pytest.raises(IgxrtError):
        BVH.build(tris, sah_bins=1)


def test_save_load_roundtrip(tmp_path):
    tris = scenes.random_triangles(5000, 11, mu=math.log(0.02))
    b = BVH.build(tris)
    p = os.path.join(tmp_path, "scene.bvh")
    b.save(p)
    c = BVH.load(p)
    c.validate()
    assert c.info == b.info
    for layout in LAYOUTS:
        n1, p1 = b.arrays(layout)
        n2, p2 = c.arrays(layout)
        assert n1.tobytes() == n2.tobytes() and p1.tobytes() == p2.tobytes()
    raw = open(p, "rb").read()
    # the primitive records are the file's last 48 * n bytes; record 0's
    # triangle index sits at byte 12 of it: the loader's validator refuses it
    corrupt = bytearray(raw)
    corrupt[len(raw) - 48 * 5000 + 12:len(raw) - 48 * 5000 + 16] = b"\xff\xff\xff\xff"
    open(p, "wb").write(bytes(corrupt))
    with pytest.raises(IgxrtError):
        BVH.load(p)
    open(p, "wb").write(raw[:-100])  # truncated
    with pytest.raises(IgxrtError):
        BVH.load(p)
    with pytest.raises(IgxrtError):
        BVH.load(os.path.join(tmp_path, "missing.bvh"))


def test_build_is_deterministic_across_thread_counts():
    tris = scenes.random_triangles(150000, 12)
    a = BVH.build(tris, threads=1)
    b = BVH.build(tris, threads=8)
    for layout in LAYOUTS:
        na, pa = a.arrays(layout)
        nb, pb = b.arrays(layout)
        assert na.tobytes() == nb.tobytes() and pa.tobytes() == pb.tobytes()


def test_fetch_counts_are_layout_specific_and_positive():
    tris, rays = scenes.workload_small()
    b = BVH.build(tris)
    n2, p2 = b.arrays(LAYOUT_BVH2)
    n4, p4 = b.arrays(LAYOUT_BVH4)
    _, nf2, pf2 = pyoracle.bvh_trace(LAYOUT_BVH2, n2, p2, rays, counts=True)
    _, nf4, pf4 = pyoracle.bvh_trace(LAYOUT_BVH4, n4, p4, rays, counts=True)
    assert (nf2 >= 1).all() and (nf4 >= 1).all()
    assert nf4.mean() < nf2.mean()
