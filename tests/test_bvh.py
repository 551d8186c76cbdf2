"""Host BVH builder (engine) + CPU traversal (oracle), no GPU needed.

The CPU traversal visits the engine's exported BVH in the kernels' order; it
must equal the brute-force linear loop bit for bit, in every node layout.
"""
import math
import os

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, assert_hits_equal, closest_rays, load_golden, nan_free,
                      occlusion_rays)
from igx_raytracing_gb300 import BVH, IgxrtError, LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8, scenes
from igx_raytracing_gb300._capi import TRIANGLE_DTYPE
from oracle import pyoracle

LAYOUTS = [LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8]


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
    assert_hits_equal(got, expect["prim"], expect["t"], expect["u"], expect["v"], "random", rays=rays, tris=tris)


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


def test_bvh8_quantized_boxes_hold_their_bvh2_sources():
    """Every BVH8 slot, decoded as the kernels decode it (fmaf(q, 2^exp,
    origin) in binary32), contains the exact padded box it was quantized
    from; the validator rejects a slot shrunk by one step."""
    tris = scenes.random_triangles(5000, 77, mu=math.log(0.02))
    b = BVH.build(tris)
    info = b.info
    assert info["bvh8_nodes"] > 0 and info["max_stack"][LAYOUT_BVH8] <= 128
    n8, _ = b.arrays(LAYOUT_BVH8)
    n2, _ = b.arrays(LAYOUT_BVH2)
    assert (n8["exp"] >= -126).all()
    step = np.ldexp(np.float32(1), n8["exp"].astype(np.int32)).astype(np.float32)  # (N, 3)
    for axis, (lo_f, hi_f) in enumerate((("lo_x", "hi_x"), ("lo_y", "hi_y"), ("lo_z", "hi_z"))):
        org = n8["origin"][:, axis:axis + 1]
        s = step[:, axis:axis + 1]
        # float32 fma: the product of a byte and a power of two is exact, so
        # one float32 rounding of (q * s + origin) is the sum rounded once
        dec_lo = (n8[lo_f].astype(np.float64) * s + org).astype(np.float32)
        dec_hi = (n8[hi_f].astype(np.float64) * s + org).astype(np.float32)
        valid = (n8["valid"][:, None] >> np.arange(8)) & 1 == 1
        assert (dec_lo <= dec_hi)[valid].all()
    # the root's slots hold the BVH2 root's children
    root_lo = min(n2[0]["c0_x"][0], n2[0]["c1_x"][0])
    assert np.float32(n8[0]["origin"][0]) == root_lo



def test_bvh8_validator_rejects_a_collapsed_slot(tmp_path):
    tris = scenes.random_triangles(3000, 78, mu=math.log(0.03))
    b = BVH.build(tris)
    path = os.path.join(tmp_path, "b.bvh")
    b.save(path)
    raw = bytearray(open(path, "rb").read())
    n2, prims = b.arrays(LAYOUT_BVH2)
    n4, _ = b.arrays(LAYOUT_BVH4)
    n8, _ = b.arrays(LAYOUT_BVH8)
    header = 8 + 4 + 4 + 8 * 8 + 96
    off8 = (header + len(tris) * 48 + len(n2) * 64 + len(n4) * 128 + len(prims) * 48)
    assert off8 + len(n8) * 96 + len(n8) * 32 == len(raw)
    hi_x = off8 + 24  # node 0, slot 0
    lo_x = off8 + 16
    raw[hi_x] = raw[lo_x]  # slot 0 of the root collapses to one plane on x
    open(path, "wb").write(bytes(raw))
    with pytest.raises(IgxrtError):
        BVH.load(path)
