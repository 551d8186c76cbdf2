"""Scenes with spheres, cubes and planes (the reference's other primitive
types, primitive.glsl:173-333, in the global order of trace.glsl:22-46).

Tolerance: object ids and t bit-exact; u, v within 2 ulp (the tolerance of
the traversal's floating-point outputs), and bit-exact in practice.  A sphere
hit's uv is asin/atan(..) * 0.3183.. + 0.5 (primitive.glsl:198-204), which
cancels towards 0 near the poles and the seam, so one ulp of difference in
asin or atan would show as many ulp of u; the engine and the oracle both
evaluate asin and atan correctly rounded (binary64, rounded once to
binary32), which leaves them no room to differ."""
import math
import os

import numpy as np
import pytest

from conftest import NO_HIT, bits, load_golden
from igx_raytracing_gb300 import BVH, IgxrtError, scenes
from igx_raytracing_gb300._capi import CUBE_DTYPE
from oracle import pyoracle

UV_ULPS = 2


def golden_scene():
    g = load_golden("niels_mixed")
    return g, dict(tris=g["tris"], spheres=g["spheres"], cubes=g["cubes"], planes=g["planes"])


def ulp_diff(a, b):
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7fffffff), ia)
    ib = np.where(ib < 0, -(ib & 0x7fffffff), ib)
    return np.abs(ia - ib)


def assert_mixed_equal(got, prim, t, u, v, n_tris, n_spheres):
    assert np.array_equal(got["prim"], prim)
    hit = prim != 0xFFFFFFFF
    assert np.array_equal(bits(got["t"])[hit], bits(t)[hit])
    sphere = hit & (prim >= n_tris) & (prim < n_tris + n_spheres)
    other = hit & ~sphere
    for f, e in (("u", u), ("v", v)):
        assert np.array_equal(bits(got[f])[other], bits(e)[other])
        if sphere.any():
            d = ulp_diff(got[f][sphere], e[sphere])
            assert d.max() <= UV_ULPS, (f, int(d.max()), int((d > 0).sum()))


def random_mixed(seed, nt=3000, ns=400, nc=300, npl=2):
    rng = np.random.default_rng(seed)
    tris = scenes.random_triangles(nt, 6000 + seed, mu=math.log(0.05))
    spheres = np.concatenate([rng.uniform(0, 1, (ns, 3)), rng.uniform(0.005, 0.05, (ns, 1))], 1)
    lo = rng.uniform(0, 1, (nc, 3))
    hi = lo + rng.uniform(0.01, 0.08, (nc, 3))
    cubes = np.zeros(nc, CUBE_DTYPE)
    cubes["xy0"] = lo[:, :2]
    cubes["z0_x1"] = np.stack([lo[:, 2], hi[:, 0]], 1)
    cubes["yz1"] = hi[:, 1:]
    normals = rng.normal(size=(npl, 3))
    planes = np.concatenate([normals, rng.uniform(-2.5, -1.5, (npl, 1))], 1)
    return dict(tris=tris, spheres=spheres.astype(np.float32), cubes=cubes,
                planes=planes.astype(np.float32))


def mixed_rays(seed, n=6000, scene=None):
    rays = scenes.incoherent_rays(n, 7000 + seed, tmax=float(NO_HIT))
    if scene is not None:  # a few rays start inside cubes: negative-t cube hits
        c = scene["cubes"][: n // 50]
        inside = np.stack([(c["xy0"][:, 0] + c["z0_x1"][:, 1]) / 2, (c["xy0"][:, 1] + c["yz1"][:, 0]) / 2,
                           (c["z0_x1"][:, 0] + c["yz1"][:, 1]) / 2], 1)
        rays["org"][: len(inside)] = inside
    return rays


def test_oracle_matches_reference_mixed_golden():
    g, sc = golden_scene()
    h, _ = pyoracle.trace_geometry_mixed(g["rays"], **sc)
    miss = g["hit_t"] == NO_HIT
    prim = np.where(miss, 0xFFFFFFFF, g["hit_object"]).astype(np.uint32)
    assert np.array_equal(h["prim"], prim)
    for f, e in (("t", g["hit_t"]), ("u", g["hit_u"]), ("v", g["hit_v"])):
        assert np.array_equal(bits(h[f])[~miss], bits(e)[~miss])
    assert (h["t"][~miss] < 0).any()  # rays starting inside a cube hit it at negative t


@pytest.mark.skipif(not pyoracle.have_reference(), reason="reference shaders not built here")
def test_oracle_matches_reference_mixed_live():
    sc = random_mixed(1)
    rays = mixed_rays(1, 3000, sc)
    r6 = np.concatenate([rays["org"], rays["dir"]], 1)
    ref = pyoracle.ref_trace_geometry(sc["tris"], r6, None, spheres=sc["spheres"], cubes=sc["cubes"],
                                      planes=sc["planes"])
    got, _ = pyoracle.trace_geometry_mixed(rays, **sc)
    miss = ref["hitT"] == NO_HIT
    assert np.array_equal(got["prim"], np.where(miss, 0xFFFFFFFF, ref["object"]).astype(np.uint32))
    assert np.array_equal(bits(got["t"])[~miss], bits(ref["hitT"])[~miss])
    assert np.array_equal(bits(got["u"])[~miss], bits(ref["uv"][:, 0])[~miss])


def test_mixed_bvh_builds_validates_and_roundtrips(tmp_path):
    sc = random_mixed(2)
    b = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    b.validate()
    info = b.info
    assert (info["triangle_count"], info["sphere_count"], info["cube_count"], info["plane_count"]) == (
        3000, 400, 300, 2)
    _, prims = b.arrays()
    assert set(np.unique(prims["pad"])) == {0, 1, 2}
    p = os.path.join(tmp_path, "mixed.bvh")
    b.save(p)
    c = BVH.load(p)
    c.validate()
    assert c.info == info
    bad = sc["spheres"].copy()
    bad[5, 3] = np.inf
    with pytest.raises(IgxrtError):
        BVH.build_mixed(sc["tris"], bad, sc["cubes"], sc["planes"])


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_gpu_mixed_golden(ctx, layout):
    g, sc = golden_scene()
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    got = scene.trace_geometry(g["rays"])
    ctx.set_launch_params(**saved)
    miss = g["hit_t"] == NO_HIT
    prim = np.where(miss, 0xFFFFFFFF, g["hit_object"]).astype(np.uint32)
    assert_mixed_equal(got, prim, g["hit_t"], g["hit_u"], g["hit_v"], len(sc["tris"]), len(sc["spheres"]))


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("seed", [3, 4])
def test_gpu_mixed_matches_oracle(ctx, layout, seed):
    sc = random_mixed(seed)
    rays = mixed_rays(seed, 8000, sc)
    rng = np.random.default_rng(seed)
    prev = rng.integers(0, 3702, len(rays)).astype(np.uint32)
    saved = ctx.launch_params
    ctx.set_launch_params(layout=layout)
    scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    for p in (None, prev):
        expect, flags = pyoracle.trace_geometry_mixed(rays, p, **sc)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        got = scene.trace_geometry(rays, p)
        assert_mixed_equal(got[ok], expect["prim"][ok], expect["t"][ok], expect["u"][ok],
                           expect["v"][ok], len(sc["tris"]), len(sc["spheres"]))
        sh = rays.copy()
        sh["tmax"] = rng.uniform(0.01, 1.0, len(rays)).astype(np.float32)
        occ_e, _ = pyoracle.trace_occlusion_mixed(sh, p, **sc)
        assert np.array_equal(scene.trace_occlusion(sh, p)[ok], occ_e[ok])
    ctx.set_launch_params(**saved)
    assert (expect["t"] < 0).any()  # enclosing cubes were exercised


@pytest.mark.gpu
def test_mixed_scene_fetch_counts(ctx):
    # the G-buffer, shadow, batch and server passes over mixed scenes are
    # checked against the oracle in test_mixed_passes.py
    sc = random_mixed(5, nt=100, ns=10, nc=10, npl=1)
    scene = ctx.create_scene_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    rays = mixed_rays(5, 64)
    nf, pf = ctx.count_fetches(scene, rays)  # GPU-side counts (no host traversal of typed leaves)
    hit = scene.trace_geometry(rays)["prim"] < 120
    assert (nf[hit] >= 1).all() and (pf[hit] >= 1).all()
