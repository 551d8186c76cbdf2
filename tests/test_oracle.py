"""The oracle restatement, pinned against the reference's own traversal code.

The golden fixtures were produced by igx_raytracing's primitive.glsl +
trace.glsl compiled for the host (tests/golden/make_golden.py); the
restatement in oracle/trace_oracle.c must reproduce them bit for bit.
"""
import numpy as np
import pytest

from conftest import (GOLDEN_CASES, NO_HIT, assert_hits_equal, bits, closest_rays, load_golden,
                      occlusion_rays)
from igx_raytracing_gb300 import scenes
from igx_raytracing_gb300._capi import RAY_DTYPE, TRIANGLE_DTYPE
from oracle import pyoracle


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_restatement_matches_reference_closest(case):
    g = load_golden(case)
    # The restatement reproduces the reference even where the linear loop
    # accepts a NaN t (rays lying in a triangle's plane, edge_cases only).
    got, flags = pyoracle.trace_geometry(g["tris"], closest_rays(g), g["prev"])
    assert case == "edge_cases" or not (flags & pyoracle.EVENT_NAN_T).any()
    assert_hits_equal(got, g["hit_prim"], g["hit_t"], g["hit_u"], g["hit_v"], case)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_restatement_matches_reference_occlusion(case):
    g = load_golden(case)
    got, _ = pyoracle.trace_occlusion(g["tris"], occlusion_rays(g), g["prev"])
    assert np.array_equal(got, g["occluded"])


def _ray(o, d, tmin=0.0, tmax=float(NO_HIT)):
    r = np.zeros(1, dtype=RAY_DTYPE)
    r["org"], r["dir"], r["tmin"], r["tmax"] = o, d, tmin, tmax
    return r


def _quad_z(z, n_copies=1):
    t = np.zeros(2 * n_copies, dtype=TRIANGLE_DTYPE)
    for k in range(n_copies):
        t[2 * k]["p0"], t[2 * k]["p1"], t[2 * k]["p2"] = (0, 0, z), (1, 0, z), (1, 1, z)
        t[2 * k + 1]["p0"], t[2 * k + 1]["p1"], t[2 * k + 1]["p2"] = (0, 0, z), (1, 1, z), (0, 1, z)
    return t


def test_known_answer_axis_ray():
    # p0=(0,0,5), e1=(1,0,0), e2=(1,1,0); ray (0.75,0.25,0)+t(0,0,1):
    # h = d x e2 = (-1, 1, 0), a = -1, f = -1, s = (0.75,0.25,-5),
    # u = -(-0.75+0.25) = 0.5, q = s x e1 = (0,-5,-0.25), v = 0.25, t = 5.
    tris = _quad_z(5.0)
    h, _ = pyoracle.trace_geometry(tris, _ray((0.75, 0.25, 0), (0, 0, 1)))
    assert h["prim"][0] == 0 and h["t"][0] == 5.0 and h["u"][0] == 0.5 and h["v"][0] == 0.25


def test_known_answer_tie_lowest_index():
    tris = _quad_z(5.0, n_copies=3)  # triangles 0,2,4 identical; 1,3,5 identical
    h, _ = pyoracle.trace_geometry(tris, _ray((0.75, 0.25, 0), (0, 0, 1)))
    assert h["prim"][0] == 0
    h, _ = pyoracle.trace_geometry(tris, _ray((0.25, 0.75, 0), (0, 0, 1)))
    assert h["prim"][0] == 1
    # on the shared diagonal both triangles accept at t = 5: index 0 wins
    h, _ = pyoracle.trace_geometry(tris, _ray((0.5, 0.5, 0), (0, 0, 1)))
    assert h["prim"][0] == 0


def test_known_answer_prev_hit_and_interval():
    tris = _quad_z(5.0, n_copies=2)
    r = _ray((0.75, 0.25, 0), (0, 0, 1))
    h, _ = pyoracle.trace_geometry(tris, r, prev=np.array([0], np.uint32))
    assert h["prim"][0] == 2  # the duplicate behind the excluded one
    r5 = _ray((0.75, 0.25, 0), (0, 0, 1), tmax=5.0)
    h, _ = pyoracle.trace_geometry(tris, r5)
    assert h["prim"][0] == 0xFFFFFFFF and h["t"][0] == NO_HIT
    on = _ray((0.75, 0.25, 5), (0, 0, 1))  # origin on the plane: t == 0 rejected
    h, _ = pyoracle.trace_geometry(tris, on)
    assert h["prim"][0] == 0xFFFFFFFF
    occ, _ = pyoracle.trace_occlusion(tris, _ray((0.75, 0.25, 0), (0, 0, 1), tmax=5.0))
    assert occ[0] == 0
    occ, _ = pyoracle.trace_occlusion(tris, _ray((0.75, 0.25, 0), (0, 0, 1), tmax=5.5))
    assert occ[0] == 1


def test_reintersect_f64_agrees_on_simple_hit():
    tris = _quad_z(5.0)
    ok, t, u, v = pyoracle.reintersect_f64(_ray((0.75, 0.25, 0), (0, 0, 1))[0], tris[0])
    assert ok and t == 5.0 and u == 0.5 and v == 0.25


@pytest.mark.skipif(not pyoracle.have_reference(), reason="reference shaders not built here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_restatement_matches_reference_live(seed):
    import math

    tris = scenes.random_triangles(512, 9000 + seed, mu=math.log(0.08))
    rays = scenes.incoherent_rays(2048, 9100 + seed, tmax=float(NO_HIT))
    rng = np.random.default_rng(seed)
    prev = rng.integers(0, 600, len(rays)).astype(np.uint32)
    r6 = np.concatenate([rays["org"], rays["dir"]], axis=1)
    ref = pyoracle.ref_trace_geometry(tris, r6, prev)
    got, _ = pyoracle.trace_geometry(tris, rays, prev)
    miss = ref["hitT"] == NO_HIT
    prim = np.where(miss, 0xFFFFFFFF, ref["object"]).astype(np.uint32)
    assert_hits_equal(got, prim, ref["hitT"], ref["uv"][:, 0], ref["uv"][:, 1], f"seed {seed}")
    md = rng.uniform(0.01, 0.6, len(rays)).astype(np.float32)
    sh = rays.copy()
    sh["tmax"] = md
    assert np.array_equal(pyoracle.trace_occlusion(tris, sh, prev)[0],
                          pyoracle.ref_trace_occlusion(tris, r6, md, prev))


def test_golden_fixtures_are_bitwise_stable():
    # guards against accidental regeneration with other semantics
    g = load_golden("edge_cases")
    assert len(g["tris"]) == 10 and len(g["rays"]) == 69
    hit = g["hit_prim"] != 0xFFFFFFFF
    assert set(np.unique(g["hit_prim"][hit])) <= set(range(10))
    assert (bits(g["hit_t"][~hit]) == bits(np.float32(NO_HIT))).all()


def test_disagreements_are_reintersected_in_f64(capsys):
    """A planted disagreement (the oracle's own answer with one primitive id
    changed, on the CPU) fails the parity check and logs the binary64
    re-intersection of both candidates."""
    from conftest import assert_hits_equal

    g = load_golden("heightfield")
    rays = g["rays"].copy()
    rays["tmin"] = 0.0
    rays["tmax"] = NO_HIT
    got, _ = pyoracle.trace_geometry(g["tris"], rays)
    i = int(np.nonzero(got["prim"] != 0xFFFFFFFF)[0][0])
    planted = got.copy()
    planted["prim"][i] = (planted["prim"][i] + 1) % len(g["tris"])
    with pytest.raises(AssertionError):
        assert_hits_equal(planted, got["prim"], got["t"], got["u"], got["v"], "planted",
                          rays=rays, tris=g["tris"])
    out = capsys.readouterr().out
    assert f"ray {i}:" in out and "f64 hit" in out
