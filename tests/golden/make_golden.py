"""Generates the golden fixtures in this directory from the reference's own
traversal code.

The expected values come from oracle/_ref/libigxref.so: igx_raytracing's
res/shaders/primitive.glsl and trace.glsl compiled for the host
(oracle/Makefile, target `ref`).  Building that library needs the reference
checkout, so this script runs where the checkout is; the .npz files it writes
are committed and checked everywhere.

    python tests/golden/make_golden.py [REFERENCE_CHECKOUT]

(the checkout defaults to the IGXRT_REFERENCE environment variable).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from igx_raytracing_gb300 import scenes  # noqa: E402
from igx_raytracing_gb300._capi import NO_HIT, RAY_DTYPE, TRIANGLE_DTYPE  # noqa: E402
from oracle import pyoracle  # noqa: E402

CUBE_DTYPE = np.dtype([("xy0", "<f4", (2,)), ("z0_x1", "<f4", (2,)), ("yz1", "<f4", (2,))])


def rays6(r: np.ndarray) -> np.ndarray:
    return np.concatenate([r["org"], r["dir"]], axis=1).astype(np.float32)


def tri(p0, p1, p2) -> np.ndarray:
    t = np.zeros(1, dtype=TRIANGLE_DTYPE)
    t["p0"], t["p1"], t["p2"] = p0, p1, p2
    return t


def ray(o, d, tmax=float(NO_HIT)) -> np.ndarray:
    r = np.zeros(1, dtype=RAY_DTYPE)
    r["org"], r["dir"], r["tmin"], r["tmax"] = o, d, 0.0, tmax
    return r


def edge_case_scene():
    """Hand-built triangles and rays for the reference's edge behaviour:
    equal-t ties (lowest index wins), shared edges and vertices (u+v == 1,
    u == 0), t <= 0 rejection, prevHit exclusion, rays parallel to a
    triangle, axis-aligned directions, and the NielsScene triangles
    (test/scene/niels_scene.cpp:26-42)."""
    T = []
    # 0-2: NielsScene's triangles
    T.append(tri((1, 1, 0), (-1, 1, 0), (1, 0, 1)))
    T.append(tri((-1, 4, 0), (1, 4, 0), (1, 3, 1)))
    T.append(tri((-1, 7, 0), (1, 7, 0), (1, 5, 1)))
    # 3-6: a unit quad at z = 5 as two triangles sharing the diagonal, plus an
    # exact duplicate of each (ties at equal t: the lower index must win)
    qa = tri((0, 0, 5), (1, 0, 5), (1, 1, 5))
    qb = tri((0, 0, 5), (1, 1, 5), (0, 1, 5))
    T += [qb, qa, qb, qa]
    # 7: triangle whose plane contains the ray origin (t == 0 rejected)
    T.append(tri((-0.5, -0.5, 0), (2, -0.5, 0), (-0.5, 2, 0)))
    # 8: a far triangle behind the quad
    T.append(tri((-1, -1, 9), (3, -1, 9), (-1, 3, 9)))
    # 9: a vertical triangle (plane x = 0.25)
    T.append(tri((0.25, -1, -1), (0.25, 3, -1), (0.25, -1, 12)))
    tris = np.concatenate(T)

    R = []
    for x, y in [(0.25, 0.75), (0.75, 0.25), (0.5, 0.5), (0.0, 0.0), (1.0, 1.0), (1.0, 0.0),
                 (0.0, 1.0), (0.3, 0.3), (0.999, 0.001), (1.0, 0.5), (0.5, 1.0)]:
        R.append(ray((x, y, 0), (0, 0, 1)))          # through the quad, diagonal, corners, edges
        R.append(ray((x, y, 0), (0, 0, 1), 5.0))      # tmax == t: must miss the quad
        R.append(ray((x, y, 0), (0, 0, 1), 5.0001))
        R.append(ray((x, y, 10), (0, 0, -1)))         # from above
        R.append(ray((x, y, 5), (0, 0, 1)))           # origin on the quad: t == 0 rejected
    R.append(ray((0.5, 0.5, 5), (1, 0, 0)))           # in the quad's plane (parallel)
    R.append(ray((0.5, 0.5, 4), (1, 0, 0)))           # parallel, off plane
    R.append(ray((0.25, 0.5, 2), (0, 1, 0)))          # inside the vertical triangle's plane
    R.append(ray((-1, 0.5, 2), (1, 0, 0)))            # hits the vertical triangle
    R.append(ray((0, 0.5, 0.5), (0, 1, 0)))           # NielsScene triangles along +y
    R.append(ray((0.5, -2, 0.25), (0, 1, 0.05)))
    R.append(ray((0.9, 0, 0.2), (0, 1, 0)))
    R.append(ray((2, 2, 2), (-1, -1, -1)))
    R.append(ray((0.5, 0.5, -3), (0, 0, 1)))
    R.append(ray((0.5, 0.5, -3), (0, 0, -1)))         # away from everything
    R.append(ray((0.5, 0.5, 20), (0, 0, -1), 10.9))   # stops before the far triangle
    R.append(ray((0.5, 0.5, 20), (0, 0, -1), 11.1))
    R.append(ray((0.5, 0.5, 3), (1e-30, 0, 1)))       # tiny direction component
    R.append(ray((0.5, 0.5, 3), (-0.0, 0.0, 1)))
    rays = np.concatenate(R)
    # prevHit: exclude the lowest duplicate on some rays, nothing on others
    prev = np.full(len(rays), 0xFFFFFFFF, dtype=np.uint32)
    prev[0::3] = 3
    prev[1::5] = 4
    prev[2::7] = 8
    return tris, rays, prev


def niels_mixed():
    """NielsScene's primitives (test/scene/niels_scene.cpp:21-47): 3
    triangles, 4 spheres (centre, radius), 2 cubes (min, max), 1 plane."""
    tris = edge_case_scene()[0][:3].copy()
    spheres = np.array([[0, 1, 5, 1], [0, 1, -5, 1], [3, 1, 0, 1], [0, 6, 0, 1]], dtype=np.float32)
    cubes = np.zeros(2, dtype=CUBE_DTYPE)
    for i, (lo, hi) in enumerate([((0, 0, 0), (1, 1, 1)), ((-2, 0, -2), (-1, 1, -1))]):
        cubes[i]["xy0"] = lo[:2]
        cubes[i]["z0_x1"] = (lo[2], hi[0])
        cubes[i]["yz1"] = hi[1:]
    planes = np.array([[0, 1, 0, 0]], dtype=np.float32)
    rng = np.random.default_rng(scenes.seed_for(9))
    n = 2048
    o = rng.uniform(-6, 6, (n, 3)) + np.array([0, 3, 0])
    d = scenes.sphere_dirs(n, rng)
    rays = np.zeros(n, dtype=RAY_DTYPE)
    rays["org"], rays["dir"], rays["tmax"] = o, d, float(NO_HIT)
    return tris, spheres, cubes, planes, rays


def main() -> None:
    pyoracle.build(with_reference=True, reference=sys.argv[1] if len(sys.argv) > 1 else None)
    if not pyoracle.have_reference():
        raise SystemExit("oracle/_ref/libigxref.so is not built: the reference checkout is needed")

    out = {}
    # 1. the small heightfield workload, every 8th primary ray
    tris, rays = scenes.workload_small()
    rays = rays[::8].copy()
    rng = np.random.default_rng(scenes.seed_for(1, 7))
    out["heightfield"] = (tris, rays, None, rng.uniform(0.5, 3.0, len(rays)).astype(np.float32))

    # 2. hand-built edge cases
    et, er, ep = edge_case_scene()
    out["edge_cases"] = (et, er, ep, np.where(er["tmax"] < NO_HIT, er["tmax"], NO_HIT).astype(np.float32))

    # 3. small random-triangle scene with incoherent rays and prevHit
    rt = scenes.random_triangles(2048, scenes.seed_for(3, 77), mu=math.log(0.05), sigma=0.7)
    rr = scenes.incoherent_rays(4096, scenes.seed_for(3, 78), tmax=float(NO_HIT))
    rp = np.full(len(rr), 0xFFFFFFFF, dtype=np.uint32)
    pick = rng.integers(0, len(rr), 1024)
    rp[pick] = rng.integers(0, len(rt), 1024).astype(np.uint32)
    out["random_small"] = (rt, rr, rp, rng.uniform(0.01, 0.5, len(rr)).astype(np.float32))

    for name, (t, r, p, maxd) in out.items():
        h = pyoracle.ref_trace_geometry(t, rays6(r), p)
        occ = pyoracle.ref_trace_occlusion(t, rays6(r), maxd, p)
        miss = h["hitT"] == NO_HIT
        prim = np.where(miss, np.uint32(0xFFFFFFFF), h["object"]).astype(np.uint32)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            tris=t, rays=r, prev=p if p is not None else np.full(len(r), 0xFFFFFFFF, np.uint32),
            hit_t=h["hitT"], hit_u=h["uv"][:, 0], hit_v=h["uv"][:, 1], hit_prim=prim,
            geometry_normal=h["geometryNormal"], object_normal=h["objectNormal"],
            max_dist=maxd, occluded=occ)
        print(f"{name}: {len(t)} triangles, {len(r)} rays, {int((~miss).sum())} hits, "
              f"{int(occ.sum())} occluded")

    # 4. mixed primitives (spheres, cubes, planes) in the reference's index order
    t, s, c, pl, r = niels_mixed()
    h = pyoracle.ref_trace_geometry(t, rays6(r), None, spheres=s, cubes=c, planes=pl)
    np.savez_compressed(os.path.join(HERE, "niels_mixed.npz"), tris=t, spheres=s, cubes=c, planes=pl,
                        rays=r, hit_t=h["hitT"], hit_u=h["uv"][:, 0], hit_v=h["uv"][:, 1],
                        hit_object=h["object"], geometry_normal=h["geometryNormal"],
                        object_normal=h["objectNormal"])
    print(f"niels_mixed: {len(r)} rays, {int((h['hitT'] < NO_HIT).sum())} hits")

    # 4b. the primary pass over the mixed scene: raygen.comp's two images
    #     (:39-51) from the reference's traceGeometry on the camera's rays
    #     (trace.glsl:48-63: an interpolated vertex normal for triangles, the
    #     geometry normal for spheres, cubes and planes)
    cam = scenes.camera_record(96, 64, eye=(7.0, 11.0, 6.0), target=(0.0, 2.5, 0.0), vfov_deg=70.0)
    crays = pyoracle.camera_rays(cam)
    h = pyoracle.ref_trace_geometry(t, rays6(crays), None, spheres=s, cubes=c, planes=pl)
    hit = h["hitT"] != NO_HIT
    d = crays["dir"].astype(np.float32)
    do = np.zeros((len(crays), 4), np.float32)
    do[:, :3] = np.where(hit[:, None], d * h["hitT"][:, None].astype(np.float32), d)
    do[:, 3] = np.where(hit, h["object"], np.uint32(0xFFFFFFFF)).astype(np.uint32).view(np.float32)
    uvn = np.zeros((len(crays), 4), np.float32)
    enc = pyoracle.ref_encode_normal(h["objectNormal"])
    uvn[:, :2] = np.where(hit[:, None], h["uv"], 0.0)
    uvn[:, 2:] = np.where(hit[:, None], enc, 0).astype(np.uint32).view(np.float32)
    np.savez_compressed(os.path.join(HERE, "niels_gbuffer.npz"), tris=t, spheres=s, cubes=c, planes=pl,
                        camera=cam, dir_object=do.reshape(64, 96, 4), uv_normal=uvn.reshape(64, 96, 4))
    kinds = np.searchsorted([len(t), len(t) + len(s), len(t) + len(s) + len(c)], h["object"][hit], "right")
    print(f"niels_gbuffer: {int(hit.sum())} hits of {len(crays)} pixels, per kind "
          f"{np.bincount(kinds, minlength=4).tolist()} (triangle, sphere, cube, plane)")

    # 5. packed vertex normals: decodeSpheremap, interpolate and encodeNormal
    rng2 = np.random.default_rng(scenes.seed_for(9, 1))

    def packed(n):
        rad = np.sqrt(rng2.uniform(0, 1, n)) * 0.999
        ang = rng2.uniform(0, 2 * np.pi, n)
        hx = (rad * np.cos(ang)).astype(np.float16).view(np.uint16).astype(np.uint32)
        hy = (rad * np.sin(ang)).astype(np.float16).view(np.uint16).astype(np.uint32)
        return (hx | (hy << 16)).astype(np.uint32)

    nt = scenes.random_triangles(1024, scenes.seed_for(3, 79), mu=math.log(0.06))
    for f in ("n0", "n1", "n2"):
        nt[f] = packed(len(nt))
    nr = scenes.incoherent_rays(4096, scenes.seed_for(3, 80), tmax=float(NO_HIT))
    h = pyoracle.ref_trace_geometry(nt, rays6(nr))
    miss = h["hitT"] == NO_HIT
    dec_in = packed(2048)
    enc_in = rng2.normal(size=(2048, 3)).astype(np.float32) * rng2.uniform(0.2, 3.0, (2048, 1)).astype(np.float32)
    np.savez_compressed(
        os.path.join(HERE, "normals.npz"), tris=nt, rays=nr, hit_t=h["hitT"], hit_u=h["uv"][:, 0],
        hit_v=h["uv"][:, 1], hit_prim=np.where(miss, np.uint32(0xFFFFFFFF), h["object"]).astype(np.uint32),
        object_normal=h["objectNormal"], dec_in=dec_in, dec_out=pyoracle.ref_decode_spheremap(dec_in),
        enc_in=enc_in, enc_out=pyoracle.ref_encode_normal(enc_in))
    print(f"normals: {len(nr)} rays, {int((~miss).sum())} hits")


if __name__ == "__main__":
    main()
