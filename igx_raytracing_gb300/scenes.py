"""Seeded synthetic scenes and ray batches for the five benchmark workloads.

No external dataset is involved.  Seeds: base 20261203, stream per workload
and scene = base + 1000 * workload + scene.  Geometry is generated in float64
and rounded once to float32.

Primary rays follow the reference's screen mapping (camera.glsl:72-87,
113-116): centerPixel = (loc + 0.5) / res with y flipped, pos = p0 +
x * (p1 - p0) + y * (p2 - p0), dir = normalize(pos - eye), origin = eye; the
corners p0 (top left), p1 (top right), p2 (bottom left) are those of a
standard pinhole with the given vertical field of view.
"""
from __future__ import annotations

import math

import numpy as np

from ._capi import NO_HIT, RAY_DTYPE, TRIANGLE_DTYPE

BASE_SEED = 20261203


def seed_for(workload: int, scene: int = 0) -> int:
    return BASE_SEED + 1000 * workload + scene


def _tris_from_vertices(v0, v1, v2) -> np.ndarray:
    t = np.zeros(len(v0), dtype=TRIANGLE_DTYPE)
    t["p0"] = np.asarray(v0, dtype=np.float32)
    t["p1"] = np.asarray(v1, dtype=np.float32)
    t["p2"] = np.asarray(v2, dtype=np.float32)
    return t


# --------------------------------------------------------------------------
# Scenes
# --------------------------------------------------------------------------

def heightfield(nx: int = 64, ny: int = 32, seed: int | None = None) -> np.ndarray:
    """nx x ny quads over [0,1]^2, two triangles per quad with a fixed
    diagonal; z = sum of 4 sinusoids (amplitude 0.05, frequency U[1,8])."""
    rng = np.random.default_rng(seed_for(1) if seed is None else seed)
    f = rng.uniform(1.0, 8.0, 4)
    theta = rng.uniform(0.0, 2 * np.pi, 4)
    phi = rng.uniform(0.0, 2 * np.pi, 4)
    xs = np.linspace(0.0, 1.0, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")  # (ny+1, nx+1)
    Z = np.zeros_like(X)
    for k in range(4):
        Z += 0.05 * np.sin(2 * np.pi * f[k] * (X * np.cos(theta[k]) + Y * np.sin(theta[k])) + phi[k])
    P = np.stack([X, Y, Z], axis=-1)
    v00 = P[:-1, :-1].reshape(-1, 3)
    v10 = P[:-1, 1:].reshape(-1, 3)
    v01 = P[1:, :-1].reshape(-1, 3)
    v11 = P[1:, 1:].reshape(-1, 3)
    a0, a1, a2 = v00, v10, v11
    b0, b1, b2 = v00, v11, v01
    v0 = np.stack([a0, b0], axis=1).reshape(-1, 3)
    v1 = np.stack([a1, b1], axis=1).reshape(-1, 3)
    v2 = np.stack([a2, b2], axis=1).reshape(-1, 3)
    return _tris_from_vertices(v0, v1, v2)


def displaced_sphere(nlon: int = 1024, nlat: int = 512, sigma: float = 0.02,
                     seed: int | None = None) -> np.ndarray:
    """Radius-1 lat-long sphere, nlon x nlat quads x 2 triangles, per-vertex
    radius 1 + N(0, sigma^2).  The pole rows keep one vertex per column, so
    no triangle is exactly degenerate."""
    rng = np.random.default_rng(seed_for(2) if seed is None else seed)
    th = np.linspace(0.0, np.pi, nlat + 1)           # polar angle
    ph = np.arange(nlon) * (2 * np.pi / nlon)          # longitude, wraps
    T, PH = np.meshgrid(th, ph, indexing="ij")         # (nlat+1, nlon)
    R = 1.0 + rng.normal(0.0, sigma, T.shape)
    P = np.stack([R * np.sin(T) * np.cos(PH), R * np.sin(T) * np.sin(PH), R * np.cos(T)], axis=-1)
    Pw = np.concatenate([P, P[:, :1]], axis=1)         # wrap the seam column
    v00 = Pw[:-1, :-1].reshape(-1, 3)
    v10 = Pw[:-1, 1:].reshape(-1, 3)
    v01 = Pw[1:, :-1].reshape(-1, 3)
    v11 = Pw[1:, 1:].reshape(-1, 3)
    v0 = np.stack([v00, v00], axis=1).reshape(-1, 3)
    v1 = np.stack([v10, v11], axis=1).reshape(-1, 3)
    v2 = np.stack([v11, v01], axis=1).reshape(-1, 3)
    return _tris_from_vertices(v0, v1, v2)


def random_triangles(n: int, seed: int, mu: float = math.log(0.005), sigma: float = 0.7) -> np.ndarray:
    """n triangles: centroids U[0,1]^3, equilateral with edge ~ LogNormal(mu,
    sigma), uniformly random orientation (normalised Gaussian quaternion)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, (n, 3))
    L = rng.lognormal(mu, sigma, n)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    s3 = math.sqrt(3.0)
    unit = np.array([[1 / s3, 0.0, 0.0], [-0.5 / s3, 0.5, 0.0], [-0.5 / s3, -0.5, 0.0]])
    verts = c[:, None, :] + L[:, None, None] * np.einsum("nij,kj->nki", R, unit)
    return _tris_from_vertices(verts[:, 0], verts[:, 1], verts[:, 2])


# --------------------------------------------------------------------------
# Rays
# --------------------------------------------------------------------------

def pinhole_rays(width: int, height: int, eye, target, up=(0.0, 0.0, 1.0), vfov_deg: float = 60.0,
                 tmax: float = float(NO_HIT), count: int | None = None) -> np.ndarray:
    """Primary rays through pixel centres, in the reference's row order
    (row 0 at the bottom of the image, camera.glsl:115-116)."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    h = math.tan(math.radians(vfov_deg) * 0.5)
    aspect = width / height
    p0 = eye + fwd - aspect * h * right + h * upv   # top left
    p1 = eye + fwd + aspect * h * right + h * upv   # top right
    p2 = eye + fwd - aspect * h * right - h * upv   # bottom left
    ys, xs = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    cx = (xs.reshape(-1) + 0.5) / width
    cy = 1.0 - (ys.reshape(-1) + 0.5) / height
    pos = p0 + cx[:, None] * (p1 - p0) + cy[:, None] * (p2 - p0)
    d = pos - eye
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    if count is not None:
        d = d[:count]
    r = np.zeros(len(d), dtype=RAY_DTYPE)
    r["org"] = eye.astype(np.float32)
    r["dir"] = d.astype(np.float32)
    r["tmin"] = 0.0
    r["tmax"] = tmax
    return r


def camera_record(width: int, height: int, eye, target, up=(0.0, 0.0, 1.0), vfov_deg: float = 60.0,
                  jitter=(0.5, 0.5)) -> np.ndarray:
    """igxrt_camera for the G-buffer pass: the same pinhole corners as
    pinhole_rays (p0 top left, p1 top right, p2 bottom left at distance 1)."""
    from ._capi import CAMERA_DTYPE

    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    h = math.tan(math.radians(vfov_deg) * 0.5)
    aspect = width / height
    c = np.zeros(1, dtype=CAMERA_DTYPE)
    c["eye"] = eye
    c["p0"] = eye + fwd - aspect * h * right + h * upv
    c["p1"] = eye + fwd + aspect * h * right + h * upv
    c["p2"] = eye + fwd - aspect * h * right - h * upv
    c["width"], c["height"] = width, height
    c["jitter_x"], c["jitter_y"] = jitter
    return c


def sphere_dirs(n: int, rng: np.random.Generator) -> np.ndarray:
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def incoherent_rays(n: int, seed: int, tmax: float = float("inf")) -> np.ndarray:
    """Origins U[0,1]^3, directions uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(0.0, 1.0, (n, 3))
    d = sphere_dirs(n, rng)
    r = np.zeros(n, dtype=RAY_DTYPE)
    r["org"] = o.astype(np.float32)
    r["dir"] = d.astype(np.float32)
    r["tmin"] = 0.0
    r["tmax"] = tmax
    return r


def geometric_normals(tris: np.ndarray, prim: np.ndarray) -> np.ndarray:
    t = tris[prim]
    e1 = t["p1"].astype(np.float64) - t["p0"]
    e2 = t["p2"].astype(np.float64) - t["p0"]
    n = np.cross(e1, e2)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def secondary_rays(tris: np.ndarray, primary: np.ndarray, hits: np.ndarray, light, seed: int):
    """For every primary hit: one cosine-weighted bounce about the ray-facing
    geometric normal and one shadow ray toward the point light (tmax = the
    light distance).  Both start at the hit point and exclude the hit
    triangle through prev_hit.  Returns (bounce, shadow, prev)."""
    m = hits["prim"] != 0xFFFFFFFF
    idx = np.nonzero(m)[0]
    prim = hits["prim"][idx]
    o = primary["org"][idx].astype(np.float64)
    d = primary["dir"][idx].astype(np.float64)
    p = o + hits["t"][idx, None].astype(np.float64) * d
    n = geometric_normals(tris, prim)
    flip = np.sum(n * d, axis=1) > 0
    n[flip] = -n[flip]
    rng = np.random.default_rng(seed)
    u1 = rng.uniform(0.0, 1.0, len(idx))
    u2 = rng.uniform(0.0, 2 * np.pi, len(idx))
    r = np.sqrt(u1)
    local = np.stack([r * np.cos(u2), r * np.sin(u2), np.sqrt(np.maximum(0.0, 1 - u1))], axis=1)
    a = np.where(np.abs(n[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t1 = np.cross(n, a)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(n, t1)
    bdir = local[:, 0:1] * t1 + local[:, 1:2] * t2 + local[:, 2:3] * n
    bounce = np.zeros(len(idx), dtype=RAY_DTYPE)
    bounce["org"] = p.astype(np.float32)
    bounce["dir"] = bdir.astype(np.float32)
    bounce["tmin"] = 0.0
    bounce["tmax"] = float(NO_HIT)
    L = np.asarray(light, dtype=np.float64)
    to_l = L - p
    dist = np.linalg.norm(to_l, axis=1)
    shadow = np.zeros(len(idx), dtype=RAY_DTYPE)
    shadow["org"] = p.astype(np.float32)
    shadow["dir"] = (to_l / dist[:, None]).astype(np.float32)
    shadow["tmin"] = 0.0
    shadow["tmax"] = dist.astype(np.float32)
    return bounce, shadow, prim.astype(np.uint32)


# --------------------------------------------------------------------------
# Workload descriptions (sizes of the five configurations)
# --------------------------------------------------------------------------

def workload_small():
    """4,096-triangle heightfield, 256x256 pinhole primaries (closest hit)."""
    tris = heightfield(64, 32, seed_for(1))
    rays = pinhole_rays(256, 256, eye=(0.5, -1.0, 0.5), target=(0.5, 0.5, 0.0))
    return tris, rays


def workload_sphere_primary(width: int = 1920, height: int = 1080, nlon: int = 1024, nlat: int = 512):
    """1,048,576-triangle displaced sphere, 1080p primaries from (0,-3,0)."""
    tris = displaced_sphere(nlon, nlat, 0.02, seed_for(2))
    rays = pinhole_rays(width, height, eye=(0.0, -3.0, 0.0), target=(0.0, 0.0, 0.0))
    return tris, rays


SPHERE_LIGHT = (3.0, 3.0, 3.0)


def workload_incoherent(ntris: int = 2_097_152, nrays: int = 4_194_304, variant: int = 0):
    tris = random_triangles(ntris, seed_for(3, variant))
    rays = incoherent_rays(nrays, seed_for(3, 100 + variant))
    return tris, rays


def workload_mixed(ntris: int = 1_048_576, nspheres: int = 65_536, ncubes: int = 65_536,
                   nplanes: int = 4) -> dict:
    """All four of the reference's primitive types at scale, in the unit cube:
    random triangles as workload_incoherent, spheres with radius log-normal
    around 0.004, axis-aligned cubes with edges log-normal around 0.006, and
    planes bounding the cube from below and the sides (normals pointing in)."""
    from ._capi import CUBE_DTYPE

    rng = np.random.default_rng(seed_for(6))
    tris = random_triangles(ntris, seed_for(6, 1))
    c = rng.uniform(0.0, 1.0, (nspheres, 3))
    r = np.exp(rng.normal(math.log(0.004), 0.5, (nspheres, 1)))
    spheres = np.concatenate([c, r], axis=1).astype(np.float32)
    lo = rng.uniform(0.0, 1.0, (ncubes, 3))
    hi = lo + np.exp(rng.normal(math.log(0.006), 0.5, (ncubes, 3)))
    cubes = np.zeros(ncubes, CUBE_DTYPE)
    cubes["xy0"] = lo[:, :2]
    cubes["z0_x1"] = np.stack([lo[:, 2], hi[:, 0]], axis=1)
    cubes["yz1"] = hi[:, 1:]
    base = [(0.0, 0.0, 1.0, 0.05), (1.0, 0.0, 0.0, 0.05), (-1.0, 0.0, 0.0, -1.05), (0.0, 1.0, 0.0, 0.05)]
    planes = np.asarray(base[:nplanes], dtype=np.float32).reshape(-1, 4)
    return dict(tris=tris, spheres=spheres, cubes=cubes, planes=planes)


def log_uniform_ints(rng: np.random.Generator, lo: int, hi: int, n: int) -> np.ndarray:
    return np.exp(rng.uniform(math.log(lo), math.log(hi), n)).astype(np.int64)


def workload_batch_plan(nscenes: int = 64, tri_range=(1024, 524288), ray_range=(4096, 2_097_152)):
    """Triangle and ray counts of the 64-scene batching workload."""
    rng = np.random.default_rng(seed_for(4))
    return (log_uniform_ints(rng, *tri_range, nscenes), log_uniform_ints(rng, *ray_range, nscenes))


def batch_rays(scene_index: int, n: int) -> np.ndarray:
    """Half pinhole primaries from (0.5,0.5,-1.5) toward the cube centre,
    half uniform-sphere incoherent rays."""
    half = n // 2
    side = max(1, int(math.ceil(math.sqrt(half))))
    prim = pinhole_rays(side, side, eye=(0.5, 0.5, -1.5), target=(0.5, 0.5, 0.5),
                        up=(0.0, 1.0, 0.0), count=half)
    inc = incoherent_rays(n - half, seed_for(4, 500 + scene_index), tmax=float(NO_HIT))
    return np.concatenate([prim, inc])
