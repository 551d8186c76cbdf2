"""ctypes front end of the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
benchmark's CPU-baseline leg; never by the engine package.

  liboracle.so      CPU restatement of traceGeometry / traceOcclusion
                    (brute force) and the CPU BVH traversal baseline.
  _ref/libigxref.so the reference's own primitive.glsl + trace.glsl compiled
                    for the host (present only where the reference checkout
                    was available to generate it).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libigxref.so")
REF_GEN = os.path.join(ORACLE_DIR, "_ref", "gen")
# The reference checkout, needed only to (re)generate _ref/: taken from the
# IGXRT_REFERENCE environment variable (no default location).
REFERENCE_ENV = "IGXRT_REFERENCE"

EVENT_NAN_T = 1
EVENT_ZERO_DET = 2

RAY_DTYPE = np.dtype([("org", "<f4", (3,)), ("tmin", "<f4"), ("dir", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])
REF_HIT_DTYPE = np.dtype([("rayDir", "<f4", (3,)), ("hitT", "<f4"), ("uv", "<f4", (2,)),
                          ("object", "<u4"), ("geometryNormal", "<f4", (3,)),
                          ("objectNormal", "<f4", (3,))])


def build(with_reference: bool = True, reference: str | None = None) -> None:
    """Builds liboracle.so, and _ref/libigxref.so when its sources are
    available: the reference checkout `reference` (default: the
    IGXRT_REFERENCE environment variable), or an _ref/gen/ left by an earlier
    build."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)
    reference = reference or os.environ.get(REFERENCE_ENV) or ""
    have_checkout = bool(reference) and os.path.exists(os.path.join(reference, "res", "shaders", "trace.glsl"))
    if with_reference and (have_checkout or os.path.isdir(REF_GEN)):
        cmd = ["make", "-s", "-C", ORACLE_DIR, "ref"]
        if have_checkout:
            cmd.append(f"REF={reference}")
        subprocess.run(cmd, check=True)


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_reference=False)
        h = C.CDLL(LIB)
        vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        h.orc_trace_geometry.argtypes = [vp, u32, vp, vp, u32, vp, vp, i32]
        h.orc_trace_geometry.restype = None
        h.orc_trace_occlusion.argtypes = [vp, u32, vp, vp, u32, vp, vp, i32]
        h.orc_trace_occlusion.restype = None
        h.orc_reintersect_f64.argtypes = [vp, vp, vp, vp, vp]
        h.orc_reintersect_f64.restype = i32
        h.orc_bvh_trace.argtypes = [u32, vp, u64, vp, u64, vp, vp, u32, u32, vp, vp, vp, vp, i32]
        h.orc_bvh_trace.restype = i32
        h.orc_shadow_mask.argtypes = [vp, u32, vp, vp, u32, u32, u32, vp, vp, i32]
        h.orc_shadow_mask.restype = None
        h.orc_gbuffer.argtypes = [vp, u32, vp, vp, vp, vp, i32]
        h.orc_gbuffer.restype = None
        h.orc_decode_spheremap.argtypes = [u32, vp]
        h.orc_decode_spheremap.restype = None
        h.orc_encode_normal.argtypes = [vp, vp]
        h.orc_encode_normal.restype = None
        h.orc_trace_geometry_mixed.argtypes = [vp, vp, vp, u32, vp, vp, i32]
        h.orc_trace_geometry_mixed.restype = None
        h.orc_trace_occlusion_mixed.argtypes = [vp, vp, vp, u32, vp, vp, i32]
        h.orc_trace_occlusion_mixed.restype = None
        h.orc_camera_rays.argtypes = [vp, vp]
        h.orc_camera_rays.restype = None
        h.orc_gbuffer_mixed.argtypes = [vp, vp, vp, vp, vp, i32]
        h.orc_gbuffer_mixed.restype = None
        h.orc_shadow_mask_mixed.argtypes = [vp, vp, vp, u32, u32, u32, vp, vp, i32]
        h.orc_shadow_mask_mixed.restype = None
        h.orc_bvh_build.argtypes = [vp, u32, vp, vp]
        h.orc_bvh_build.restype = C.c_int64
        h.orc_hardware_threads.argtypes = []
        h.orc_hardware_threads.restype = i32
        _lib = h
    return _lib


def have_reference() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is None:
        h = C.CDLL(REF_LIB)
        vp, u32 = C.c_void_p, C.c_uint32
        h.igxref_trace_geometry.argtypes = [vp, vp, vp, u32, vp]
        h.igxref_trace_geometry.restype = None
        h.igxref_trace_occlusion.argtypes = [vp, vp, vp, vp, u32, vp]
        h.igxref_trace_occlusion.restype = None
        h.igxref_encode_normal.argtypes = [vp, u32, vp]
        h.igxref_encode_normal.restype = None
        h.igxref_decode_spheremap.argtypes = [vp, u32, vp]
        h.igxref_decode_spheremap.restype = None
        _ref = h
    return _ref


def hardware_threads() -> int:
    return lib().orc_hardware_threads()


def _ptr(a):
    return None if a is None else a.ctypes.data


def _prev(prev, n):
    if prev is None:
        return None
    p = np.ascontiguousarray(prev, dtype=np.uint32)
    assert len(p) == n
    return p


def trace_geometry(tris: np.ndarray, rays: np.ndarray, prev=None, threads: int = 0):
    """Brute-force closest hits + per-ray event flags."""
    rays = np.ascontiguousarray(rays)
    tris = np.ascontiguousarray(tris)
    n = len(rays)
    out = np.zeros(n, dtype=HIT_DTYPE)
    flags = np.zeros(n, dtype=np.uint32)
    p = _prev(prev, n)
    if n:
        lib().orc_trace_geometry(_ptr(tris), len(tris), _ptr(rays), _ptr(p), n, _ptr(out),
                                 _ptr(flags), threads)
    return out, flags


def trace_occlusion(tris: np.ndarray, rays: np.ndarray, prev=None, threads: int = 0):
    rays = np.ascontiguousarray(rays)
    tris = np.ascontiguousarray(tris)
    n = len(rays)
    out = np.zeros(n, dtype=np.uint32)
    flags = np.zeros(n, dtype=np.uint32)
    p = _prev(prev, n)
    if n:
        lib().orc_trace_occlusion(_ptr(tris), len(tris), _ptr(rays), _ptr(p), n, _ptr(out),
                                  _ptr(flags), threads)
    return out, flags


def shadow_mask(tris, rays, object_, width: int, height: int, samples: int, threads: int = 0):
    """The reference's shadow pass (brute force) packed into ballot words."""
    tris = np.ascontiguousarray(tris)
    rays = np.ascontiguousarray(rays)
    obj = np.ascontiguousarray(object_, dtype=np.uint32)
    assert len(rays) == width * height * samples and len(obj) == width * height
    words = ((width + 15) // 16) * ((height + 1) // 2) * samples
    mask = np.zeros(words, dtype=np.uint32)
    flags = np.zeros(len(rays), dtype=np.uint32)
    lib().orc_shadow_mask(_ptr(tris), len(tris), _ptr(rays), _ptr(obj), width, height, samples,
                          _ptr(mask), _ptr(flags), threads)
    return mask, flags


CAMERA_DTYPE = np.dtype([("eye", "<f4", (3,)), ("width", "<u4"), ("p0", "<f4", (3,)),
                         ("height", "<u4"), ("p1", "<f4", (3,)), ("jitter_x", "<f4"),
                         ("p2", "<f4", (3,)), ("jitter_y", "<f4")])


def gbuffer(tris, camera: np.ndarray, threads: int = 0, uv_fill: float = 0.0):
    """The reference's primary pass: (dir_object, uv_normal, flags), images
    (height, width, 4) float32; uv_normal keeps uv_fill where rays miss."""
    tris = np.ascontiguousarray(tris)
    cam = np.ascontiguousarray(camera, dtype=CAMERA_DTYPE).reshape(1)
    w, h = int(cam["width"][0]), int(cam["height"][0])
    do = np.zeros((h, w, 4), dtype=np.float32)
    uv = np.full((h, w, 4), uv_fill, dtype=np.float32)
    flags = np.zeros(w * h, dtype=np.uint32)
    lib().orc_gbuffer(_ptr(tris), len(tris), _ptr(cam), _ptr(do), _ptr(uv), _ptr(flags), threads)
    return do, uv, flags


def decode_spheremap(packed) -> np.ndarray:
    out = np.zeros((len(packed), 3), dtype=np.float32)
    tmp = np.zeros(3, dtype=np.float32)
    for i, p in enumerate(np.asarray(packed, dtype=np.uint32)):
        lib().orc_decode_spheremap(int(p), _ptr(tmp))
        out[i] = tmp
    return out


def encode_normal(normals) -> np.ndarray:
    n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((len(n), 2), dtype=np.uint32)
    tmp = np.zeros(2, dtype=np.uint32)
    for i in range(len(n)):
        row = np.ascontiguousarray(n[i])
        lib().orc_encode_normal(_ptr(row), _ptr(tmp))
        out[i] = tmp
    return out


def ref_decode_spheremap(packed) -> np.ndarray:
    p = np.ascontiguousarray(packed, dtype=np.uint32)
    out = np.zeros((len(p), 3), dtype=np.float32)
    ref_lib().igxref_decode_spheremap(_ptr(p), len(p), _ptr(out))
    return out


def ref_encode_normal(normals) -> np.ndarray:
    n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((len(n), 2), dtype=np.uint32)
    ref_lib().igxref_encode_normal(_ptr(n), len(n), _ptr(out))
    return out


class _SceneDesc(C.Structure):
    _fields_ = [("triangles", C.c_void_p), ("triangle_count", C.c_uint32),
                ("sphere_count", C.c_uint32), ("spheres", C.c_void_p), ("cubes", C.c_void_p),
                ("cube_count", C.c_uint32), ("plane_count", C.c_uint32), ("planes", C.c_void_p)]


def scene_desc(tris=None, spheres=None, cubes=None, planes=None):
    """An igxrt_scene_desc over numpy arrays (kept alive in the returned tuple)."""
    keep = [None if a is None else np.ascontiguousarray(a) for a in (tris, spheres, cubes, planes)]
    d = _SceneDesc()
    d.triangles, d.triangle_count = _ptr(keep[0]), 0 if keep[0] is None else len(keep[0])
    d.spheres, d.sphere_count = _ptr(keep[1]), 0 if keep[1] is None else len(keep[1])
    d.cubes, d.cube_count = _ptr(keep[2]), 0 if keep[2] is None else len(keep[2])
    d.planes, d.plane_count = _ptr(keep[3]), 0 if keep[3] is None else len(keep[3])
    return d, keep


def trace_geometry_mixed(rays, prev=None, tris=None, spheres=None, cubes=None, planes=None,
                         threads: int = 0):
    d, keep = scene_desc(tris, spheres, cubes, planes)
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    out = np.zeros(n, dtype=HIT_DTYPE)
    flags = np.zeros(n, dtype=np.uint32)
    p = _prev(prev, n)
    if n:
        lib().orc_trace_geometry_mixed(C.addressof(d), _ptr(rays), _ptr(p), n, _ptr(out),
                                       _ptr(flags), threads)
    return out, flags


def trace_occlusion_mixed(rays, prev=None, tris=None, spheres=None, cubes=None, planes=None,
                          threads: int = 0):
    d, keep = scene_desc(tris, spheres, cubes, planes)
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    out = np.zeros(n, dtype=np.uint32)
    flags = np.zeros(n, dtype=np.uint32)
    p = _prev(prev, n)
    if n:
        lib().orc_trace_occlusion_mixed(C.addressof(d), _ptr(rays), _ptr(p), n, _ptr(out),
                                        _ptr(flags), threads)
    return out, flags


def camera_rays(camera: np.ndarray) -> np.ndarray:
    """The oracle's primary rays of a camera (calculateScreen), pixel order."""
    cam = np.ascontiguousarray(camera, dtype=CAMERA_DTYPE).reshape(1)
    rays = np.zeros(int(cam["width"][0]) * int(cam["height"][0]), dtype=RAY_DTYPE)
    lib().orc_camera_rays(_ptr(cam), _ptr(rays))
    return rays


def gbuffer_mixed(camera: np.ndarray, tris=None, spheres=None, cubes=None, planes=None,
                  threads: int = 0, uv_fill: float = 0.0):
    """The reference's primary pass over a mixed scene (brute force):
    (dir_object, uv_normal, flags) as gbuffer()."""
    d, keep = scene_desc(tris, spheres, cubes, planes)
    cam = np.ascontiguousarray(camera, dtype=CAMERA_DTYPE).reshape(1)
    w, h = int(cam["width"][0]), int(cam["height"][0])
    do = np.zeros((h, w, 4), dtype=np.float32)
    uv = np.full((h, w, 4), uv_fill, dtype=np.float32)
    flags = np.zeros(w * h, dtype=np.uint32)
    lib().orc_gbuffer_mixed(C.addressof(d), _ptr(cam), _ptr(do), _ptr(uv), _ptr(flags), threads)
    return do, uv, flags


def shadow_mask_mixed(rays, object_, width: int, height: int, samples: int, tris=None, spheres=None,
                      cubes=None, planes=None, threads: int = 0):
    """The reference's shadow pass over a mixed scene, packed as shadow_mask()."""
    d, keep = scene_desc(tris, spheres, cubes, planes)
    rays = np.ascontiguousarray(rays)
    obj = np.ascontiguousarray(object_, dtype=np.uint32)
    assert len(rays) == width * height * samples and len(obj) == width * height
    words = ((width + 15) // 16) * ((height + 1) // 2) * samples
    mask = np.zeros(words, dtype=np.uint32)
    flags = np.zeros(len(rays), dtype=np.uint32)
    lib().orc_shadow_mask_mixed(C.addressof(d), _ptr(rays), _ptr(obj), width, height, samples,
                                _ptr(mask), _ptr(flags), threads)
    return mask, flags


def reintersect_f64(ray: np.ndarray, tri: np.ndarray):
    t, u, v = C.c_double(), C.c_double(), C.c_double()
    r = np.ascontiguousarray(ray)
    tr = np.ascontiguousarray(tri)
    ok = lib().orc_reintersect_f64(_ptr(r), _ptr(tr), C.byref(t), C.byref(u), C.byref(v))
    return bool(ok), t.value, u.value, v.value


def bvh_trace(layout: int, nodes: np.ndarray, prims: np.ndarray, rays: np.ndarray, prev=None,
              mode: int = 0, threads: int = 0, counts: bool = False):
    """CPU BVH traversal over the engine's exported arrays (closest or any)."""
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    hits = np.zeros(n, dtype=HIT_DTYPE) if mode == 0 else None
    occ = np.zeros(n, dtype=np.uint32) if mode == 1 else None
    nf = np.zeros(n, dtype=np.uint32) if counts else None
    pf = np.zeros(n, dtype=np.uint32) if counts else None
    p = _prev(prev, n)
    rc = 0
    if n:
        rc = lib().orc_bvh_trace(layout, _ptr(nodes), len(nodes), _ptr(prims), len(prims),
                                 _ptr(rays), _ptr(p), n, mode, _ptr(hits), _ptr(occ), _ptr(nf),
                                 _ptr(pf), threads)
    if rc != 0:
        raise RuntimeError("oracle BVH traversal met a malformed BVH")
    res = hits if mode == 0 else occ
    return (res, nf, pf) if counts else res


BVH2_NODE_DTYPE = np.dtype([("c0_x", "<f4", (2,)), ("c0_y", "<f4", (2,)), ("c1_x", "<f4", (2,)),
                            ("c1_y", "<f4", (2,)), ("c0_z", "<f4", (2,)), ("c1_z", "<f4", (2,)),
                            ("child", "<i4", (2,)), ("pad", "<u4", (2,))])
PRIM_RECORD_DTYPE = np.dtype([("p0", "<f4", (3,)), ("prim", "<u4"), ("e1", "<f4", (3,)),
                              ("leaf_end", "<u4"), ("e2", "<f4", (3,)), ("pad", "<u4")])


def bvh_build(tris: np.ndarray):
    """The oracle's own binned-SAH BVH2 (bvh_build_oracle.c) over `tris`:
    (nodes, prims) in the arrays bvh_trace(0, ...) reads.  Used by the CPU
    reference arm, which must not run the engine's builder."""
    tris = np.ascontiguousarray(tris)
    n = len(tris)
    nodes = np.zeros(max(1, n), dtype=BVH2_NODE_DTYPE)
    prims = np.zeros(n, dtype=PRIM_RECORD_DTYPE)
    count = lib().orc_bvh_build(_ptr(tris), n, _ptr(nodes), _ptr(prims)) if n else 0
    if count < 0:
        raise MemoryError("oracle BVH build ran out of memory")
    return nodes[:count], prims


# --- the reference's own shader code --------------------------------------

class _RefScene(C.Structure):
    _fields_ = [("triangles", C.c_void_p), ("triangle_count", C.c_uint32),
                ("spheres", C.c_void_p), ("sphere_count", C.c_uint32),
                ("cubes", C.c_void_p), ("cube_count", C.c_uint32),
                ("planes", C.c_void_p), ("plane_count", C.c_uint32)]


def _ref_scene(tris, spheres=None, cubes=None, planes=None):
    keep = [np.ascontiguousarray(x) if x is not None else None for x in (tris, spheres, cubes, planes)]
    s = _RefScene()
    s.triangles, s.triangle_count = _ptr(keep[0]), len(keep[0]) if keep[0] is not None else 0
    s.spheres, s.sphere_count = _ptr(keep[1]), len(keep[1]) if keep[1] is not None else 0
    s.cubes, s.cube_count = _ptr(keep[2]), len(keep[2]) if keep[2] is not None else 0
    s.planes, s.plane_count = _ptr(keep[3]), len(keep[3]) if keep[3] is not None else 0
    return s, keep


def ref_trace_geometry(tris, rays6: np.ndarray, prev=None, spheres=None, cubes=None, planes=None):
    """The reference's traceGeometry; rays6 is (N, 6) float32 {pos, dir}."""
    s, keep = _ref_scene(tris, spheres, cubes, planes)
    r = np.ascontiguousarray(rays6, dtype=np.float32)
    n = len(r)
    out = np.zeros(n, dtype=REF_HIT_DTYPE)
    p = _prev(prev, n)
    if n:
        ref_lib().igxref_trace_geometry(C.addressof(s), _ptr(r), _ptr(p), n, _ptr(out))
    return out


def ref_trace_occlusion(tris, rays6: np.ndarray, max_dist: np.ndarray, prev=None, spheres=None,
                        cubes=None, planes=None):
    s, keep = _ref_scene(tris, spheres, cubes, planes)
    r = np.ascontiguousarray(rays6, dtype=np.float32)
    md = np.ascontiguousarray(max_dist, dtype=np.float32)
    n = len(r)
    out = np.zeros(n, dtype=np.uint32)
    p = _prev(prev, n)
    if n:
        ref_lib().igxref_trace_occlusion(C.addressof(s), _ptr(r), _ptr(md), _ptr(p), n, _ptr(out))
    return out
