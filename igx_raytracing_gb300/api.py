"""Host-side API of the ray-query engine, mirroring igx_raytracing's traversal.

The reference exposes its ray queries as two GLSL functions,
traceGeometry(ray, prevHit) -> Hit and traceOcclusion(ray, maxDist, prevHit)
-> bool (res/shaders/trace.glsl:9-66, 70-98), evaluated per thread by the
raygen and shadow dispatches.  Here the same queries take a whole batch:

    ctx = Context()
    scene = ctx.create_scene(triangles)          # SceneGraph buffers + BVH
    hits = scene.trace_geometry(rays, prev_hit)  # traceGeometry per ray
    occ = scene.trace_occlusion(rays, prev_hit)  # traceOcclusion, maxDist = ray.tmax

Arrays may be numpy (host memory: staged by the library) or CUDA torch
tensors (device memory: stream-ordered on torch's current stream).  Every
call runs the CUDA kernels of libigxrt.so; there is no host fallback.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _capi
from ._capi import (HIT_DTYPE, LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8, RAY_DTYPE, TRACE_HOST_MEMORY,
                    TRACE_INDEPENDENT, TRACE_STAGED, TRIANGLE_DTYPE, TUNE_PLAIN, BuildOptions, BvhInfo,
                    IgxrtError, LaunchParams, check, lib)

try:  # torch is only needed for device-memory calls
    import torch
except Exception:  # pragma: no cover - torch is present in every supported image
    torch = None


def _is_cuda_tensor(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


def _is_addressable_tensor(x) -> bool:
    """A tensor the kernels can read and write in place: CUDA memory, or
    pinned host memory (reached over NVLink-C2C on a GB300)."""
    return torch is not None and isinstance(x, torch.Tensor) and (x.is_cuda or x.is_pinned())


def as_triangles(tris) -> np.ndarray:
    """Accepts a TRIANGLE_DTYPE array, or (N,3,3) / (N,9) vertex positions."""
    a = np.asarray(tris)
    if a.dtype == TRIANGLE_DTYPE:
        return np.ascontiguousarray(a)
    a = np.asarray(a, dtype=np.float32)
    if a.ndim == 2 and a.shape[1] == 9:
        a = a.reshape(-1, 3, 3)
    if a.ndim != 3 or a.shape[1:] != (3, 3):
        raise ValueError("triangles must be TRIANGLE_DTYPE records or (N, 3, 3) vertices")
    out = np.zeros(a.shape[0], dtype=TRIANGLE_DTYPE)
    out["p0"], out["p1"], out["p2"] = a[:, 0], a[:, 1], a[:, 2]
    return out


def as_rays(rays) -> np.ndarray:
    """Accepts a RAY_DTYPE array or an (N, 8) float32 array {org, tmin, dir, tmax}."""
    a = np.asarray(rays)
    if a.dtype == RAY_DTYPE:
        return np.ascontiguousarray(a)
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 8:
        raise ValueError("rays must be RAY_DTYPE records or an (N, 8) float32 array")
    return a.view(RAY_DTYPE).reshape(-1)


def make_rays(org, dirs, tmin=0.0, tmax=float(_capi.NO_HIT)) -> np.ndarray:
    org = np.asarray(org, dtype=np.float32).reshape(-1, 3)
    dirs = np.asarray(dirs, dtype=np.float32).reshape(-1, 3)
    r = np.zeros(len(org), dtype=RAY_DTYPE)
    r["org"], r["dir"] = org, dirs
    r["tmin"], r["tmax"] = tmin, tmax
    return r


def _build_options(max_leaf_size=0, sah_bins=0, node_cost=0.0, tri_cost=0.0, threads=0):
    o = BuildOptions()
    o.max_leaf_size, o.sah_bins = max_leaf_size, sah_bins
    o.node_cost, o.tri_cost, o.threads = node_cost, tri_cost, threads
    return o


def _info_dict(info: BvhInfo) -> dict:
    return {
        "triangle_count": info.triangle_count, "bvh2_nodes": info.bvh2_nodes,
        "bvh4_nodes": info.bvh4_nodes, "bvh8_nodes": info.bvh8_nodes, "leaf_count": info.leaf_count,
        "max_depth": info.max_depth, "max_leaf_size": info.max_leaf_size,
        "sah_cost": info.sah_cost, "bounds": list(info.bounds), "pad_abs": info.pad_abs,
        "max_stack": list(info.max_stack), "device_bytes": info.device_bytes,
        "sphere_count": info.sphere_count, "cube_count": info.cube_count,
        "plane_count": info.plane_count,
    }


def scene_desc(triangles=None, spheres=None, cubes=None, planes=None):
    """igxrt_scene_desc over host arrays; returns (desc, arrays kept alive).
    spheres / planes: (N, 4) float32; cubes: CUBE_DTYPE or (N, 6) float32."""
    t = None if triangles is None else as_triangles(triangles)
    s = None if spheres is None else np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4)
    c = None
    if cubes is not None:
        c = np.asarray(cubes)
        c = (np.ascontiguousarray(c) if c.dtype == _capi.CUBE_DTYPE
             else np.ascontiguousarray(c, dtype=np.float32).reshape(-1, 6).view(_capi.CUBE_DTYPE).reshape(-1))
    p = None if planes is None else np.ascontiguousarray(planes, dtype=np.float32).reshape(-1, 4)
    d = _capi.SceneDesc()
    for field, arr in (("triangles", t), ("spheres", s), ("cubes", c), ("planes", p)):
        setattr(d, field, arr.ctypes.data if arr is not None and len(arr) else None)
    d.triangle_count = 0 if t is None else len(t)
    d.sphere_count = 0 if s is None else len(s)
    d.cube_count = 0 if c is None else len(c)
    d.plane_count = 0 if p is None else len(p)
    return d, (t, s, c, p)


class BVH:
    """A BVH built on the host (no GPU needed): igxrt_bvh_*."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def build(cls, triangles, **opts) -> "BVH":
        tris = as_triangles(triangles)
        h = C.c_void_p()
        o = _build_options(**opts)
        check(lib().igxrt_bvh_build(tris.ctypes.data if len(tris) else None, len(tris),
                                    C.byref(o), C.byref(h)), what="igxrt_bvh_build")
        return cls(h.value)

    @classmethod
    def build_mixed(cls, triangles=None, spheres=None, cubes=None, planes=None, **opts) -> "BVH":
        d, keep = scene_desc(triangles, spheres, cubes, planes)
        h = C.c_void_p()
        o = _build_options(**opts)
        check(lib().igxrt_bvh_build_mixed(C.byref(d), C.byref(o), C.byref(h)),
              what="igxrt_bvh_build_mixed")
        return cls(h.value)

    @classmethod
    def load(cls, path: str) -> "BVH":
        h = C.c_void_p()
        check(lib().igxrt_bvh_load(path.encode(), C.byref(h)), what=f"igxrt_bvh_load({path})")
        return cls(h.value)

    def save(self, path: str) -> None:
        check(lib().igxrt_bvh_save(self._h, path.encode()), what=f"igxrt_bvh_save({path})")

    def close(self) -> None:
        if self._h and self._h.value:
            lib().igxrt_bvh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def info(self) -> dict:
        i = BvhInfo()
        check(lib().igxrt_bvh_get_info(self._h, C.byref(i)))
        return _info_dict(i)

    def arrays(self, layout: int = LAYOUT_BVH2):
        """Copies of (nodes, prim records) in the export format of include/igxrt.h."""
        nodes, nn, prims, np_ = C.c_void_p(), C.c_uint64(), C.c_void_p(), C.c_uint64()
        check(lib().igxrt_bvh_get_data(self._h, layout, C.byref(nodes), C.byref(nn),
                                       C.byref(prims), C.byref(np_)))
        ndt = _capi.NODE_DTYPES[layout]
        node_arr = np.zeros(nn.value, dtype=ndt)
        prim_arr = np.zeros(np_.value, dtype=_capi.PRIM_RECORD_DTYPE)
        if nn.value:
            C.memmove(node_arr.ctypes.data, nodes.value, nn.value * ndt.itemsize)
        if np_.value:
            C.memmove(prim_arr.ctypes.data, prims.value, np_.value * 48)
        return node_arr, prim_arr

    def validate(self) -> None:
        buf = C.create_string_buffer(512)
        st = lib().igxrt_bvh_validate(self._h, buf, 512)
        if st != 0:
            raise IgxrtError(st, buf.value.decode())

    def refit(self, triangles=None, spheres=None, cubes=None, planes=None) -> None:
        """igxrt_bvh_refit: moved primitives (the counts of the build), same tree."""
        d, keep = scene_desc(triangles, spheres, cubes, planes)
        check(lib().igxrt_bvh_refit(self._h, C.byref(d)), what="igxrt_bvh_refit")


def _device_desc(triangles=None, spheres=None, cubes=None, planes=None):
    """igxrt_scene_desc over CUDA tensors: triangles (N, 12) float32 in the
    igxrt_triangle layout (vertex, pad word, ...); spheres / planes (N, 4);
    cubes (N, 6) float32."""
    d = _capi.SceneDesc()
    keep = []
    for field, count, arr, width in (("triangles", "triangle_count", triangles, 12),
                                     ("spheres", "sphere_count", spheres, 4),
                                     ("cubes", "cube_count", cubes, 6),
                                     ("planes", "plane_count", planes, 4)):
        if arr is None:
            setattr(d, field, None)
            setattr(d, count, 0)
            continue
        if not _is_cuda_tensor(arr) or arr.dtype != torch.float32:
            raise TypeError(f"{field}: a float32 CUDA tensor")
        t = arr.contiguous().reshape(-1, width)
        keep.append(t)
        setattr(d, field, t.data_ptr() if len(t) else None)
        setattr(d, count, len(t))
    return d, keep


class Scene:
    """A BVH resident in device memory, traced through its context."""

    def __init__(self, ctx: "Context", handle: int, ntris: int):
        self.ctx = ctx
        self._h = C.c_void_p(handle)
        self.triangle_count = ntris

    @property
    def handle(self):
        return self._h

    @property
    def info(self) -> dict:
        i = BvhInfo()
        check(lib().igxrt_scene_get_info(self._h, C.byref(i)))
        return _info_dict(i)

    def close(self) -> None:
        if self._h and self._h.value:
            lib().igxrt_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # Mirrors of the reference's GLSL entry points -------------------------
    def trace_geometry(self, rays, prev_hit=None, stream=None):
        """traceGeometry (trace.glsl:9-66) for every ray: closest hits."""
        return self.ctx.trace_closest(self, rays, prev_hit, stream=stream)

    def trace_occlusion(self, rays, prev_hit=None, stream=None):
        """traceOcclusion (trace.glsl:70-98) for every ray, maxDist = ray.tmax."""
        return self.ctx.trace_any(self, rays, prev_hit, stream=stream)

    # Moving geometry ---------------------------------------------------------
    def refit(self, triangles=None, spheres=None, cubes=None, planes=None, stream=None) -> None:
        """igxrt_scene_refit: new positions (the counts of the scene's creation),
        node boxes recomputed on the GPU.  numpy arrays are staged by the
        library; CUDA tensors are read in place (see _device_desc)."""
        args = (triangles, spheres, cubes, planes)
        on_device = any(_is_cuda_tensor(a) for a in args)
        if on_device:
            d, keep = _device_desc(*args)
            flags = 0
        else:
            d, keep = scene_desc(*args)
            flags = TRACE_HOST_MEMORY
        check(lib().igxrt_scene_refit(self.ctx.handle, self._h, C.byref(d), flags,
                                      Context._stream(stream, on_device)),
              self.ctx.handle, "igxrt_scene_refit")

    def download(self) -> BVH:
        """igxrt_scene_download: the resident tree as a validated host BVH."""
        h = C.c_void_p()
        check(lib().igxrt_scene_download(self.ctx.handle, self._h, C.byref(h)), self.ctx.handle,
              "igxrt_scene_download")
        return BVH(h.value)

    def read_bvh(self, layout: int = LAYOUT_BVH2):
        """igxrt_scene_read_bvh: (nodes, prim records) of the resident scene."""
        i = self.info
        nn = i[("bvh2_nodes", "bvh4_nodes", "bvh8_nodes")[layout]]
        nrec = i["triangle_count"] + i["sphere_count"] + i["cube_count"]
        ndt = _capi.NODE_DTYPES[layout]
        nodes = np.zeros(nn, dtype=ndt)
        prims = np.zeros(nrec, dtype=_capi.PRIM_RECORD_DTYPE)
        check(lib().igxrt_scene_read_bvh(self.ctx.handle, self._h, layout,
                                         nodes.ctypes.data if nn else None, nn,
                                         prims.ctypes.data if nrec else None, nrec),
              self.ctx.handle, "igxrt_scene_read_bvh")
        return nodes, prims


class Context:
    """igxrt_create / igxrt_destroy: one device, launch parameters, staging."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().igxrt_create(device, C.byref(h)), what=f"igxrt_create(device={device})")
        self._h = h
        self.device = device
        # True: host arrays of trace, G-buffer, camera-ray and shadow-mask
        # calls are staged through device buffers (IGXRT_TRACE_STAGED) even
        # where the kernels could read and write them in place
        self.stage_host_arrays = False

    @property
    def handle(self):
        return self._h

    def _host_flags(self) -> int:
        return TRACE_HOST_MEMORY | (TRACE_STAGED if self.stage_host_arrays else 0)

    def close(self) -> None:
        if self._h and self._h.value:
            lib().igxrt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- launch parameters -------------------------------------------------
    @property
    def launch_params(self) -> dict:
        p = LaunchParams()
        check(lib().igxrt_get_launch_params(self._h, C.byref(p)), self._h)
        return {"block_size": p.block_size, "stack_depth": p.stack_depth,
                "packet_size": p.packet_size, "layout": p.layout, "ctas_per_sm": p.ctas_per_sm,
                "refill_lanes": p.refill_lanes, "phase_break": p.phase_break}

    def set_launch_params(self, **kw) -> None:
        cur = self.launch_params
        cur.update(kw)
        p = LaunchParams()
        for k, v in cur.items():
            setattr(p, k, int(v))
        check(lib().igxrt_set_launch_params(self._h, C.byref(p)), self._h, "set_launch_params")

    # -- scenes ------------------------------------------------------------
    def create_scene(self, triangles=None, bvh: Optional[BVH] = None, **opts) -> Scene:
        h = C.c_void_p()
        if bvh is not None:
            check(lib().igxrt_scene_create_from_bvh(self._h, bvh.handle, C.byref(h)), self._h,
                  "igxrt_scene_create_from_bvh")
            return Scene(self, h.value, bvh.info["triangle_count"])
        tris = as_triangles(triangles)
        o = _build_options(**opts)
        check(lib().igxrt_scene_create(self._h, tris.ctypes.data if len(tris) else None,
                                       len(tris), C.byref(o), C.byref(h)), self._h,
              "igxrt_scene_create")
        return Scene(self, h.value, len(tris))

    def create_scene_mixed(self, triangles=None, spheres=None, cubes=None, planes=None,
                           **opts) -> Scene:
        """A scene of all the reference's primitive types (scene.glsl:22-39);
        object ids: triangles, then spheres, cubes, planes."""
        d, keep = scene_desc(triangles, spheres, cubes, planes)
        h = C.c_void_p()
        o = _build_options(**opts)
        check(lib().igxrt_scene_create_mixed(self._h, C.byref(d), C.byref(o), C.byref(h)),
              self._h, "igxrt_scene_create_mixed")
        return Scene(self, h.value, d.triangle_count)

    def create_scene_gpu(self, triangles=None, spheres=None, cubes=None, planes=None,
                         max_leaf_size: int = 0, stream=None) -> Scene:
        """igxrt_scene_create_gpu: the BVH built on the GPU (linear BVH).
        numpy arrays are staged by the library; CUDA tensors are read in place
        (triangles (N, 12) float32 in the igxrt_triangle layout, spheres /
        planes (N, 4), cubes (N, 6))."""
        args = (triangles, spheres, cubes, planes)
        on_device = any(_is_cuda_tensor(a) for a in args)
        if on_device:
            d, keep = _device_desc(*args)
            flags = 0
        else:
            d, keep = scene_desc(*args)
            flags = TRACE_HOST_MEMORY
        h = C.c_void_p()
        o = _build_options(max_leaf_size=max_leaf_size)
        check(lib().igxrt_scene_create_gpu(self._h, C.byref(d), C.byref(o), flags,
                                           Context._stream(stream, on_device), C.byref(h)),
              self._h, "igxrt_scene_create_gpu")
        return Scene(self, h.value, d.triangle_count)

    # -- queries -----------------------------------------------------------
    @staticmethod
    def _stream(stream, device_call: bool):
        if stream is not None:
            return C.c_void_p(int(stream))
        if device_call and torch is not None:
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        return C.c_void_p(0)

    def _trace(self, scene: Scene, rays, prev_hit, mode: int, stream, out=None, independent=False):
        """CUDA or pinned CPU tensors: the stream-ordered device call (returns
        once queued; pinned arrays are read and written in place).  numpy
        arrays: IGXRT_TRACE_HOST_MEMORY (returns once the results are in host
        memory)."""
        fn = lib().igxrt_trace_closest if mode == 0 else lib().igxrt_trace_any
        if _is_addressable_tensor(rays):
            assert rays.dtype == torch.float32 and rays.is_contiguous() and rays.shape[-1] == 8
            n = rays.shape[0]
            if out is None:
                shape = (n, 4) if mode == 0 else (n,)
                dtype = torch.float32 if mode == 0 else torch.int32
                out = (torch.empty(shape, dtype=dtype, device=rays.device) if rays.is_cuda
                       else torch.empty(shape, dtype=dtype).pin_memory())
            assert _is_addressable_tensor(out) and out.is_contiguous()
            prev_ptr = None
            if prev_hit is not None:
                assert _is_addressable_tensor(prev_hit) and prev_hit.dtype == torch.int32
                prev_ptr = prev_hit.data_ptr()
            st = fn(self._h, scene.handle, rays.data_ptr(), prev_ptr, n, out.data_ptr(),
                    TRACE_INDEPENDENT if independent else 0, self._stream(stream, True))
            check(st, self._h, "trace")
            return out
        r = as_rays(rays)
        n = len(r)
        prev = None
        if prev_hit is not None:
            prev = np.ascontiguousarray(prev_hit, dtype=np.uint32)
            if len(prev) != n:
                raise ValueError("prev_hit must have one entry per ray")
        if out is None:
            out = np.empty(n, dtype=HIT_DTYPE) if mode == 0 else np.empty(n, dtype=np.uint32)
        if n == 0:
            return out
        st = fn(self._h, scene.handle, r.ctypes.data, prev.ctypes.data if prev is not None else None,
                n, out.ctypes.data, self._host_flags(), self._stream(stream, False))
        check(st, self._h, "trace")
        return out

    def trace_closest(self, scene: Scene, rays, prev_hit=None, stream=None, out=None,
                      independent: bool = False):
        """independent=True (CUDA tensors): IGXRT_TRACE_INDEPENDENT, this call
        neither reads what the kernel queued before it on the stream writes
        nor writes what that kernel touches, so it may start during that
        kernel's last rays."""
        return self._trace(scene, rays, prev_hit, 0, stream, out, independent)

    def trace_any(self, scene: Scene, rays, prev_hit=None, stream=None, out=None,
                  independent: bool = False):
        return self._trace(scene, rays, prev_hit, 1, stream, out, independent)

    def trace_shadow_mask(self, scene: Scene, rays, object_, width: int, height: int,
                          samples: int, stream=None, out=None):
        """The reference's shadow pass (nv_all.shadow.comp): ballot words per
        16x2 tile and sample.  rays: width*height*samples in (sample, y, x)
        order; object_: width*height primary objects (NO_RAY_HIT = no ray)."""
        words = ((width + 15) // 16) * ((height + 1) // 2) * samples
        fn = lib().igxrt_trace_shadow_mask
        if _is_cuda_tensor(rays):
            if out is None:
                out = torch.empty(words, dtype=torch.int32, device=rays.device)
            check(fn(self._h, scene.handle, rays.data_ptr(), object_.data_ptr(), width, height,
                     samples, out.data_ptr(), 0, self._stream(stream, True)), self._h, "shadow_mask")
            return out
        r = as_rays(rays)
        obj = np.ascontiguousarray(object_, dtype=np.uint32)
        if len(r) != width * height * samples or len(obj) != width * height:
            raise ValueError("rays must be width*height*samples, object width*height")
        if out is None:
            out = np.zeros(words, dtype=np.uint32)
        if words:
            check(fn(self._h, scene.handle, r.ctypes.data, obj.ctypes.data, width, height, samples,
                     out.ctypes.data, self._host_flags(), self._stream(stream, False)), self._h,
                  "shadow_mask")
        return out

    def trace_gbuffer(self, scene: Scene, camera, dir_object=None, uv_normal=None, stream=None):
        """The reference's primary pass (raygen.comp): returns the two
        (height, width, 4) float32 images dir_object and uv_normal.  camera is
        a CAMERA_DTYPE record; uv_normal keeps its contents where rays miss."""
        cam = np.ascontiguousarray(camera, dtype=_capi.CAMERA_DTYPE).reshape(1)
        w, h = int(cam["width"][0]), int(cam["height"][0])
        fn = lib().igxrt_trace_gbuffer
        if dir_object is not None and _is_cuda_tensor(dir_object):
            check(fn(self._h, scene.handle, cam.ctypes.data, dir_object.data_ptr(),
                     uv_normal.data_ptr(), 0, self._stream(stream, True)), self._h, "gbuffer")
            return dir_object, uv_normal
        if dir_object is None:
            dir_object = np.zeros((h, w, 4), dtype=np.float32)
        if uv_normal is None:
            uv_normal = np.zeros((h, w, 4), dtype=np.float32)
        check(fn(self._h, scene.handle, cam.ctypes.data, dir_object.ctypes.data,
                 uv_normal.ctypes.data, self._host_flags(), self._stream(stream, False)), self._h,
              "gbuffer")
        return dir_object, uv_normal

    def camera_rays(self, camera, out=None, stream=None):
        """igxrt_camera_rays: the G-buffer pass's primary rays in pixel order
        (numpy RAY_DTYPE, or into `out`, an (n, 8) float32 CUDA tensor)."""
        cam = np.ascontiguousarray(camera, dtype=_capi.CAMERA_DTYPE).reshape(1)
        n = int(cam["width"][0]) * int(cam["height"][0])
        fn = lib().igxrt_camera_rays
        if out is not None and _is_cuda_tensor(out):
            check(fn(self._h, cam.ctypes.data, out.data_ptr(), 0, self._stream(stream, True)), self._h,
                  "camera_rays")
            return out
        rays = np.zeros(n, dtype=RAY_DTYPE)
        check(fn(self._h, cam.ctypes.data, rays.ctypes.data if n else None, self._host_flags(),
                 self._stream(stream, False)), self._h, "camera_rays")
        return rays

    def count_fetches(self, scene: Scene, rays, prev_hit=None, mode: int = 0,
                      layout: int = LAYOUT_BVH2):
        """Node and primitive records the kernel fetches per ray (host arrays)."""
        r = as_rays(rays)
        n = len(r)
        nf = np.zeros(n, dtype=np.uint32)
        pf = np.zeros(n, dtype=np.uint32)
        prev = None if prev_hit is None else np.ascontiguousarray(prev_hit, dtype=np.uint32)
        if n:
            check(lib().igxrt_count_fetches(
                self._h, scene.handle, r.ctypes.data, prev.ctypes.data if prev is not None else None,
                n, mode, layout, nf.ctypes.data, pf.ctypes.data, None), self._h, "count_fetches")
        return nf, pf

    def sync(self, stream=None) -> None:
        check(lib().igxrt_sync(self._h, self._stream(stream, True)), self._h, "sync")

    # -- batched multi-scene queries ---------------------------------------
    @staticmethod
    def batch_items(items) -> "C.Array":
        """items: iterables (scene, rays, prev_hit or None, out, mode) of CUDA
        tensors or pinned CPU tensors (which the kernel reads and writes in
        place); mode 0 = closest (out: (n,4) float32), 1 = any (out: n int32)."""
        arr = (_capi.BatchItem * max(1, len(items)))()
        addressable = lambda t: _is_cuda_tensor(t) or (torch is not None and isinstance(t, torch.Tensor)
                                                      and t.is_pinned())
        for i, (scene, rays, prev, out, mode) in enumerate(items):
            assert addressable(rays) and addressable(out) and (prev is None or addressable(prev))
            arr[i].scene = scene.handle.value
            arr[i].rays = rays.data_ptr()
            arr[i].prev_hit = prev.data_ptr() if prev is not None else None
            arr[i].out = out.data_ptr()
            arr[i].count = rays.shape[0]
            arr[i].mode = mode
        return arr

    def trace_batch(self, items, stream=None) -> None:
        """One persistent launch over all items (no graph)."""
        arr = self.batch_items(items)
        check(lib().igxrt_trace_batch(self._h, arr, len(items), self._stream(stream, True)),
              self._h, "trace_batch")

    def create_batch(self, items, params: Optional[dict] = None) -> "Batch":
        arr = self.batch_items(items)
        p = None
        if params is not None:
            p = LaunchParams()
            for k, v in params.items():
                setattr(p, k, int(v))
        h = C.c_void_p()
        check(lib().igxrt_batch_create(self._h, arr, len(items), C.byref(p) if p is not None else None,
                                       C.byref(h)), self._h, "batch_create")
        return Batch(self, h.value, items)

    def autotune(self, items, reps: int = 3, layouts=None, cache_path: Optional[str] = None,
                 class_key: Optional[str] = None, force: bool = False, plain: bool = False):
        """Times candidate launch parameters on the items; returns (params, ms).
        plain=True times one plain launch per item (IGXRT_TUNE_PLAIN) instead
        of one batched launch."""
        arr = self.batch_items(items)
        o = _capi.TuneOptions()
        o.reps = reps
        o.flags = TUNE_PLAIN if plain else 0
        o.layouts_mask = 0 if layouts is None else sum(1 << int(l) for l in layouts)
        o.cache_path = cache_path.encode() if cache_path else None
        o.class_key = class_key.encode() if class_key else None
        o.force = 1 if force else 0
        p = LaunchParams()
        ms = C.c_float()
        check(lib().igxrt_autotune(self._h, arr, len(items), C.byref(o), C.byref(p), C.byref(ms)),
              self._h, "autotune")
        return ({"block_size": p.block_size, "stack_depth": p.stack_depth,
                 "packet_size": p.packet_size, "layout": p.layout, "ctas_per_sm": p.ctas_per_sm,
                 "refill_lanes": p.refill_lanes, "phase_break": p.phase_break}, ms.value)


class Server:
    """igxrt_server: resident scenes, admission by device memory, continuous
    batching.  Host arrays passed to submit() are kept referenced until the
    request has been waited for."""

    def __init__(self, ctx: Context, memory_cap_bytes: int = 0, max_batch_rays: int = 0,
                 max_batch_requests: int = 0, streams: int = 0, slice_rays: int = 0):
        o = _capi.ServerOptions()
        o.memory_cap_bytes, o.max_batch_rays = memory_cap_bytes, max_batch_rays
        o.max_batch_requests, o.streams, o.slice_rays = max_batch_requests, streams, slice_rays
        h = C.c_void_p()
        check(lib().igxrt_server_create(ctx.handle, C.byref(o), C.byref(h)), ctx.handle,
              "server_create")
        self.ctx = ctx
        self._h = h
        self._keep = {}

    def add_scene(self, scene: Scene) -> int:
        sid = C.c_uint32()
        check(lib().igxrt_server_add_scene(self._h, scene.handle, C.byref(sid)), what="add_scene")
        return sid.value

    @staticmethod
    def _request(q, scene_id: int, rays, prev_hit, mode: int, out):
        r = as_rays(rays)
        prev = None if prev_hit is None else np.ascontiguousarray(prev_hit, dtype=np.uint32)
        if out is None:
            out = np.empty(len(r), dtype=HIT_DTYPE) if mode == 0 else np.empty(len(r), dtype=np.uint32)
        q.scene_id, q.mode, q.count = scene_id, mode, len(r)
        q.rays = r.ctypes.data if len(r) else None
        q.prev_hit = prev.ctypes.data if prev is not None else None
        q.out = out.ctypes.data if len(r) else None
        return (r, prev, out)

    def submit(self, scene_id: int, rays, prev_hit=None, mode: int = 0, out=None) -> int:
        q = _capi.Request()
        keep = Server._request(q, scene_id, rays, prev_hit, mode, out)
        t = C.c_uint64()
        check(lib().igxrt_server_submit(self._h, C.byref(q), C.byref(t)), what="server_submit")
        self._keep[t.value] = keep
        return t.value

    def replay(self, requests, arrivals) -> list:
        """igxrt_server_replay: requests = [(scene_id, rays, prev_hit, mode,
        out)], submitted natively at arrivals[i] seconds after the call starts;
        each request's latency counts from that scheduled time.  Returns the
        tickets (0 for a request refused at admission)."""
        n = len(requests)
        arr = (_capi.Request * max(n, 1))()
        keep = [Server._request(arr[i], *req) for i, req in enumerate(requests)]
        times = np.ascontiguousarray(arrivals, dtype=np.float64)
        assert len(times) == n
        tickets = (C.c_uint64 * max(n, 1))()
        check(lib().igxrt_server_replay(self._h, arr, times.ctypes.data_as(C.POINTER(C.c_double)), n,
                                        tickets), what="server_replay")
        out = [int(tickets[i]) for i in range(n)]
        for t, k in zip(out, keep):
            if t:
                self._keep[t] = k
        return out

    def batch_times(self, max_batches: int = 1 << 20) -> np.ndarray:
        """igxrt_server_batch_times: (start_ns, end_ns, batch, stream, rays) of
        every completed batch kernel, from %globaltimer on the device."""
        buf = (_capi.BatchTime * max_batches)()
        n = C.c_uint32()
        check(lib().igxrt_server_batch_times(self._h, buf, max_batches, C.byref(n)), what="batch_times")
        dt = np.dtype([("start_ns", "<u8"), ("end_ns", "<u8"), ("batch", "<u4"), ("stream", "<u4"),
                       ("rays", "<u8")])
        return np.frombuffer(bytes(buf)[: n.value * C.sizeof(_capi.BatchTime)], dtype=dt).copy()

    def wait(self, ticket: int, timeout: float = -1.0) -> dict:
        s = _capi.RequestStats()
        st = lib().igxrt_server_wait(self._h, ticket, timeout, C.byref(s))
        if st != 0:
            raise IgxrtError(st, f"request {ticket}")
        kept = self._keep.pop(ticket, None)
        return {"submitted": s.submitted, "admitted": s.admitted, "launched": s.launched,
                "completed": s.completed, "arrival": s.arrival, "batch": s.batch,
                "out": kept[2] if kept is not None else None}

    def stats(self) -> dict:
        s = _capi.ServerStats()
        check(lib().igxrt_server_get_stats(self._h, C.byref(s)), what="server_stats")
        return {f: getattr(s, f) for f, _ in _capi.ServerStats._fields_}

    def close(self) -> None:
        if self._h and self._h.value:
            lib().igxrt_server_destroy(self._h)
            self._h = C.c_void_p()
        self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """igxrt_batch: an item table plus a captured CUDA graph, replayed by launch()."""

    def __init__(self, ctx: Context, handle: int, items):
        self.ctx = ctx
        self._h = C.c_void_p(handle)
        self._items = items  # keep the tensors alive while the graph may run

    def launch(self, stream=None) -> None:
        check(lib().igxrt_batch_launch(self._h, Context._stream(stream, True)), self.ctx.handle,
              "batch_launch")

    def close(self) -> None:
        if self._h and self._h.value:
            lib().igxrt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["BVH", "Batch", "Context", "Scene", "Server", "IgxrtError", "as_rays", "as_triangles",
           "make_rays", "LAYOUT_BVH2", "LAYOUT_BVH4", "LAYOUT_BVH8"]
