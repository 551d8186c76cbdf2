"""ctypes bindings of include/igxrt.h (the engine's C ABI).

The library is loaded from this package directory.  There is no fallback:
if libigxrt.so is missing, importing the package raises, because every query
must run on the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libigxrt.so")

NO_HIT = np.float32(3.4028235e38)
NO_RAY_HIT = 0xFFFFFFFF

LAYOUT_BVH2 = 0
LAYOUT_BVH4 = 1
LAYOUT_BVH8 = 2
LAYOUT_COUNT = 3
TRACE_HOST_MEMORY = 1
TRACE_STAGED = 2
TRACE_INDEPENDENT = 4
TUNE_PLAIN = 1
STATIC_SCRATCH_BYTES = 16 << 20
STATIC_MAX_RAYS = 320000

STATUS = {
    0: "IGXRT_OK",
    1: "IGXRT_ERROR_INVALID_ARGUMENT",
    2: "IGXRT_ERROR_CUDA",
    3: "IGXRT_ERROR_OUT_OF_MEMORY",
    4: "IGXRT_ERROR_INVALID_BVH",
    5: "IGXRT_ERROR_KERNEL_STATUS",
    6: "IGXRT_ERROR_ADMISSION",
    7: "IGXRT_ERROR_TIMEOUT",
    8: "IGXRT_ERROR_UNSUPPORTED",
    9: "IGXRT_ERROR_NOT_READY",
    10: "IGXRT_ERROR_IO",
}

# numpy views of the ABI records (little-endian, packed exactly as the C structs)
TRIANGLE_DTYPE = np.dtype([("p0", "<f4", (3,)), ("n0", "<u4"), ("p1", "<f4", (3,)), ("n1", "<u4"),
                           ("p2", "<f4", (3,)), ("n2", "<u4")])
RAY_DTYPE = np.dtype([("org", "<f4", (3,)), ("tmin", "<f4"), ("dir", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])
PRIM_RECORD_DTYPE = np.dtype([("p0", "<f4", (3,)), ("prim", "<u4"), ("e1", "<f4", (3,)),
                              ("leaf_end", "<u4"), ("e2", "<f4", (3,)), ("pad", "<u4")])
BVH2_NODE_DTYPE = np.dtype([("c0_x", "<f4", (2,)), ("c0_y", "<f4", (2,)), ("c1_x", "<f4", (2,)),
                            ("c1_y", "<f4", (2,)), ("c0_z", "<f4", (2,)), ("c1_z", "<f4", (2,)),
                            ("child", "<i4", (2,)), ("pad", "<u4", (2,))])
BVH4_NODE_DTYPE = np.dtype([("lo_x", "<f4", (4,)), ("hi_x", "<f4", (4,)), ("lo_y", "<f4", (4,)),
                            ("hi_y", "<f4", (4,)), ("lo_z", "<f4", (4,)), ("hi_z", "<f4", (4,)),
                            ("child", "<i4", (4,)), ("pad", "<u4", (4,))])
BVH8_NODE_DTYPE = np.dtype([("origin", "<f4", (3,)), ("exp", "i1", (3,)), ("valid", "u1"),
                            ("lo_x", "u1", (8,)), ("hi_x", "u1", (8,)), ("lo_y", "u1", (8,)),
                            ("hi_y", "u1", (8,)), ("lo_z", "u1", (8,)), ("hi_z", "u1", (8,)),
                            ("child", "<i4", (8,))])
NODE_DTYPES = {LAYOUT_BVH2: BVH2_NODE_DTYPE, LAYOUT_BVH4: BVH4_NODE_DTYPE, LAYOUT_BVH8: BVH8_NODE_DTYPE}
assert TRIANGLE_DTYPE.itemsize == 48 and RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 16
assert BVH8_NODE_DTYPE.itemsize == 96
assert PRIM_RECORD_DTYPE.itemsize == 48 and BVH2_NODE_DTYPE.itemsize == 64
assert BVH4_NODE_DTYPE.itemsize == 128


class BuildOptions(C.Structure):
    _fields_ = [("max_leaf_size", C.c_uint32), ("sah_bins", C.c_uint32), ("node_cost", C.c_float),
                ("tri_cost", C.c_float), ("threads", C.c_uint32), ("reserved", C.c_uint32 * 3)]


class BvhInfo(C.Structure):
    _fields_ = [("triangle_count", C.c_uint32), ("bvh2_nodes", C.c_uint32),
                ("bvh4_nodes", C.c_uint32), ("leaf_count", C.c_uint32), ("max_depth", C.c_uint32),
                ("max_leaf_size", C.c_uint32), ("sah_cost", C.c_float), ("bounds", C.c_float * 6),
                ("pad_abs", C.c_float), ("max_stack", C.c_uint32 * LAYOUT_COUNT),
                ("bvh8_nodes", C.c_uint32), ("device_bytes", C.c_uint64), ("sphere_count", C.c_uint32),
                ("cube_count", C.c_uint32), ("plane_count", C.c_uint32), ("reserved", C.c_uint32)]


class LaunchParams(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("stack_depth", C.c_uint32),
                ("packet_size", C.c_uint32), ("layout", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("refill_lanes", C.c_uint32), ("phase_break", C.c_uint32), ("reserved", C.c_uint32)]


class BatchItem(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("rays", C.c_void_p), ("prev_hit", C.c_void_p),
                ("out", C.c_void_p), ("count", C.c_uint32), ("mode", C.c_uint32)]


class TuneOptions(C.Structure):
    _fields_ = [("reps", C.c_uint32), ("layouts_mask", C.c_uint32), ("cache_path", C.c_char_p),
                ("class_key", C.c_char_p), ("force", C.c_uint32), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


MODE_CLOSEST = 0
MODE_ANY = 1

_vp = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_i32 = C.c_int
_st = C.c_int

# (name, restype, argtypes) for every entry point of include/igxrt.h.
PROTOTYPES = [
    ("igxrt_bvh_build", _st, [_vp, _u32, C.POINTER(BuildOptions), C.POINTER(_vp)]),
    ("igxrt_bvh_destroy", _st, [_vp]),
    ("igxrt_bvh_get_info", _st, [_vp, C.POINTER(BvhInfo)]),
    ("igxrt_bvh_get_data", _st, [_vp, _u32, C.POINTER(_vp), C.POINTER(_u64), C.POINTER(_vp),
                                 C.POINTER(_u64)]),
    ("igxrt_bvh_validate", _st, [_vp, C.c_char_p, C.c_size_t]),
    ("igxrt_bvh_save", _st, [_vp, C.c_char_p]),
    ("igxrt_bvh_load", _st, [C.c_char_p, C.POINTER(_vp)]),
    ("igxrt_create", _st, [_i32, C.POINTER(_vp)]),
    ("igxrt_destroy", _st, [_vp]),
    ("igxrt_last_error", C.c_char_p, [_vp]),
    ("igxrt_status_string", C.c_char_p, [_st]),
    ("igxrt_scene_create", _st, [_vp, _vp, _u32, C.POINTER(BuildOptions), C.POINTER(_vp)]),
    ("igxrt_scene_create_from_bvh", _st, [_vp, _vp, C.POINTER(_vp)]),
    ("igxrt_scene_destroy", _st, [_vp]),
    ("igxrt_scene_get_info", _st, [_vp, C.POINTER(BvhInfo)]),
    ("igxrt_set_launch_params", _st, [_vp, C.POINTER(LaunchParams)]),
    ("igxrt_get_launch_params", _st, [_vp, C.POINTER(LaunchParams)]),
    ("igxrt_trace_closest", _st, [_vp, _vp, _vp, _vp, _u32, _vp, _u32, _vp]),
    ("igxrt_trace_any", _st, [_vp, _vp, _vp, _vp, _u32, _vp, _u32, _vp]),
    ("igxrt_trace_closest_static", _st, [_vp, _vp, _vp, _vp, _u32, _vp, _vp]),
    ("igxrt_batch_create", _st, [_vp, C.POINTER(BatchItem), _u32, C.POINTER(LaunchParams),
                                 C.POINTER(_vp)]),
    ("igxrt_batch_launch", _st, [_vp, _vp]),
    ("igxrt_batch_destroy", _st, [_vp]),
    ("igxrt_trace_batch", _st, [_vp, C.POINTER(BatchItem), _u32, _vp]),
    ("igxrt_autotune", _st, [_vp, C.POINTER(BatchItem), _u32, C.POINTER(TuneOptions),
                             C.POINTER(LaunchParams), C.POINTER(C.c_float)]),
    ("igxrt_fetch_hits", _st, [_vp, _vp, _u32, _vp, _vp]),
    ("igxrt_sync", _st, [_vp, _vp]),
    ("igxrt_count_fetches", _st, [_vp, _vp, _vp, _vp, _u32, _u32, _u32, _vp, _vp, _vp]),
]


class IgxrtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    """Loads libigxrt.so (raising if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA engine first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        h = C.CDLL(LIB_PATH)
        for name, res, args in PROTOTYPES:
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status: int, ctx=None, what: str = "") -> None:
    if status != 0:
        msg = ""
        if ctx:
            raw = lib().igxrt_last_error(ctx)
            msg = raw.decode() if raw else ""
        if not msg:
            msg = lib().igxrt_status_string(status).decode()
        raise IgxrtError(status, f"{what}: {msg}" if what else msg)


class ServerOptions(C.Structure):
    _fields_ = [("memory_cap_bytes", C.c_uint64), ("max_batch_rays", C.c_uint32),
                ("max_batch_requests", C.c_uint32), ("streams", C.c_uint32),
                ("slice_rays", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("mode", C.c_uint32), ("count", C.c_uint32),
                ("reserved", C.c_uint32), ("rays", C.c_void_p), ("prev_hit", C.c_void_p),
                ("out", C.c_void_p)]


class RequestStats(C.Structure):
    _fields_ = [("submitted", C.c_double), ("admitted", C.c_double), ("launched", C.c_double),
                ("completed", C.c_double), ("batch", C.c_uint32), ("status", C.c_uint32),
                ("arrival", C.c_double)]


class BatchTime(C.Structure):
    _fields_ = [("start_ns", C.c_uint64), ("end_ns", C.c_uint64), ("batch", C.c_uint32),
                ("stream", C.c_uint32), ("rays", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("rays_completed", C.c_uint64), ("batches", C.c_uint64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("first_submit", C.c_double), ("last_complete", C.c_double),
                ("peak_memory_bytes", C.c_uint64), ("peak_pending", C.c_uint32),
                ("peak_in_flight_batches", C.c_uint32)]


PROTOTYPES += [
    ("igxrt_server_create", _st, [_vp, C.POINTER(ServerOptions), C.POINTER(_vp)]),
    ("igxrt_server_add_scene", _st, [_vp, _vp, C.POINTER(_u32)]),
    ("igxrt_server_submit", _st, [_vp, C.POINTER(Request), C.POINTER(_u64)]),
    ("igxrt_server_replay", _st, [_vp, C.POINTER(Request), C.POINTER(C.c_double), _u32,
                                  C.POINTER(_u64)]),
    ("igxrt_server_wait", _st, [_vp, _u64, C.c_double, C.POINTER(RequestStats)]),
    ("igxrt_server_batch_times", _st, [_vp, C.POINTER(BatchTime), _u32, C.POINTER(_u32)]),
    ("igxrt_server_get_stats", _st, [_vp, C.POINTER(ServerStats)]),
    ("igxrt_server_destroy", _st, [_vp]),
]

PROTOTYPES += [
    ("igxrt_trace_shadow_mask", _st, [_vp, _vp, _vp, _vp, _u32, _u32, _u32, _vp, _u32, _vp]),
]

# igxrt_camera (64 bytes)
CAMERA_DTYPE = np.dtype([("eye", "<f4", (3,)), ("width", "<u4"), ("p0", "<f4", (3,)),
                         ("height", "<u4"), ("p1", "<f4", (3,)), ("jitter_x", "<f4"),
                         ("p2", "<f4", (3,)), ("jitter_y", "<f4")])
assert CAMERA_DTYPE.itemsize == 64

PROTOTYPES += [
    ("igxrt_trace_gbuffer", _st, [_vp, _vp, _vp, _vp, _vp, _u32, _vp]),
    ("igxrt_camera_rays", _st, [_vp, _vp, _vp, _u32, _vp]),
]

# igxrt_cube (24 bytes) and igxrt_scene_desc
CUBE_DTYPE = np.dtype([("xy0", "<f4", (2,)), ("z0_x1", "<f4", (2,)), ("yz1", "<f4", (2,))])
assert CUBE_DTYPE.itemsize == 24


class SceneDesc(C.Structure):
    _fields_ = [("triangles", C.c_void_p), ("triangle_count", C.c_uint32),
                ("sphere_count", C.c_uint32), ("spheres", C.c_void_p), ("cubes", C.c_void_p),
                ("cube_count", C.c_uint32), ("plane_count", C.c_uint32), ("planes", C.c_void_p)]


PROTOTYPES += [
    ("igxrt_bvh_build_mixed", _st, [C.POINTER(SceneDesc), C.POINTER(BuildOptions), C.POINTER(_vp)]),
    ("igxrt_scene_create_mixed", _st, [_vp, C.POINTER(SceneDesc), C.POINTER(BuildOptions),
                                       C.POINTER(_vp)]),
]

# refit of moved geometry (host BVH and resident scene) and scene read-back
PROTOTYPES += [
    ("igxrt_bvh_refit", _st, [_vp, C.POINTER(SceneDesc)]),
    ("igxrt_scene_refit", _st, [_vp, _vp, C.POINTER(SceneDesc), _u32, _vp]),
    ("igxrt_scene_read_bvh", _st, [_vp, _vp, _u32, _vp, _u64, _vp, _u64]),
    ("igxrt_scene_create_gpu", _st, [_vp, C.POINTER(SceneDesc), C.POINTER(BuildOptions), _u32, _vp,
                                     C.POINTER(_vp)]),
    ("igxrt_scene_download", _st, [_vp, _vp, C.POINTER(_vp)]),
]
