"""GB300-native ray-query engine for igx_raytracing's traversal hot path.

Closest-hit and any-hit ray/triangle queries (the reference's traceGeometry /
traceOcclusion, res/shaders/trace.glsl) over a host-built BVH, traversed by
CUDA kernels for sm_103a behind the C ABI in include/igxrt.h.
"""
from ._capi import (HIT_DTYPE, LAYOUT_BVH2, LAYOUT_BVH4, LAYOUT_BVH8, NO_HIT, NO_RAY_HIT, RAY_DTYPE,
                    TRIANGLE_DTYPE, IgxrtError, lib)
from .api import BVH, Batch, Context, Scene, Server, as_rays, as_triangles, make_rays

__all__ = ["BVH", "Batch", "Context", "Scene", "Server", "IgxrtError", "as_rays", "as_triangles", "make_rays", "lib",
           "HIT_DTYPE", "RAY_DTYPE", "TRIANGLE_DTYPE", "NO_HIT", "NO_RAY_HIT", "LAYOUT_BVH2",
           "LAYOUT_BVH4", "LAYOUT_BVH8"]
