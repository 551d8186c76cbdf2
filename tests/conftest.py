import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")
NO_HIT = np.float32(3.4028235e38)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


GOLDEN_CASES = ["heightfield", "edge_cases", "random_small"]


def closest_rays(g: dict) -> np.ndarray:
    """The reference's traceGeometry has no ray interval: tmin 0, tmax noHit."""
    r = g["rays"].copy()
    r["tmin"] = 0.0
    r["tmax"] = NO_HIT
    return r


def occlusion_rays(g: dict) -> np.ndarray:
    """traceOcclusion(ray, maxDist, prevHit): maxDist travels as ray.tmax."""
    r = g["rays"].copy()
    r["tmin"] = 0.0
    r["tmax"] = g["max_dist"]
    return r


def nan_free(g: dict, which: str = "closest") -> np.ndarray:
    """Rays whose linear loop never accepts a NaN t.

    A ray lying in a triangle's plane can make u, v and t all NaN; the
    reference's comparisons are then all false, so the linear loop accepts a
    NaN hit and every later decision depends on index order alone
    (primitive.glsl:258-276).  No BVH order can reproduce that; the oracle
    flags such rays and the BVH/GPU comparisons leave exactly those out.
    """
    from oracle import pyoracle

    rays = closest_rays(g) if which == "closest" else occlusion_rays(g)
    fn = pyoracle.trace_geometry if which == "closest" else pyoracle.trace_occlusion
    _, flags = fn(g["tris"], rays, g["prev"])
    return (flags & pyoracle.EVENT_NAN_T) == 0


def bits(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def f64_report(rays, tris, idx, got_prim, expect_prim, limit: int = 8) -> str:
    """Re-intersects both candidate triangles of each disagreeing ray in
    binary64 (oracle/pyoracle.reintersect_f64) and prints the result, so a
    failure shows which side the exact arithmetic supports."""
    from oracle import pyoracle

    lines = []
    for i in idx[:limit]:
        parts = [f"ray {i}:"]
        for name, p in (("got", int(got_prim[i])), ("expected", int(expect_prim[i]))):
            if p == 0xFFFFFFFF or p >= len(tris):
                parts.append(f"{name} miss")
                continue
            ok, t, u, v = pyoracle.reintersect_f64(rays[i:i + 1], tris[p:p + 1])
            parts.append(f"{name} prim {p}: f64 {'hit' if ok else 'no hit'} t={t:.17g} u={u:.17g} v={v:.17g}")
        lines.append(" ".join(parts))
    text = "\n".join(lines)
    if text:
        print("FP64 re-intersection of disagreements:\n" + text)
    return text


def assert_hits_equal(got, expect_prim, expect_t, expect_u, expect_v, what="", rays=None, tris=None):
    """Bit-exact prim, t, u, v (misses: prim = NO_RAY_HIT and t = noHit).  With
    the rays and triangles given, every disagreement is re-intersected in
    binary64 and logged."""
    hit = expect_prim != 0xFFFFFFFF
    bad_mask = got["prim"] != expect_prim
    for f, e in (("t", expect_t), ("u", expect_u), ("v", expect_v)):
        g, x = bits(got[f]), bits(e)
        # NaN payloads differ between host ISAs (x86 0xffc00000, Arm 0x7fc00000)
        both_nan = np.isnan(np.asarray(got[f])) & np.isnan(np.asarray(e))
        bad_mask |= hit & (g != x) & ~both_nan
    bad = np.nonzero(bad_mask)[0]
    if len(bad) and rays is not None and tris is not None:
        f64_report(rays, tris, bad, got["prim"], expect_prim)
    assert len(bad) == 0, (f"{what}: {len(bad)} rays disagree (prim {int((got['prim'] != expect_prim).sum())}),"
                           f" first rays {bad[:8]}")


@pytest.fixture(scope="session")
def engine_lib():
    import igx_raytracing_gb300 as igx

    return igx.lib()


@pytest.fixture(scope="session")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import igx_raytracing_gb300 as igx

    c = igx.Context(0)
    yield c
    c.close()
