"""Builds the engine library (libigxrt.so) with nvcc for sm_103a.

Sources are compiled in parallel into objects under csrc/_build/ and linked
into igx_raytracing_gb300/libigxrt.so.  Host code is compiled with
-ffp-contract=off so the BVH builder produces the same tree on every host
architecture.  Run `python -m igx_raytracing_gb300.build` or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(CSRC, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libigxrt.so")
INCLUDE = os.path.join(REPO_DIR, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["bvh_build.cpp", "capi.cpp", "autotune.cpp", "server.cpp", "trace_kernels.cu",
           "batch.cu", "shadow.cu", "gbuffer.cu", "refit.cu", "lbvh.cu", "static_scratch.cu"]
HEADERS = ["internal.h", "engine.h", "traverse.cuh", "geometry.cuh", "share.cuh", "gbuffer.cuh"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _common_flags() -> list[str]:
    return ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-I" + INCLUDE,
        "-I" + CSRC,
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-Wall",
    ]


def _newest_input_mtime() -> float:
    paths = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    paths.append(os.path.join(INCLUDE, "igxrt.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(nvcc: str, src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc] + _common_flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    if verbose_ptxas and proc.stderr:
        sys.stderr.write(proc.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compiles libigxrt.so if any source is newer than it; returns its path."""
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= _newest_input_mtime()):
        return LIB_PATH
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose_ptxas), SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
