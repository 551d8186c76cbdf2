"""The C ABI library: loads, exports every entry point of include/igxrt.h,
and its ctypes prototypes cover the header.  No compute calls."""
import os
import re

import pytest

from conftest import REPO
from igx_raytracing_gb300 import _capi

HEADER = os.path.join(REPO, "include", "igxrt.h")


def declared_functions() -> list:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(igxrt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "igxrt_trace_closest" in names and "igxrt_trace_any" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_ctypes_prototypes_cover_header():
    proto = {p[0] for p in _capi.PROTOTYPES}
    assert set(declared_functions()) == proto


def test_status_strings(engine_lib):
    for code in _capi.STATUS:
        assert engine_lib.igxrt_status_string(code)


def test_null_arguments_are_rejected_without_a_gpu(engine_lib):
    import ctypes as C

    assert engine_lib.igxrt_bvh_get_info(None, None) == 1
    assert engine_lib.igxrt_trace_closest(None, None, None, None, 0, None, 0, None) == 1
    assert engine_lib.igxrt_sync(None, None) == 1
    assert engine_lib.igxrt_last_error(None) == b"context is NULL"
    h = C.c_void_p()
    assert engine_lib.igxrt_bvh_load(b"/nonexistent/x.bvh", C.byref(h)) == 10


def test_create_without_gpu_reports_cuda_error(engine_lib):
    import ctypes as C

    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert engine_lib.igxrt_create(0, C.byref(h)) == 2
    assert not h.value


def test_python_constants_match_the_header():
    """Every #define the Python binding restates (flags, layouts, modes,
    sentinels, the static path's limits) has the header's value."""
    text = open(HEADER).read()
    defines = {}
    for name, value in re.findall(r"#define\s+(IGXRT_[A-Z0-9_]+)\s+([^\s/]+)", text):
        defines[name] = value
    as_int = lambda v: int(v.rstrip("uU"), 0)
    pairs = {"IGXRT_TRACE_HOST_MEMORY": _capi.TRACE_HOST_MEMORY, "IGXRT_TRACE_STAGED": _capi.TRACE_STAGED,
             "IGXRT_TRACE_INDEPENDENT": _capi.TRACE_INDEPENDENT, "IGXRT_TUNE_PLAIN": _capi.TUNE_PLAIN,
             "IGXRT_LAYOUT_BVH2": _capi.LAYOUT_BVH2,
             "IGXRT_LAYOUT_BVH4": _capi.LAYOUT_BVH4, "IGXRT_LAYOUT_BVH8": _capi.LAYOUT_BVH8,
             "IGXRT_LAYOUT_COUNT": _capi.LAYOUT_COUNT, "IGXRT_MODE_CLOSEST": _capi.MODE_CLOSEST,
             "IGXRT_MODE_ANY": _capi.MODE_ANY, "IGXRT_NO_RAY_HIT": _capi.NO_RAY_HIT}
    for name, value in pairs.items():
        assert name in defines, name
        assert as_int(defines[name]) == value, name
    import numpy as np

    assert np.float32(defines["IGXRT_NO_HIT"].rstrip("fF")) == _capi.NO_HIT
    assert as_int(defines["IGXRT_STATIC_MAX_RAYS"]) == _capi.STATIC_MAX_RAYS
    m = re.search(r"#define\s+IGXRT_STATIC_SCRATCH_BYTES\s+\((\d+)u\s*<<\s*(\d+)\)", text)
    assert m and int(m.group(1)) << int(m.group(2)) == _capi.STATIC_SCRATCH_BYTES
    flags = [_capi.TRACE_HOST_MEMORY, _capi.TRACE_STAGED, _capi.TRACE_INDEPENDENT]
    assert all(f & (f - 1) == 0 for f in flags) and len(set(flags)) == 3  # distinct bits


# ctypes structures of the Python binding and the C structs they mirror;
# numpy record layouts and the C records of the same memory image
_STRUCTS = {"BuildOptions": "igxrt_build_options", "BvhInfo": "igxrt_bvh_info",
            "LaunchParams": "igxrt_launch_params", "BatchItem": "igxrt_batch_item",
            "TuneOptions": "igxrt_tune_options", "ServerOptions": "igxrt_server_options",
            "Request": "igxrt_request", "RequestStats": "igxrt_request_stats",
            "ServerStats": "igxrt_server_stats", "SceneDesc": "igxrt_scene_desc",
            "BatchTime": "igxrt_batch_time"}
_RECORDS = {"TRIANGLE_DTYPE": "igxrt_triangle", "RAY_DTYPE": "igxrt_ray", "HIT_DTYPE": "igxrt_hit",
            "PRIM_RECORD_DTYPE": "igxrt_prim_record", "BVH2_NODE_DTYPE": "igxrt_bvh2_node",
            "BVH4_NODE_DTYPE": "igxrt_bvh4_node", "BVH8_NODE_DTYPE": "igxrt_bvh8_node",
            "CAMERA_DTYPE": "igxrt_camera", "CUBE_DTYPE": "igxrt_cube"}


def test_binding_layouts_match_the_header(tmp_path):
    """Every ctypes structure has the size and field offsets of its C struct
    (compiled against include/igxrt.h by the host compiler), and every numpy
    record layout the size of its C record."""
    import ctypes
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "igxrt.h"', "int main(void) {"]
    expect = []
    for py, c in _STRUCTS.items():
        cls = getattr(_capi, py)
        lines.append(f'    printf("%zu\\n", sizeof({c}));')
        expect.append((f"sizeof {c}", ctypes.sizeof(cls)))
        for name, *_ in cls._fields_:
            lines.append(f'    printf("%zu\\n", offsetof({c}, {name}));')
            expect.append((f"{c}.{name}", getattr(cls, name).offset))
    for py, c in _RECORDS.items():
        lines.append(f'    printf("%zu\\n", sizeof({c}));')
        expect.append((f"sizeof {c}", getattr(_capi, py).itemsize))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layouts"
    subprocess.run([cc, "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert len(got) == len(expect)
    wrong = [(what, want, g) for (what, want), g in zip(expect, got) if want != g]
    assert not wrong, wrong


def test_integration_cpp_example_compiles_and_links(engine_lib, tmp_path):
    """The C++ example of INTEGRATION.md, inside a function that declares its
    inputs, compiles against include/igxrt.h and links against libigxrt.so."""
    import shutil
    import subprocess

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    doc = open(os.path.join(REPO, "INTEGRATION.md")).read()
    block = re.search(r"```cpp\n(.*?)```", doc, flags=re.S).group(1)
    body = "\n".join(l for l in block.splitlines() if not l.startswith("#include"))
    src = tmp_path / "example.cpp"
    src.write_text("#include <cstdio>\n#include <vector>\n#include \"igxrt.h\"\n"
                   "void example(const std::vector<igxrt_triangle>& triangles, const igxrt_ray* d_rays,\n"
                   "             igxrt_hit* d_hits, uint32_t w, uint32_t h, void* stream,\n"
                   "             const igxrt_ray* h_rays, igxrt_hit* h_hits, uint32_t n) {\n"
                   + body + "\n}\nint main() { return 0; }\n")
    lib_dir = os.path.dirname(_capi.LIB_PATH)
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src),
                    "-o", str(tmp_path / "example"), "-L", lib_dir, "-ligxrt", "-Wl,-rpath," + lib_dir],
                   check=True)
