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
