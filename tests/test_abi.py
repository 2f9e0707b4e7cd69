"""C-ABI library checks that need no GPU: it builds for sm_103a, loads, and exports every
function include/vvgpu.h declares; the ctypes structs match the header's layouts."""
import ctypes as C
import os
import re

import pytest

from vvflow_gb300 import build as B
from vvflow_gb300 import vvgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "vvgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vvgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return vvgpu.load_library()


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(vvgpu.SIGNATURES) == names


def test_struct_layouts():
    assert C.sizeof(vvgpu.BodyParams) == 26 * 8 + 2 * 4
    assert C.sizeof(vvgpu.BodyOut) == 9 * 8
    assert C.sizeof(vvgpu.Cfg) == 24
    assert C.sizeof(vvgpu.Stats) == 19 * 8


def test_null_and_bad_arguments_are_errors(lib):
    assert lib.vvgpu_ctx_destroy(None) == -1
    assert lib.vvgpu_tree_build(None, 8.0, 0.0, 1.0) == -1
    out = C.c_void_p()
    bad = vvgpu.Cfg(0, 7, 0, 0)  # unknown precision
    assert lib.vvgpu_ctx_create(C.byref(bad), C.byref(out)) == -1
    assert not out.value


def test_no_device_is_reported_not_faked(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    out = C.c_void_p()
    rc = lib.vvgpu_ctx_create(C.byref(vvgpu.Cfg(0, 0, 0, 0)), C.byref(out))
    assert rc == -6 and not out.value  # VVGPU_ERR_CUDA, no silent CPU path
