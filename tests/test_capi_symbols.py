"""CPU checks of the boundary: the library builds for sm_103a, loads without a
GPU, exports every function the public headers declare, and reports a missing
device as an error instead of falling back."""
import ctypes
import os
import re
import subprocess

import pytest

from libgwmodel_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "gwgpu.h"), os.path.join(ROOT, "include", "IGWRBasicGpuTask.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(gwgpu_\w+|GWRBasicGpuTask\w*)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_abi():
    names = declared_functions()
    assert "gwgpu_gwr_fit" in names and "GWRBasicGpuTaskFit_Create" in names
    assert len(names) >= 45


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    bound = {n for n, _, _ in _lib.SIGNATURES + _lib.TASK_SIGNATURES}
    assert set(declared_functions()) <= bound


def test_symbols_have_default_visibility():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    for n in declared_functions():
        assert re.search(rf"\bT {n}\b", out), n


def test_no_gpu_is_an_error_not_a_fallback():
    L = _lib.lib()
    count = ctypes.c_int(-1)
    rc = L.gwgpu_device_count(ctypes.byref(count))
    if rc == _lib.OK and count.value > 0:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = L.gwgpu_engine_create(0, ctypes.byref(h))
    assert rc == _lib.ERR_CUDA
    assert L.gwgpu_last_error()


def test_null_handles_are_rejected():
    L = _lib.lib()
    assert L.gwgpu_gwr_fit(None) == _lib.ERR_INVALID
    assert L.gwgpu_engine_criterion(None, 1.0, 1, 0, 0, None) == _lib.ERR_INVALID
