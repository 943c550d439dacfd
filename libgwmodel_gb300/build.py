"""Build libgwgpu.so in-tree with nvcc for sm_103a (GB300).

    python -m libgwmodel_gb300.build [--force]

Objects go to libgwmodel_gb300/_build/, the library to
libgwmodel_gb300/libgwgpu.so.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgwgpu.so")

SOURCES = ["k_select.cu", "k_mgwr.cu", "mgwr.cpp", "k_contract64.cu", "k_contract_tc.cu", "k_refine.cu", "k_solve.cu", "engine.cpp", "gwrbasic.cpp", "capi.cpp", "task.cpp", "noalloc.cu", "server.cpp", "batch.cpp", "launch_util.cpp", "csv.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgwgpu.so")


def _headers():
    out = []
    for d in (CSRC, INCLUDE, os.path.join(INCLUDE, "gwmodel_gb300")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def _compile(src: str, force: bool, headers, extra) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if force or _stale(obj, path, headers):
        cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, headers, extra), SOURCES))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
