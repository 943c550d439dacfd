"""The IGWRBasicGpuTask binary drop-in as a real consumer sees it: a C++
client (tests/abi/task_client.cpp) dlopen()s libgwgpu.so, calls the extern "C"
factories and drives the task through its vtable only.

CPU: the client compiles against include/IGWRBasicGpuTask.h and runs; with no
GPU the task's fit() reports false instead of crashing (the reference's
GWRBasicGpuTask::fit returns false on any exception).
GPU: fit with AIC bandwidth optimisation and predict agree with the engine."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from libgwmodel_gb300 import _lib, datasets

HERE = os.path.dirname(os.path.abspath(__file__))


def build_client(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "task_client")
    subprocess.run([gxx, "-O1", "-std=c++17", os.path.join(HERE, "abi", "task_client.cpp"), "-o", exe, "-ldl"],
                   check=True, capture_output=True)
    return exe


def write_input(path, pb, bw, crit, loc):
    n, p = pb.n, pb.p
    with open(path, "wb") as f:
        np.array([n, p, int(pb.geographic), int(pb.adaptive), int(pb.kernel), crit, loc.shape[0]],
                 dtype=np.int32).tofile(f)
        np.array([bw], dtype=np.float64).tofile(f)
        for a in (np.asfortranarray(pb.coords).ravel(order="F"), np.asfortranarray(pb.x).ravel(order="F"), pb.y,
                  np.asfortranarray(loc).ravel(order="F")):
            np.asarray(a, dtype=np.float64).tofile(f)


def run(exe, inp, mode):
    out = subprocess.run([exe, _lib.LIB_PATH, inp, mode], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return [l[2:] for l in out.stdout.split("\n") if l.startswith("R ")]


def test_client_builds_and_reports_failure_without_gpu(tmp_path):
    L = _lib.lib()
    import ctypes
    count = ctypes.c_int(-1)
    if L.gwgpu_device_count(ctypes.byref(count)) == _lib.OK and count.value > 0:
        pytest.skip("a GPU is present")
    exe = build_client(tmp_path)
    pb = datasets._plain_problem(np.random.default_rng(1), 200, 3, False, "abi")
    inp = str(tmp_path / "in.bin")
    write_input(inp, pb, 30.0, 0, pb.coords[:5])
    assert run(exe, inp, "fit")[0] == "ok 0"


@pytest.mark.gpu
def test_task_fit_and_predict_match_engine(tmp_path):
    from libgwmodel_gb300 import Engine
    exe = build_client(tmp_path)
    pb = datasets._plain_problem(np.random.default_rng(2), 1500, 4, True, "abi")
    loc = pb.coords[::7] + 0.01
    inp = str(tmp_path / "in.bin")
    write_input(inp, pb, 100.0, 0, loc)
    lines = run(exe, inp, "fit")
    assert lines[0] == "ok 1"
    bw = float(lines[1].split()[1])
    betas = np.array([[float(v) for v in l.split()] for l in lines[5:5 + pb.n]])
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, True)
    want_bw, _ = e.golden(True, 2, 0, 20.0, float(pb.n))
    assert bw == want_bw
    b, _, _, _, _ = e.fit(bw, True, 2, store_s=False)
    assert np.abs(betas - b).max() <= 1e-12 * np.abs(b).max()
    write_input(inp, pb, bw, -1, loc)
    lines = run(exe, inp, "predict")
    assert lines[0] == "ok 1"
    pred = np.array([[float(v) for v in l.split()] for l in lines[1:1 + loc.shape[0]]])
    want = e.predict(loc, bw, True, 2)
    assert np.abs(pred - want).max() <= 1e-12 * np.abs(want).max()
    # the bulk helpers give exactly the per-element results
    assert run(exe, inp, "bulkpredict") == lines
    write_input(inp, pb, 100.0, 0, loc)
    assert run(exe, inp, "bulkfit") == run(exe, inp, "fit")


def test_bulk_helpers_reject_foreign_and_null_pointers():
    import ctypes
    L = _lib.lib()
    t = L.GWRBasicGpuTaskFit_Create(10, 2, 0)
    assert t
    buf = np.zeros(40)
    ptr = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.GWRBasicGpuTask_SetData(t, ptr, ptr, ptr) == 0
    assert L.GWRBasicGpuTask_SetData(t, None, ptr, ptr) == -1
    assert L.GWRBasicGpuTask_GetBetas(None, ptr) == -1
    assert L.GWRBasicGpuTask_GetBetas(t, ptr) == 0  # nothing fitted yet: an empty matrix
    L.GWRBasicGpuTask_Del(t)
