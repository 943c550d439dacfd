"""gwgpu_criterion_noalloc: the criterion entry point that allocates nothing.

It exists for callers that cannot let a library call cudaMalloc (their own
memory pool or budget, no allocation after start-up, or work about to be
captured into a CUDA graph).  This test calls it through the C ABI with
device buffers the test owns and checks it against the existing entry point
(gwgpu_engine_criterion) on two calls in a row, at the FP64 tolerance of the
parity tests (1e-9 relative).  It lives in a file of its own that pytest
collects last, and it needs nothing from earlier tests.
"""
import ctypes

import numpy as np
import pytest

from libgwmodel_gb300 import Engine, _lib, datasets

pytestmark = pytest.mark.gpu

AIC, CV = 0, 1
BISQUARE = 2


def normal_equations(torch, x, y, coords, thr, exclude_self):
    """G[i] = (upper triangle of X^T W_i X packed by rows, X^T W_i y) on the GPU."""
    dev = "cuda:0"
    X = torch.tensor(x, dtype=torch.float64, device=dev)
    Y = torch.tensor(y, dtype=torch.float64, device=dev)
    C = torch.tensor(coords, dtype=torch.float64, device=dev)
    R = torch.tensor(thr, dtype=torch.float64, device=dev)
    dx = C[None, :, 0] - C[:, None, 0]
    dy = C[None, :, 1] - C[:, None, 1]
    d = torch.sqrt(dx * dx + dy * dy)
    t = 1.0 - (d * d) / (R[:, None] * R[:, None])
    W = (d < R[:, None]).to(torch.float64) * (t * t)
    if exclude_self:
        W.fill_diagonal_(0.0)
    p = X.shape[1]
    cols = [X[:, a] * X[:, b] for a in range(p) for b in range(a, p)] + [X[:, a] * Y for a in range(p)]
    Z = torch.stack(cols, dim=1)
    return (W @ Z).contiguous(), X.contiguous(), Y.contiguous(), R.contiguous()


def call_noalloc(torch, n, p, crit, bw, G, X, Y, R):
    beta = torch.zeros((n, p), dtype=torch.float64, device="cuda:0")
    sums = torch.zeros(5, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    rc = _lib.lib().gwgpu_criterion_noalloc(n, p, crit, BISQUARE, float(bw), G.data_ptr(), X.data_ptr(),
                                            Y.data_ptr(), R.data_ptr(), beta.data_ptr(), sums.data_ptr(),
                                            ctypes.c_void_p(stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    return sums.cpu().numpy(), beta.cpu().numpy()


@pytest.mark.parametrize("crit", [AIC, CV])
def test_noalloc_matches_existing_entry_point(crit):
    torch = pytest.importorskip("torch")
    pb = datasets.config0(n=1200, seed=21)
    bw = 150
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, False)
    want = e.criterion(bw, True, BISQUARE, crit)
    thr = e.thresholds(bw)
    G, X, Y, R = normal_equations(torch, pb.x, pb.y, pb.coords, thr, crit == CV)
    first, beta1 = call_noalloc(torch, pb.n, pb.p, crit, bw, G, X, Y, R)
    second, beta2 = call_noalloc(torch, pb.n, pb.p, crit, bw, G, X, Y, R)
    for got in (first[4], second[4]):
        assert abs(got - want) <= 1e-9 * abs(want), (got, want)
    np.testing.assert_array_equal(beta1, beta2)
    assert first[3] == 0.0 and second[3] == 0.0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    buf = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    ptr = buf.data_ptr()
    rc = _lib.lib().gwgpu_criterion_noalloc(65537, 3, AIC, BISQUARE, 10.0, ptr, ptr, ptr, ptr, ptr, ptr, None)
    assert rc == _lib.ERR_INVALID
    assert b"65536" in _lib.lib().gwgpu_last_error()
