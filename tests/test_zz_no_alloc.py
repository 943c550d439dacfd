"""gwgpu_criterion_noalloc: the criterion entry point that allocates nothing.

It exists for callers that cannot let a library call cudaMalloc: their own
memory pool or budget, or no allocation after start-up (cudaMalloc and
cudaFree synchronise the whole device).  These tests call it through the C
ABI with device buffers the test owns and check it against the existing entry
point (gwgpu_engine_criterion) on two calls in a row, at the FP64 tolerance of
the parity tests (1e-9 relative): per-row adaptive thresholds and a fixed
bandwidth (thr = NULL), p = 5 and p = 24, and that a call leaves the device's
free memory unchanged.  The file is collected last and needs nothing from
earlier tests.
"""
import ctypes

import numpy as np
import pytest

from libgwmodel_gb300 import Engine, _lib, datasets

pytestmark = pytest.mark.gpu

AIC, CV = 0, 1
GAUSSIAN, BISQUARE = 0, 2


def normal_equations(torch, x, y, coords, thr, exclude_self, kernel=BISQUARE):
    """G[i] = (upper triangle of X^T W_i X packed by rows, X^T W_i y) on the GPU;
    thr is the per-row bandwidth (array) or the fixed bandwidth (scalar)."""
    dev = "cuda:0"
    X = torch.tensor(x, dtype=torch.float64, device=dev)
    Y = torch.tensor(y, dtype=torch.float64, device=dev)
    C = torch.tensor(coords, dtype=torch.float64, device=dev)
    R = torch.tensor(np.broadcast_to(thr, (len(y),)).copy(), dtype=torch.float64, device=dev)
    dx = C[None, :, 0] - C[:, None, 0]
    dy = C[None, :, 1] - C[:, None, 1]
    d = torch.sqrt(dx * dx + dy * dy)
    if kernel == GAUSSIAN:
        W = torch.exp((d * d) / (-2.0 * (R[:, None] * R[:, None])))
    else:
        t = 1.0 - (d * d) / (R[:, None] * R[:, None])
        W = (d < R[:, None]).to(torch.float64) * (t * t)
    if exclude_self:
        W.fill_diagonal_(0.0)
    p = X.shape[1]
    cols = [X[:, a] * X[:, b] for a in range(p) for b in range(a, p)] + [X[:, a] * Y for a in range(p)]
    Z = torch.stack(cols, dim=1)
    return (W @ Z).contiguous(), X.contiguous(), Y.contiguous(), R.contiguous()


def call_noalloc(torch, n, p, crit, bw, G, X, Y, R, kernel=BISQUARE, out=None):
    """One call; R = None passes thr = NULL (the fixed bandwidth bw)."""
    beta, sums = out if out else (torch.zeros((n, p), dtype=torch.float64, device="cuda:0"),
                                  torch.zeros(5, dtype=torch.float64, device="cuda:0"))
    stream = torch.cuda.current_stream().cuda_stream
    rc = _lib.lib().gwgpu_criterion_noalloc(n, p, crit, kernel, float(bw), G.data_ptr(), X.data_ptr(),
                                            Y.data_ptr(), R.data_ptr() if R is not None else None,
                                            beta.data_ptr(), sums.data_ptr(), ctypes.c_void_p(stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    return sums.cpu().numpy(), beta.cpu().numpy()


def wide_problem(n, p, seed):
    """Planar problem with p columns (intercept + p - 1 covariates)."""
    rng = np.random.default_rng(seed)
    coords = rng.uniform(0, 100, (n, 2))
    x = np.column_stack([np.ones(n), rng.standard_normal((n, p - 1))])
    beta = 1.0 + 0.3 * np.sin(coords[:, :1] / 20.0) * rng.uniform(-1, 1, (1, p))
    y = (x * beta).sum(1) + rng.normal(0, 0.5, n)
    return datasets.Problem("wide", np.asfortranarray(x), y, np.asfortranarray(coords), False, True, BISQUARE, 0,
                            beta)


def check_against_engine(torch, pb, crit, kernel, bw, adaptive):
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, False)
    want = e.criterion(bw, adaptive, kernel, crit)
    thr = e.thresholds(bw) if adaptive else bw
    G, X, Y, R = normal_equations(torch, pb.x, pb.y, pb.coords, thr, crit == CV, kernel)
    R = R if adaptive else None
    first, beta1 = call_noalloc(torch, pb.n, pb.p, crit, bw, G, X, Y, R, kernel)
    second, beta2 = call_noalloc(torch, pb.n, pb.p, crit, bw, G, X, Y, R, kernel)
    for got in (first[4], second[4]):
        assert abs(got - want) <= 1e-9 * abs(want), (got, want)
    np.testing.assert_array_equal(beta1, beta2)
    assert first[3] == 0.0 and second[3] == 0.0


@pytest.mark.parametrize("crit", [AIC, CV])
def test_noalloc_matches_existing_entry_point(crit):
    torch = pytest.importorskip("torch")
    check_against_engine(torch, datasets.config0(n=1200, seed=21), crit, BISQUARE, 150, True)


@pytest.mark.parametrize("crit", [AIC, CV])
def test_noalloc_fixed_bandwidth_without_thresholds(crit):
    """thr = NULL: the fixed bandwidth gives w_ii (gaussian kernel, bandwidth 12)."""
    torch = pytest.importorskip("torch")
    check_against_engine(torch, datasets.config0(n=1000, seed=22), crit, GAUSSIAN, 12.0, False)


@pytest.mark.parametrize("crit", [AIC, CV])
def test_noalloc_wide_problem(crit):
    """p = 24: the widest local systems of the warp-per-location solve's range."""
    torch = pytest.importorskip("torch")
    check_against_engine(torch, wide_problem(900, 24, 23), crit, BISQUARE, 300, True)


def test_noalloc_leaves_free_memory_unchanged():
    """A warm call allocates nothing: the device's free memory is the same
    before and after it (cudaMemGetInfo through torch)."""
    torch = pytest.importorskip("torch")
    pb = datasets.config0(n=800, seed=24)
    e = Engine(0)
    e.set_data(pb.x, pb.y, pb.coords, False)
    thr = e.thresholds(100)
    G, X, Y, R = normal_equations(torch, pb.x, pb.y, pb.coords, thr, False)
    out = (torch.zeros((pb.n, pb.p), dtype=torch.float64, device="cuda:0"),
           torch.zeros(5, dtype=torch.float64, device="cuda:0"))
    call_noalloc(torch, pb.n, pb.p, AIC, 100, G, X, Y, R, out=out)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    sums, _ = call_noalloc(torch, pb.n, pb.p, AIC, 100, G, X, Y, R, out=out)
    free_after = torch.cuda.mem_get_info(0)[0]
    assert free_after == free_before, (free_before, free_after)
    assert sums[3] == 0.0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    buf = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    ptr = buf.data_ptr()
    rc = _lib.lib().gwgpu_criterion_noalloc(65537, 3, AIC, BISQUARE, 10.0, ptr, ptr, ptr, ptr, ptr, ptr, None)
    assert rc == _lib.ERR_INVALID
    assert b"65536" in _lib.lib().gwgpu_last_error()
