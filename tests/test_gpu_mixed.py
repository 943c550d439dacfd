"""Mixed-precision path (tcgen05 TF32x3 contraction) against the FP64 engine.

The tensor-core self-test pins the UMMA descriptors, the 128-byte swizzle and
the TMEM read-out against numpy.  The mixed engine's errors against the FP64
engine are asserted at the levels stated beside each check."""
import numpy as np
import pytest

from libgwmodel_gb300 import Engine, datasets

pytestmark = pytest.mark.gpu


def tf32(x):
    b = np.asarray(x, np.float32).copy().view(np.uint32)
    b += 0x1000
    b &= 0xFFFFE000
    return b.view(np.float32)


@pytest.mark.parametrize("N", [16, 32, 64, 176, 192, 256])
def test_tcgen05_selftest(N):
    rng = np.random.default_rng(N)
    A = rng.standard_normal((128, 32)).astype(np.float32)
    B = rng.standard_normal((N, 32)).astype(np.float32)
    D = Engine(0).tc_selftest(A, B)
    ref = tf32(A).astype(np.float64) @ tf32(B).astype(np.float64).T
    assert np.abs(D - ref).max() <= 1e-6 * np.abs(ref).max() * 32


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def pair(pb):
    e64 = Engine(0)
    e64.set_data(pb.x, pb.y, pb.coords, pb.geographic)
    emx = Engine(0)
    emx.set_data(pb.x, pb.y, pb.coords, pb.geographic)
    emx.set_precision(1)
    return e64, emx


CASES = [("config0", dict(n=2000), [40, 400]), ("config2", dict(n=3000, k=8), [60, 900]),
         ("config1", dict(n=2000), [60.0, 150.0])]


@pytest.mark.parametrize("name,kw,bws", CASES)
def test_mixed_criterion_close_to_fp64(name, kw, bws):
    """AICc / CV of the mixed path within 1e-5 relative of FP64 (no refinement in the search)."""
    pb = datasets.CONFIGS[name](**kw)
    e64, emx = pair(pb)
    for bw in bws:
        c64 = e64.criterion(bw, pb.adaptive, pb.kernel, pb.criterion)
        cmx = emx.criterion(bw, pb.adaptive, pb.kernel, pb.criterion)
        assert abs(cmx - c64) <= 1e-5 * abs(c64), (bw, cmx, c64)


@pytest.mark.parametrize("name,kw,bws", CASES)
def test_mixed_fit_close_to_fp64(name, kw, bws):
    pb = datasets.CONFIGS[name](**kw)
    e64, emx = pair(pb)
    bw = bws[0]
    b64, se64, sh64, q64, _ = e64.fit(bw, pb.adaptive, pb.kernel, False)
    bmx, semx, shmx, qmx, _ = emx.fit(bw, pb.adaptive, pb.kernel, False)
    beta_err = max(rel(bmx[:, k], b64[:, k]) for k in range(pb.p))
    assert beta_err <= 1e-6, beta_err
    # element by element, over the coefficients at least 1e-3 of their column's largest:
    # median <= 1e-7, 99th percentile <= 1e-5, none above 1e-3
    e = np.concatenate([np.abs(bmx[m, k] - b64[m, k]) / np.abs(b64[m, k]) for k in range(pb.p)
                        for m in [np.abs(b64[:, k]) >= 1e-3 * np.abs(b64[:, k]).max()]])
    assert np.median(e) <= 1e-7 and np.quantile(e, 0.99) <= 1e-5 and e.max() <= 1e-3, \
        (np.median(e), np.quantile(e, 0.99), e.max())
    assert max(rel(semx[:, k], se64[:, k]) for k in range(pb.p)) <= 1e-4
    assert rel(shmx, sh64) <= 1e-5
    assert rel(qmx, q64) <= 1e-5


@pytest.mark.parametrize("name,kw,bw", [("config2", dict(n=3000, k=8), 900), ("config0", dict(n=2000), 400)])
def test_contraction_timeout_is_reported_and_engine_recovers(name, kw, bw):
    """With a limit of one poll the contraction's pipeline waits run out: the
    kernel waits for its own MMAs and bulk copies, frees its tensor memory and
    sets the error flag; the call fails with that error, and the next call on
    the same engine (default limit) returns the value it returned before."""
    from libgwmodel_gb300 import GwgpuError
    pb = datasets.CONFIGS[name](**kw)
    _, emx = pair(pb)
    want = emx.criterion(bw, pb.adaptive, pb.kernel, pb.criterion)
    emx.set_tc_wait_limit(1)
    with pytest.raises(GwgpuError, match="timed out"):
        emx.criterion(bw, pb.adaptive, pb.kernel, pb.criterion)
    emx.set_tc_wait_limit(0)
    assert emx.criterion(bw, pb.adaptive, pb.kernel, pb.criterion) == want
