"""Batched evaluation (one launch per phase over all problems and candidates,
replayed from a CUDA graph) against the single-problem engine: every
criterion value agrees to 1e-12 relative (the only difference is the grouping
of the final per-row sums), with and without the graph, for AICc and CV, in
both numeric forms, and after autotuning."""
import numpy as np
import pytest

from libgwmodel_gb300 import Engine, Precision, datasets
from libgwmodel_gb300.batch import Batch

pytestmark = pytest.mark.gpu

TOL = 1e-12


def problems():
    rng = np.random.default_rng(7)
    shapes = [(600, 3, False), (1500, 5, False), (2400, 8, False), (900, 4, True), (3000, 6, False), (1200, 12, True)]
    return [datasets._plain_problem(rng, n, p, geo, f"b{k}") for k, (n, p, geo) in enumerate(shapes)]


def candidates(pbs, k=5):
    return [np.unique(np.round(np.exp(np.linspace(np.log(pb.p + 20), np.log(pb.n), k)))) for pb in pbs]


def reference(pbs, cands, prec, crit):
    out = []
    for pb, cs in zip(pbs, cands):
        e = Engine(0)
        e.set_data(pb.x, pb.y, pb.coords, pb.geographic)
        e.set_precision(prec)
        out.append(np.array([e.criterion(bw, True, 2, crit) for bw in cs]))
    return out


@pytest.mark.parametrize("prec,crit", [(Precision.Mixed, 0), (Precision.FP64, 0), (Precision.Mixed, 1)])
def test_batch_matches_single_problem_engine(prec, crit):
    pbs = problems()
    cands = candidates(pbs)
    want = reference(pbs, cands, prec, crit)
    b = Batch(pbs, precision=prec)
    b.set_candidates(cands, adaptive=True, kernel=2, criterion=crit)
    got_plain = b.evaluate(use_graph=False)
    got_graph = b.evaluate(use_graph=True)
    got_again = b.evaluate(use_graph=True)
    for w, g1, g2, g3 in zip(want, got_plain, got_graph, got_again):
        np.testing.assert_array_equal(g1, g2)
        np.testing.assert_array_equal(g2, g3)
        assert np.all(np.abs(g1 - w) <= TOL * np.abs(w)), (g1, w)
    info = b.info()
    assert info["graph"] == 1 and info["segments"] == sum(len(c) for c in cands)
    assert info["launches_per_evaluate"] <= 8 if prec == Precision.Mixed else True
    b.close()


def test_autotune_keeps_results():
    pbs = problems()
    cands = candidates(pbs)
    b = Batch(pbs, precision=Precision.Mixed)
    b.set_candidates(cands)
    before = b.evaluate()
    b.autotune(repeats=1)
    info = b.info()
    assert info["tuned"] == 1 and info["tuned_ms"] > 0
    after = b.evaluate()
    for x, y in zip(before, after):
        # the FP32 chunk length may change with the schedule: mixed-path tolerance
        assert np.all(np.abs(x - y) <= 1e-5 * np.abs(y))
    b.close()


def test_batch_rejects_bad_candidates():
    from libgwmodel_gb300._lib import GwgpuError
    pbs = problems()[:2]
    b = Batch(pbs, precision=Precision.Mixed)
    with pytest.raises(GwgpuError):
        b.set_candidates([np.array([10.5]), np.array([20.0])])
    with pytest.raises(GwgpuError):
        b.set_candidates([np.array([pbs[0].n + 1.0]), np.array([20.0])])
    b.close()


def test_first_graph_reads_the_histogram_caches():
    """The graph captured at the first evaluation must carry the histogram
    caches made for it (null cache pointers leave every select scanning whole
    rows: the same values, several times slower).  The replay of the first
    graph is timed against a replay after a rebuild of the same schedule."""
    pbs, cands = datasets.config3()
    b = Batch(pbs, precision=Precision.Mixed)
    b.set_candidates(cands, adaptive=True, kernel=2, criterion=0)
    first = None
    for _ in range(3):
        v0 = b.evaluate(use_graph=True)
        t = b.info()["last_ms"]
        first = t if first is None else min(first, t)
    info = b.info()
    b.set_tuning(info["flush_tiles"], info["order"], info["solve_rows"], info["select_ctas"])
    rebuilt = None
    for _ in range(3):
        v1 = b.evaluate(use_graph=True)
        t = b.info()["last_ms"]
        rebuilt = t if rebuilt is None else min(rebuilt, t)
    for a, c in zip(v0, v1):
        np.testing.assert_array_equal(a, c)
    assert first < 2.0 * rebuilt + 20.0, (first, rebuilt)
