#!/usr/bin/env python3
"""GWR local fits/s on one GB300: GWRBasic::fit with AICc golden-section
bandwidth search at n = 200,000 geographic points, 16 covariates (+intercept),
adaptive bisquare kernel (the mixed-precision workload; --precision fp64 runs
the FP64 drop-in on the same data).

A step is one whole fit: the golden-section search (every criterion
evaluation) followed by the final fit with its diagnostics outputs.
``value`` times the steps on the device with the data resident in HBM
(CUDA events on the engine's stream); ``e2e`` times the same fit through the
public GWRBasic C ABI from host buffers (the upload of coordinates, X, y and
the download of the outputs inside the timed region).  The unit is local
fits/s = n x (criterion evaluations + 1) / seconds.

The same line carries, measured in the same run: one step of the FP64
drop-in on the same data (``fp64``, ``speedup_vs_fp64``) and the mixed path's
errors against it; the config-4 serving stream at 5, 50 and 200 requests/s in
both forms (``serve``); the config-3 batched evaluation (``batch``); the CPU
baseline (the oracle on a bounded sample of rows).

    python bench.py [--steps K] [--warmup W] [--precision mixed|fp64] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GWR local fits/s, n=200k k=16 geographic adaptive bisquare AICc search (mixed vs FP64)"
UNIT = "local fits/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--n", type=int, default=200000, help="points (smaller values for profiling only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the config-4 serving block of the main line")
    ap.add_argument("--no-batch", action="store_true", help="skip the config-3 batch block of the main line")
    ap.add_argument("--no-fp64", action="store_true", help="skip the live FP64 drop-in step of the main line")
    ap.add_argument("--serve", action="store_true", help="config-4 serving sweep instead of the config-2 line")
    ap.add_argument("--batch", action="store_true", help="config-3 batched evaluation instead of the config-2 line")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--config1", action="store_true", help="config-1 FP64 drop-in line instead of the config-2 line")
    ap.add_argument("--mgwr", action="store_true", help="GWRMultiscale back-fitting line instead of the config-2 line")
    ap.add_argument("--mgwr-n", type=int, default=20000)
    ap.add_argument("--mgwr-hat-n", type=int, default=4000)
    ap.add_argument("--mgwr-iterations", type=int, default=10)
    ap.add_argument("--rates", default="5,50,200")
    ap.add_argument("--requests", type=int, default=200, help="requests per rate (mixed form)")
    ap.add_argument("--requests-fp64", type=int, default=200, help="requests per rate (FP64 form)")
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--precision-serve", choices=["mixed", "fp64", "both"], default="both")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def ncu_traffic_per_tile(name):
    """DRAM bytes per processed 32-point tile of the contraction, from the committed
    ncu summary (a one-launch capture of the config-2 workload; the traffic grows
    with the tiles processed: every visited tile streams its distance block)."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = re.search(r"traffic_bytes_per_tile:\s*([0-9.eE+]+)", f.read())
    return float(m.group(1)) if m else None


def rel_err(a, b):
    """Largest absolute difference over the largest magnitude, per column."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 1:
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
    return max(float(np.abs(a[:, k] - b[:, k]).max() / max(np.abs(b[:, k]).max(), 1e-300)) for k in range(a.shape[1]))


def elem_rel(a, b, floor=1e-3):
    """Per-element relative error |a - b| / |b| over the elements of each column
    with |b| >= floor x the column's largest |b|: quantiles and maximum."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.ndim == 1:
        a, b = a[:, None], b[:, None]
    r = []
    for k in range(b.shape[1]):
        m = np.abs(b[:, k]) >= floor * np.abs(b[:, k]).max()
        r.append(np.abs(a[m, k] - b[m, k]) / np.abs(b[m, k]))
    r = np.concatenate(r)
    return {"p50": float(np.quantile(r, 0.5)), "p99": float(np.quantile(r, 0.99)),
            "p999": float(np.quantile(r, 0.999)), "max": float(r.max()), "elements": int(r.size),
            "floor": floor}


def accuracy_vs_fp64(engine, e64, pb, bw, out64):
    """Errors of the mixed path against the FP64 drop-in at the FP64 search's
    bandwidth: beta, betasSE, tr(S), tr(S^T S), qDiag and the AICc value."""
    b64, se64, sh64, q64, _ = out64
    c64 = e64.criterion(bw, True, pb.kernel, 0)
    bmx, semx, shmx, qmx, _ = engine.fit(bw, True, pb.kernel, store_s=False)
    cmx = engine.criterion(bw, True, pb.kernel, 0)
    return {"bandwidth": bw, "beta_rel": rel_err(bmx, b64), "betasSE_rel": rel_err(semx, se64),
            "trS_rel": abs(shmx[0] - sh64[0]) / abs(sh64[0]), "trStS_rel": abs(shmx[1] - sh64[1]) / abs(sh64[1]),
            "qdiag_rel": rel_err(qmx, q64), "aicc_rel": abs(cmx - c64) / abs(c64), "beta_tolerance": 1e-6,
            "beta_elementwise": elem_rel(bmx, b64), "betasSE_elementwise": elem_rel(semx, se64),
            "note": "*_rel: max |mixed - fp64| / max |fp64| per column; *_elementwise: |mixed - fp64| / |fp64| "
                    "per element with |fp64| >= 1e-3 of its column's largest; same bandwidth (the FP64 "
                    "search's), FP64 drop-in as the reference"}


def fp64_step(pb, local):
    """One step of the FP64 drop-in on the same workload (golden search + fit),
    timed with CUDA events on its engine's stream, clocks sampled."""
    from libgwmodel_gb300 import Engine, Precision
    e64 = Engine(local)
    e64.set_data(pb.x, pb.y, pb.coords, pb.geographic)
    e64.set_precision(Precision.FP64)
    e64.enable_stats(True)
    clocks = Clocks(local)
    clocks.start()
    e64.record_event(0)
    bw, crit, out = one_fit(e64, pb)
    e64.record_event(1)
    ms = e64.elapsed_ms(0, 1)
    clk = clocks.stop()
    st = e64.stats()
    info = {"ms_per_step": ms, "selected_bandwidth": bw, "criterion_evals": st["criterion_evals"],
            "contract_ms": st["contract_ms"], "select_ms": st["select_ms"], "clocks": clk,
            "timing": "one step, CUDA events on the FP64 engine's stream (data resident)"}
    return info, e64, out


def serve_stream(rate, count, precision, slots=8, budget_gb=150.0, seed=4, budget_x_largest=None):
    """Config 4: replay a Poisson request stream through the serving loop and
    report latency percentiles (submit to result) and throughput.  With
    budget_x_largest the HBM budget is that multiple of the largest request's
    admission estimate (admission under memory pressure)."""
    from libgwmodel_gb300 import datasets
    from libgwmodel_gb300.serve import Server, percentile, run_stream
    reqs = datasets.config4(rate, count, seed=seed)
    if budget_x_largest:
        probe = Server(0, hbm_budget_gb=budget_gb, slots=slots)
        largest = max(probe.estimate(r.problem, kind=r.kind, bandwidth=r.bandwidth, precision=precision) for r in reqs)
        big = max((r.problem for r in reqs), key=lambda pb: pb.n * pb.p)
        largest = max(largest, probe.estimate(big, kind=0, bandwidth=50.0, precision=precision))  # the warm-up's
        probe.close()
        budget_gb = budget_x_largest * largest / 1e9
    srv = Server(0, hbm_budget_gb=budget_gb, slots=slots)
    # warm-up: every slot grows its buffers to the largest dataset of the pool once
    big = max((r.problem for r in reqs), key=lambda pb: pb.n * pb.p)
    ids = [srv.submit(big, kind=0, bandwidth=50.0, precision=precision) for _ in range(slots)]
    for i in ids:
        srv.wait(i)
    warm = srv.stats()
    out, wall = run_stream(srv, reqs, precision=precision)
    st = srv.stats()
    srv.close()
    ok = [r for r, _ in out if r["status"] == 0]
    lat = [r["end_ms"] - r["submit_ms"] for r in ok]
    fits = sum(rq.problem.n * (r["evaluations"] + 1) for rq, (r, _) in zip(reqs, out) if r["status"] == 0)
    searches = [r["end_ms"] - r["submit_ms"] for rq, (r, _) in zip(reqs, out) if r["status"] == 0 and rq.kind == 1]
    return {"rate_req_s": rate, "requests": count, "completed": len(ok), "failed": count - len(ok),
            "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "mean_ms": float(np.mean(lat)) if lat else 0,
            "search_p50_ms": percentile(searches, 50), "search_p99_ms": percentile(searches, 99),
            "wall_s": wall, "requests_per_s": len(ok) / wall, "local_fits_per_s": fits / wall,
            "max_concurrent": st["max_concurrent"], "peak_reserved_gb": st["peak_reserved_bytes"] / 1e9,
            "budget_gb": budget_gb, "rejected": int(st["rejected"]), "warmup_requests": int(warm["completed"])}


def serve_block(rates, requests, precisions):
    """Config 4 inside the main line: the request stream at each rate, per form."""
    from libgwmodel_gb300 import Precision
    out = {}
    for pr in precisions:
        prec = Precision.Mixed if pr == "mixed" else Precision.FP64
        out[pr] = [serve_stream(r, requests[pr], prec) for r in rates]
    return out


def batch_block(precision, steps, warmup, autotune=True):
    """Config 3 inside the main line: evaluations/s of the batched launch and its
    largest relative difference against the one-problem-at-a-time engine."""
    from libgwmodel_gb300 import Engine, Precision, datasets
    from libgwmodel_gb300.batch import Batch
    prec = Precision.Mixed if precision == "mixed" else Precision.FP64
    pbs, cands = datasets.config3()
    b = Batch(pbs, precision=prec)
    b.set_candidates(cands, adaptive=True, kernel=2, criterion=0)
    t0 = time.perf_counter()
    if autotune:
        b.autotune(repeats=2)
    tune_s = time.perf_counter() - t0
    for _ in range(warmup):
        b.evaluate(use_graph=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        vals = b.evaluate(use_graph=True)  # replays the graph and reads the values back
    dt = (time.perf_counter() - t0) / steps
    info = b.info()
    seq = []
    for pb, cs in zip(pbs, cands):
        e = Engine(0)
        e.set_data(pb.x, pb.y, pb.coords, pb.geographic)
        e.set_precision(prec)
        e.criterion(cs[0], True, 2, 0)
        seq.append((e, cs))
    t0 = time.perf_counter()
    ref = [np.array([e.criterion(bw, True, 2, 0) for bw in cs]) for e, cs in seq]
    seq_s = time.perf_counter() - t0
    err = max(float(np.max(np.abs(v - r) / np.abs(r))) for v, r in zip(vals, ref))
    return {"evaluations_per_s": info["segments"] / dt, "ms_per_step": dt * 1e3, "evaluations": info["segments"],
            "local_fits_per_s": info["rows_total"] / dt, "precision": precision, "graph": info["graph"],
            "launches_per_step": info["launches_per_evaluate"], "autotune_s": tune_s,
            "schedule": {k: info[k] for k in ("flush_tiles", "order", "solve_rows", "select_ctas", "tuned")},
            "sequential_ms": seq_s * 1e3, "speedup_vs_sequential": seq_s / dt, "max_rel_diff_vs_sequential": err,
            "workload": "config3: 64 problems, n log-uniform [500, 20000], p in 3..12, 5 Gaussian clusters, "
                        "32 adaptive bisquare candidates each, AICc; one evaluation of every (problem, candidate) "
                        "per step under a captured CUDA graph",
            "timing": "host wall clock around evaluate(), which replays the graph and copies the values back"}


def run_batch(args):
    """Config 3: 64 problems x 32 adaptive bisquare candidates (AICc), one launch
    per phase under a captured CUDA graph, schedule autotuned on the batch;
    beside it the same evaluations one criterion call at a time."""
    rank, _, _ = dist_env()
    if rank != 0:
        return 0
    from libgwmodel_gb300 import Engine, Precision, datasets
    from libgwmodel_gb300.batch import Batch
    prec = Precision.Mixed if args.precision == "mixed" else Precision.FP64
    pbs, cands = datasets.config3()
    b = Batch(pbs, precision=prec)
    b.set_candidates(cands, adaptive=True, kernel=2, criterion=0)
    t0 = time.perf_counter()
    if not args.no_autotune:
        b.autotune(repeats=2)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.evaluate(use_graph=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals = b.evaluate(use_graph=True)
    dt = (time.perf_counter() - t0) / args.steps
    info = b.info()
    segs = info["segments"]
    fits = info["rows_total"]
    # the same criterion values one call at a time through per-problem engines
    t0 = time.perf_counter()
    seq = []
    for pb, cs in zip(pbs, cands):
        e = Engine(0)
        e.set_data(pb.x, pb.y, pb.coords, pb.geographic)
        e.set_precision(prec)
        e.criterion(cs[0], True, 2, 0)  # histogram cache, as the batch has it
        seq.append((e, pb, cs))
    prep_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = [np.array([e.criterion(bw, True, 2, 0) for bw in cs]) for e, pb, cs in seq]
    seq_s = time.perf_counter() - t0
    err = max(float(np.max(np.abs(v - r) / np.abs(r))) for v, r in zip(vals, ref))
    best = [float(c[int(np.argmin(v))]) for c, v in zip(cands, vals)]
    line = {"metric": "GWR batched criterion evaluations, config 3 (64 problems x 32 candidates)",
            "value": segs / dt, "unit": "criterion evaluations/s", "higher_is_better": True, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "precision": args.precision,
            "local_fits_per_s": fits / dt, "dtype": "tf32x3+f64" if prec == Precision.Mixed else "f64",
            "data": "synthetic (seeded config-3 generator, numpy PCG64 seed 3)",
            "config": {"workload": "config3: 64 problems, n log-uniform [500, 20000], p in 3..12, 5 Gaussian "
                                   "clusters, 32 adaptive bisquare candidates each, AICc"},
            "schedule": {k: info[k] for k in ("flush_tiles", "order", "solve_rows", "select_ctas", "tuned")},
            "autotune_s": tune_s, "graph": info["graph"], "launches_per_step": info["launches_per_evaluate"],
            "contract_ctas": info["contract_ctas"],
            "sequential_ms": seq_s * 1e3, "speedup_vs_sequential": seq_s / dt,
            "max_rel_diff_vs_sequential": err, "best_bandwidth_first5": best[:5]}
    print(json.dumps(line), flush=True)
    return 0


def run_config1(args):
    """Config 1: the FP64 drop-in on n = 50,000 planar points, fixed gaussian
    kernel, CV golden-section search over [0, maxDistance] then the fit, beside
    the CPU restatement of the reference on a bounded sample of rows."""
    rank, _, local = dist_env()
    if rank != 0:
        return 0
    from libgwmodel_gb300 import Engine, Precision, datasets
    pb = datasets.config1()
    e = Engine(local)
    e.set_data(pb.x, pb.y, pb.coords, False)
    e.set_precision(Precision.FP64)
    e.enable_stats(True)
    upper = e.max_distance()
    for _ in range(args.warmup):
        e.clear_cache()
        e.golden(False, 0, 1, 0.0, upper)
    e.reset_stats()
    e.record_event(0)
    for _ in range(args.steps):
        e.clear_cache()
        bw, _ = e.golden(False, 0, 1, 0.0, upper)
        e.fit(bw, False, 0, store_s=False)
    e.record_event(1)
    ms = e.elapsed_ms(0, 1) / args.steps
    st = e.stats()
    evals = st["criterion_evals"] / args.steps
    value = pb.n * (evals + 1) / (ms / 1e3)
    line = {"metric": "GWR local fits/s, config 1 FP64 drop-in (n=50k planar, fixed gaussian, CV search)",
            "value": value, "unit": UNIT, "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "dtype": "f64",
            "data": "synthetic (seeded config-1 generator, numpy PCG64 seed 1)",
            "config": {"workload": "config1: n=50000 planar U[0,1000]^2, p=9 (x1,x2 rho=0.7), fixed gaussian, "
                                   "CV golden search over [0, maxDistance] + fit", "criterion_evals_per_step": evals,
                       "selected_bandwidth": bw},
            "gpu_launches": int(st["kernel_launches"]),
            "contract_tflops": st["contract_flops"] / (st["contract_ms"] / 1e3) / 1e12 if st["contract_ms"] else 0}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        prob = O.Problem(pb.x, pb.y, pb.coords, geographic=False, threads=threads)
        rows = threads * 4
        t0 = time.perf_counter()
        prob.criterion_rows(bw, False, 0, 1, 0, rows)
        dt = time.perf_counter() - t0
        rows = min(pb.n, max(rows, int(rows * min(args.cpu_seconds, 20.0) / max(dt, 1e-6))))
        t0 = time.perf_counter()
        prob.criterion_rows(bw, False, 0, 1, 0, rows)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": rows / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{rows} local fits of the CV criterion at bandwidth {bw:.4g} in {dt:.1f}s"}
    print(json.dumps(line), flush=True)
    return 0


def mgwr_fit(pb, hat, iterations, precision=0):
    """One GWRMultiscale fit through the public C ABI from host buffers:
    p = 3, adaptive bisquare, AICc searches, Null initialisation, the last two
    predictors centred, back-fitting capped at `iterations`."""
    from libgwmodel_gb300 import BandwidthWeight, CRSDistance, SpatialWeight
    from libgwmodel_gb300.mgwr import GWRMultiscale
    alg = GWRMultiscale()
    alg.setCoords(pb.coords)
    alg.setDependentVariable(pb.y)
    alg.setIndependentVariables(pb.x)
    alg.setSpatialWeights([SpatialWeight(BandwidthWeight(0, True, BandwidthWeight.Bisquare),
                                         CRSDistance(pb.geographic)) for _ in range(pb.p)])
    alg.setHasHatMatrix(hat)
    alg.setPreditorCentered([False] + [True] * (pb.p - 1))
    alg.setBandwidthInitilize([GWRMultiscale.Null] * pb.p)
    alg.setBandwidthSelectionApproach([GWRMultiscale.AIC] * pb.p)
    alg.setBandwidthSelectThreshold([1e-5] * pb.p)
    alg.setMaxIteration(iterations)
    alg.setPrecision(precision)
    t0 = time.perf_counter()
    alg.fit()
    dt = time.perf_counter() - t0
    return alg, dt


def run_mgwr(args):
    """GWRMultiscale (GWRMultiscale.cpp:68-317) on the seeded multiscale problem:
    the whole fit (initial searches, all-variable search and fit, back-fitting
    with a golden search and a fit per variable per iteration) timed through
    the C ABI, beside the oracle's per-variable criterion on the host cores."""
    rank, _, _ = dist_env()
    if rank != 0:
        return 0
    from libgwmodel_gb300 import datasets
    pb = datasets.multiscale(args.mgwr_n, seed=13)
    for _ in range(max(args.warmup, 1)):
        mgwr_fit(datasets.multiscale(2000, seed=14), False, 2)
    clocks = Clocks(0)
    clocks.start()
    times, alg = [], None
    for _ in range(args.steps):
        alg, dt = mgwr_fit(pb, False, args.mgwr_iterations)
        times.append(dt)
    clk = clocks.stop()
    c = alg.counters()
    sec = float(np.median(times))
    value = pb.n * (c["criterion_evals"] + c["fits"]) / sec
    bws = alg.bandwidths().tolist()
    line = {"metric": "GWRMultiscale local fits/s (n=20k planar, p=3, adaptive bisquare, AICc searches)",
            "value": value, "unit": UNIT, "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "dtype": "f64", "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded multiscale generator, numpy PCG64 seed 13)",
            "config": {"workload": f"multiscale: n={pb.n} planar U[0,24]^2, p=3 (global, regional, local "
                                   f"coefficients), adaptive bisquare, AICc golden searches, Null initial "
                                   f"bandwidths, back-fitting capped at {args.mgwr_iterations} iterations, "
                                   f"no hat matrix",
                       "bandwidths": bws, "initial_bandwidth": alg.initialBandwidth(),
                       "iterations": alg.iterations(), "criterion_evals": c["criterion_evals"], "fits": c["fits"],
                       "phase_seconds": {"search": c["search_s"], "fit": c["fit_s"]},
                       "timing": "host wall clock around fit() (a synchronous call)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(pb.n * (pb.p + 3) * 8),
                    "d2h_bytes_per_step": int(pb.n * pb.p * 8 * (c["fits"]))},
            "gpu_launches": c["kernel_launches"], "clocks": clk}
    # the same fit with the tensor-core criterion in the searches (fits stay FP64)
    am, dtm = mgwr_fit(pb, False, args.mgwr_iterations, precision=1)
    cm = am.counters()
    line["mixed"] = {"seconds": dtm, "value": pb.n * (cm["criterion_evals"] + cm["fits"]) / dtm,
                     "bandwidths": am.bandwidths().tolist(), "iterations": am.iterations(),
                     "criterion_evals": cm["criterion_evals"],
                     "max_abs_beta_diff_vs_fp64": float(np.abs(am.betas() - alg.betas()).max())}
    # hat-matrix form on a smaller n: (p + 3) n^2 doubles resident, one DGEMM per variable update
    if args.mgwr_hat_n > 0:
        ph = datasets.multiscale(args.mgwr_hat_n, seed=15)
        ah, dth = mgwr_fit(ph, True, args.mgwr_iterations)
        ch = ah.counters()
        nn = float(ph.n) ** 3
        line["hat"] = {"n": ph.n, "seconds": dth, "iterations": ah.iterations(), "bandwidths": ah.bandwidths().tolist(),
                       "hat_updates": ch["hat_updates"], "hat_seconds": ch["hat_s"],
                       "dgemm_tflops": 2 * nn * ch["hat_updates"] / ch["hat_s"] / 1e12 if ch["hat_s"] else None,
                       "AICc": ah.diagnostic().AICc, "phase_seconds": {"search": ch["search_s"], "fit": ch["fit_s"],
                                                                       "hat": ch["hat_s"]}}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        # the reference's per-variable criterion (GWRMultiscale.cpp:560-638) on variable 2 at its selected bandwidth
        k = 2
        xk = np.asfortranarray(pb.x[:, k:k + 1] - pb.x[:, k].mean())
        prob = O.Problem(xk, pb.y, pb.coords, geographic=False, threads=threads)
        bw = float(bws[k])
        rows = threads * 8
        t0 = time.perf_counter()
        prob.criterion_rows(bw, True, 2, 0, 0, rows)
        dt = time.perf_counter() - t0
        rows = min(pb.n, max(rows, int(rows * min(args.cpu_seconds, 20.0) / max(dt, 1e-6))))
        t0 = time.perf_counter()
        prob.criterion_rows(bw, True, 2, 0, 0, rows)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": rows / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{rows} local fits of the per-variable AICc criterion (p=1, bandwidth "
                                          f"{int(bw)} of n={pb.n}) in {dt:.1f}s with {threads} OpenMP threads"}
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args):
    rank, _, _ = dist_env()
    if rank != 0:
        return 0
    from libgwmodel_gb300 import Precision
    precs = ["mixed", "fp64"] if args.precision_serve == "both" else [args.precision_serve]
    rates = [float(r) for r in args.rates.split(",")]
    for pr in precs:
        prec = Precision.Mixed if pr == "mixed" else Precision.FP64
        count = args.requests if pr == "mixed" else args.requests_fp64
        rows = [serve_stream(r, count, prec, slots=args.slots) for r in rates]
        line = {"metric": "GWR serving latency, config-4 request stream (70% fits, 30% AICc searches)",
                "value": rows[0]["p99_ms"], "unit": "ms (p99, first rate)", "higher_is_better": False,
                "n_gpus": 1, "precision": pr, "slots": args.slots, "hbm_budget_gb": 150.0,
                "data": "synthetic (seeded config-4 generator, numpy PCG64 seed 4)",
                "config": {"workload": "config4: Poisson arrivals; n log-uniform [1e3, 1e5], p in 3..20, "
                                       "planar/geographic 50/50, adaptive bisquare"},
                "rates": rows}
        print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(value, dist):
    """The largest value over all ranks (the slowest replica sets the time)."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def d2_cache_bytes(n):
    """Size of the distance cache: 128-row blocks x 32-point tiles x 16 KB."""
    return ((n + 127) // 128) * ((n + 31) // 32) * 128 * 32 * 4


def one_fit(engine, pb):
    """GWRBasic::fit body on resident data: golden search, then the final fit.
    Every step starts from empty caches: nothing computed by an earlier step
    (order statistics, distance histograms, the distance cache) is reused."""
    engine.clear_cache()
    lower, upper = 20.0, float(pb.n)  # GWRBasic.cpp:78-79 for adaptive bandwidths
    bw, crit = engine.golden(True, pb.kernel, 0, lower, upper)
    out = engine.fit(bw, True, pb.kernel, store_s=False)
    return bw, crit, out


def e2e_fit(pb, precision):
    from libgwmodel_gb300 import BandwidthWeight, CRSDistance, GWRBasic, SpatialWeight
    alg = GWRBasic()
    alg.setCoords(pb.coords)
    alg.setDependentVariable(pb.y)
    alg.setIndependentVariables(pb.x)
    alg.setSpatialWeight(SpatialWeight(BandwidthWeight(0, True, BandwidthWeight.Bisquare), CRSDistance(True)))
    alg.setIsAutoselectBandwidth(True)
    alg.setBandwidthSelectionCriterion(GWRBasic.AIC)
    alg.setPrecision(precision)
    betas = alg.fit()
    return alg, betas


def cpu_baseline(pb, seconds, threads=None):
    """The oracle (a C/OpenMP restatement of GWRBasic's criterion loop,
    GWRBasic.cpp:487-535) on a bounded sample of rows at the first golden
    bandwidth, with the reference's libm great-circle formula."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = threads or os.cpu_count() or 1
    prob = O.Problem(pb.x, pb.y, pb.coords, geographic=pb.geographic, threads=threads)
    bw = float(np.floor(20 + (np.sqrt(5) - 1) / 2 * (pb.n - 20)))
    rows = threads
    t0 = time.perf_counter()
    prob.criterion_rows(bw, True, pb.kernel, 0, 0, rows)
    dt = time.perf_counter() - t0
    rows2 = max(rows, int(rows * seconds / max(dt, 1e-6)))
    rows2 = min(rows2, pb.n)
    t0 = time.perf_counter()
    prob.criterion_rows(bw, True, pb.kernel, 0, 0, rows2)
    dt = time.perf_counter() - t0
    return {"value": rows2 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{rows2} local fits of one AICc criterion evaluation (bandwidth {int(bw)} of n={pb.n}) "
                      f"in {dt:.1f}s with {threads} OpenMP threads; a local fit costs the same at every golden "
                      f"bandwidth in the reference (full sort + n-length products), so rows/s is fits/s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from libgwmodel_gb300 import datasets
    pb = datasets.config2(n=args.n)
    vals = []
    base = None
    for _ in range(args.steps):
        base = cpu_baseline(pb, seconds=min(args.cpu_seconds, 20.0))
        vals.append(base["value"])
    value = float(np.mean(vals))
    base["value"] = value
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded config-2 generator)", "impl": "reference",
            "config": {"workload": f"config2: n={pb.n} geographic, p={pb.p}, adaptive bisquare, AICc golden search",
                       "cpu_sample": "bounded"},
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    rank, world, local = dist_env()
    from libgwmodel_gb300 import Engine, Precision, datasets
    prec = Precision.Mixed if args.precision == "mixed" else Precision.FP64
    pb = datasets.config2(n=args.n)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo")
        dist = dist_mod
    engine = Engine(local)
    engine.set_data(pb.x, pb.y, pb.coords, pb.geographic)
    engine.set_precision(prec)
    engine.enable_stats(True)
    for _ in range(args.warmup):
        one_fit(engine, pb)
    engine.reset_stats()
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    clocks.start()
    engine.record_event(0)
    results = []
    for _ in range(args.steps):
        results.append(one_fit(engine, pb))
    engine.record_event(1)
    ms = engine.elapsed_ms(0, 1)
    clk = clocks.stop()
    stats = engine.stats()
    ms = max_over_ranks(ms, dist)
    evals = stats["criterion_evals"] / args.steps
    fits_per_step = pb.n * (evals + 1)
    value = world * fits_per_step * args.steps / (ms / 1e3)
    bw = results[-1][0]

    # e2e through the public C ABI (host buffers in, outputs out)
    e2e = None
    if not args.no_e2e:
        # warm-up of the facade path; kept alive so the device's distance cache
        # passes from engine to engine instead of being freed and allocated again
        warm = e2e_fit(pb, prec)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            alg, _ = e2e_fit(pb, prec)
        dt = time.perf_counter() - t0
        warm = alg = None  # frees the distance cache with its last owner
        n, p = pb.n, pb.p
        e2e = {"value": world * fits_per_step * args.steps / dt, "unit": UNIT,
               "h2d_bytes_per_step": 8 * n * (2 + p + 1),
               "d2h_bytes_per_step": 8 * n * (2 * p + 2)}

    hbm, bf16, src = peaks()
    tf32_peak = bf16 / 2.0
    achieved = stats["contract_flops"] / (stats["contract_ms"] / 1e3) / 1e12 if stats["contract_ms"] else 0.0
    per_tile = ncu_traffic_per_tile("contract_tc_config2.md") if prec == Precision.Mixed else None
    tiles_per_launch = stats["contract_tiles"] / max(stats["contract_launches"], 1)
    traffic = per_tile * tiles_per_launch if per_tile else None
    launch_s = stats["contract_ms"] / 1e3 / max(stats["contract_launches"], 1)
    if prec == Precision.Mixed:
        roof = {"bound": "tensor", "achieved": achieved, "peak": tf32_peak, "unit": "TFLOP/s",
                "frac": achieved / tf32_peak, "traffic": traffic,
                "traffic_note": "DRAM bytes per processed tile from the ncu capture of the first config-2 launch "
                                "(profiles/contract_tc_config2.md) x mean tiles per launch of this step",
                "tiles_per_launch": tiles_per_launch,
                "dram_gbs": traffic / launch_s / 1e9 if traffic and launch_s > 0 else None,
                "dram_frac_of_measured_hbm": traffic / launch_s / 1e9 / hbm if traffic and launch_s > 0 else None,
                "kernel": "k_contract_tc (tcgen05 TF32x3 W.Z)",
                "note": f"useful 2*m*P FLOPs (m=170, P=nonzero-weight pairs) / event-timed launch; peak = {src} "
                        f"bf16 burst {bf16:.0f} TF/s halved for dense TF32"}
    else:
        roof = {"bound": "tensor", "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
                "frac": achieved / 1.25, "traffic": None, "kernel": "k_contract64 (FP64 SIMT W.Z)",
                "note": "FP64 pipe bound; peak = nominal 1.25 TF/s FP64 (no measured FP64 peak)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "tf32x3+f64" if prec == Precision.Mixed else "f64",
            "data": "synthetic (seeded config-2 generator, numpy PCG64 seed 2)",
            "config": {"workload": f"config2: n={pb.n} geographic lon U(-10,30) lat U(35,60), p={pb.p}, "
                                   f"adaptive bisquare, AICc golden-section search + final fit",
                       "precision": args.precision, "criterion_evals_per_step": evals,
                       "selected_bandwidth": bw, "l2": "inputs larger than L2 (Z tiles 300 MB; the distance cache, n^2 x 4 B, refilled every step)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": int(stats["kernel_launches"]),
            "roofline": roof,
            "select_ms_per_step": stats["select_ms"] / args.steps,
            "contract_ms_per_step": stats["contract_ms"] / args.steps,
            "distance_cache": {"fills_per_step": stats["d2c_fills"] / args.steps,
                               "fill_ms_per_step": stats["d2c_fill_ms"] / args.steps,
                               "bytes": d2_cache_bytes(pb.n) if stats["d2c_fills"] else 0}}
    if e2e:
        line["e2e"] = e2e
    if clk:
        line["clocks"] = clk
    if prec == Precision.Mixed and rank == 0 and not args.no_fp64:
        # the FP64 drop-in on the same workload, measured in this run: the >= 5x target's denominator
        engine.release_distance_cache()
        f64, e64, out64 = fp64_step(pb, local)
        line["fp64"] = f64
        line["fp64_ms_per_step"] = f64["ms_per_step"]
        line["speedup_vs_fp64"] = f64["ms_per_step"] / (ms / args.steps)
        line["same_bandwidth_as_fp64"] = f64["selected_bandwidth"] == bw
        if not args.no_accuracy:
            line["accuracy_vs_fp64"] = accuracy_vs_fp64(engine, e64, pb, f64["selected_bandwidth"], out64)
        e64 = out64 = None
    engine.release_distance_cache()
    engine = None
    if rank == 0 and not args.no_serve:
        rates = [float(r) for r in args.rates.split(",")]
        line["serve"] = serve_block(rates, {"mixed": args.requests, "fp64": args.requests_fp64},
                                    ["mixed", "fp64"] if args.precision_serve == "both" else [args.precision_serve])
        from libgwmodel_gb300 import Precision as _P
        # the same stream at 50 req/s under memory pressure: budget = 2.5 x the largest request's estimate
        line["serve"]["mixed_budget_pressure"] = serve_stream(50.0, args.requests, _P.Mixed, budget_x_largest=2.5)
        line["serve"]["note"] = ("config 4: Poisson arrivals, 70% fits at a given adaptive bandwidth / 30% AICc "
                                 "searches, n log-uniform [1e3, 1e5], p 3..20, planar/geographic 50/50, 150 GB "
                                 "budget (mixed_budget_pressure: 2.5 x the largest request's estimate), 8 slots; "
                                 "latency = submit to result")
    if rank == 0 and not args.no_batch:
        line["batch"] = batch_block("mixed", steps=5, warmup=2)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(pb, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.serve:
        return run_serve(args)
    if args.batch:
        return run_batch(args)
    if args.config1:
        return run_config1(args)
    if args.mgwr:
        return run_mgwr(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
