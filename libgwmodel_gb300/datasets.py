"""Seeded synthetic GWR problems with the shapes of the benchmark workloads.

No public dataset is involved: coordinates, covariates, smooth local
coefficients and noise are drawn from numpy's PCG64 generator with a fixed
seed, so every run and every machine sees the same inputs.

* ``config0``  n=2,000 planar U[0,100]^2, p=5, adaptive bisquare, AICc search
* ``config1``  n=50,000 planar U[0,1000]^2, p=9 (x1, x2 correlated at 0.7),
               sigma=1, fixed gaussian, CV search
* ``config2``  n=200,000 geographic lon U(-10,30), lat U(35,60), p=17 with
               column scales log-uniform over [1e-2, 1e3], adaptive bisquare, AICc
* ``config3``  64 independent problems, n log-uniform [500, 20,000], p uniform
               {3..12}, planar coordinates from a mixture of 5 Gaussian clusters,
               32 adaptive bisquare bandwidth candidates each
* ``config4``  a Poisson request stream: 70% fits at a given adaptive bandwidth,
               30% AICc bandwidth searches; n log-uniform [1,000, 100,000], p
               uniform {3..20}, planar or geographic 50/50, data as config 0
* ``multiscale`` n points planar U[0,24]^2, p=3: a global intercept, a
               coefficient that varies over the whole region and one that varies
               locally (the standard multiscale GWR simulation), sigma=0.5
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

KERNELS = {"gaussian": 0, "exponential": 1, "bisquare": 2, "tricube": 3, "boxcar": 4}


@dataclass
class Problem:
    name: str
    x: np.ndarray          # n x p, column 0 is the intercept
    y: np.ndarray          # n
    coords: np.ndarray     # n x 2
    geographic: bool
    adaptive: bool
    kernel: int
    criterion: int         # 0 AIC, 1 CV
    beta_true: np.ndarray = field(repr=False, default=None)

    @property
    def n(self):
        return self.x.shape[0]

    @property
    def p(self):
        return self.x.shape[1]


def _smooth_betas(rng, u, v, p, length):
    a = rng.uniform(-2, 2, p)
    b = rng.uniform(-2, 2, p)
    wave = np.sin(u / length) * np.cos(v / length)
    return a[None, :] + b[None, :] * wave[:, None]


def config0(n=2000, seed=0):
    rng = np.random.default_rng(seed)
    coords = rng.uniform(0, 100, (n, 2))
    x = np.column_stack([np.ones(n), rng.standard_normal((n, 4))])
    beta = _smooth_betas(rng, coords[:, 0], coords[:, 1], 5, 20.0)
    y = (x * beta).sum(1) + rng.normal(0, 0.5, n)
    return Problem("config0", np.asfortranarray(x), y, np.asfortranarray(coords), False, True,
                   KERNELS["bisquare"], 0, beta)


def config1(n=50000, seed=1, rho=0.7):
    rng = np.random.default_rng(seed)
    coords = rng.uniform(0, 1000, (n, 2))
    z = rng.standard_normal((n, 8))
    z[:, 1] = rho * z[:, 0] + np.sqrt(1 - rho * rho) * z[:, 1]
    x = np.column_stack([np.ones(n), z])
    beta = _smooth_betas(rng, coords[:, 0], coords[:, 1], 9, 200.0)
    y = (x * beta).sum(1) + rng.normal(0, 1.0, n)
    return Problem("config1", np.asfortranarray(x), y, np.asfortranarray(coords), False, False,
                   KERNELS["gaussian"], 1, beta)


def config2(n=200000, seed=2, k=16):
    rng = np.random.default_rng(seed)
    lon = rng.uniform(-10, 30, n)
    lat = rng.uniform(35, 60, n)
    coords = np.column_stack([lon, lat])
    scales = np.exp(rng.uniform(np.log(1e-2), np.log(1e3), k))
    x = np.column_stack([np.ones(n), rng.standard_normal((n, k)) * scales[None, :]])
    beta = _smooth_betas(rng, lon * 5.0, lat * 5.0, k + 1, 20.0)
    beta[:, 1:] /= scales[None, :]
    y = (x * beta).sum(1) + rng.normal(0, 0.5, n)
    return Problem("config2", np.asfortranarray(x), y, np.asfortranarray(coords), True, True,
                   KERNELS["bisquare"], 0, beta)


CONFIGS = {"config0": config0, "config1": config1, "config2": config2}


def _plain_problem(rng, n, p, geographic, name):
    """Intercept + (p - 1) N(0,1) covariates, smooth local coefficients, noise 0.5."""
    if geographic:
        coords = np.column_stack([rng.uniform(-10, 30, n), rng.uniform(35, 60, n)])
        u, v, length = coords[:, 0] * 5.0, coords[:, 1] * 5.0, 20.0
    else:
        coords = rng.uniform(0, 100, (n, 2))
        u, v, length = coords[:, 0], coords[:, 1], 20.0
    x = np.column_stack([np.ones(n), rng.standard_normal((n, p - 1))])
    beta = _smooth_betas(rng, u, v, p, length)
    y = (x * beta).sum(1) + rng.normal(0, 0.5, n)
    return Problem(name, np.asfortranarray(x), y, np.asfortranarray(coords), geographic, True,
                   KERNELS["bisquare"], 0, beta)


def config3(seed=3, problems=64, candidates=32):
    """The batched workload: (problems, candidate bandwidths per problem)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0, 1000, (5, 2))
    spread = rng.uniform(20, 120, 5)
    out, cands = [], []
    for q in range(problems):
        n = int(round(np.exp(rng.uniform(np.log(500), np.log(20000)))))
        p = int(rng.integers(3, 13))
        k = rng.integers(0, 5, n)
        coords = centres[k] + rng.standard_normal((n, 2)) * spread[k, None]
        x = np.column_stack([np.ones(n), rng.standard_normal((n, p - 1))])
        beta = _smooth_betas(rng, coords[:, 0], coords[:, 1], p, 150.0)
        y = (x * beta).sum(1) + rng.normal(0, 0.5, n)
        out.append(Problem(f"config3/{q}", np.asfortranarray(x), y, np.asfortranarray(coords), False, True,
                           KERNELS["bisquare"], 0, beta))
        lo, hi = max(p + 2, 20), n
        cands.append(np.unique(np.round(np.exp(np.linspace(np.log(lo), np.log(hi), candidates)))).astype(float))
    return out, cands


@dataclass
class StreamRequest:
    arrival_s: float       # seconds after the stream starts
    problem: Problem
    kind: int              # 0 fit at `bandwidth`, 1 AICc search then fit
    bandwidth: float


def config4(rate, count, seed=4, pool=48, n_min=1000, n_max=100000):
    """`count` requests arriving as a Poisson process of `rate` per second.
    Datasets come from a pool of `pool` seeded problems (a request copies its
    data at submit, so sharing a dataset between requests changes nothing)."""
    rng = np.random.default_rng(seed)
    problems = []
    for q in range(pool):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        p = int(rng.integers(3, 21))
        problems.append(_plain_problem(rng, n, p, bool(rng.integers(0, 2)), f"config4/{q}"))
    t = 0.0
    reqs = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        pb = problems[int(rng.integers(0, pool))]
        kind = 1 if rng.uniform() < 0.3 else 0
        bw = float(rng.integers(max(pb.p + 10, 30), min(300, pb.n - 1) + 1))
        reqs.append(StreamRequest(t, pb, kind, bw))
    return reqs


def multiscale(n=1000, seed=5, geographic=False):
    """Multiscale GWR problem: beta0 = 3 everywhere, beta1 = 1 + (u + v) / 12
    (regional), beta2 = 1 + (36 - (6 - u/2)^2)(36 - (6 - v/2)^2) / 324 (local);
    x1, x2 standard normal.  Geographic: the square mapped onto 24 x 24 degrees
    around lon 10, lat 45."""
    rng = np.random.default_rng(seed)
    uv = rng.uniform(0, 24, (n, 2))
    u, v = uv[:, 0], uv[:, 1]
    beta = np.column_stack([np.full(n, 3.0), 1 + (u + v) / 12,
                            1 + (36 - (6 - u / 2) ** 2) * (36 - (6 - v / 2) ** 2) / 324])
    x = np.column_stack([np.ones(n), rng.standard_normal((n, 2))])
    y = (x * beta).sum(axis=1) + rng.normal(0, 0.5, n)
    coords = np.column_stack([u - 2.0, v + 33.0]) if geographic else uv
    return Problem("multiscale", np.asfortranarray(x), y, np.asfortranarray(coords), geographic, True,
                   KERNELS["bisquare"], 0, beta)
