"""Seeded synthetic GWR problems with the shapes of the benchmark workloads.

No public dataset is involved: coordinates, covariates, smooth local
coefficients and noise are drawn from numpy's PCG64 generator with a fixed
seed, so every run and every machine sees the same inputs.

* ``config0``  n=2,000 planar U[0,100]^2, p=5, adaptive bisquare, AICc search
* ``config1``  n=50,000 planar U[0,1000]^2, p=9 (x1, x2 correlated at 0.7),
               sigma=1, fixed gaussian, CV search
* ``config2``  n=200,000 geographic lon U(-10,30), lat U(35,60), p=17 with
               column scales log-uniform over [1e-2, 1e3], adaptive bisquare, AICc
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
