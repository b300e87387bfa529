"""Seeded synthetic problems shaped like the benchmark configurations.

readme_example: the deterministic example of the reference README
(README.md:111-124): exponential vs. two-normal mixture on linspace grids.
erot_points: n x m squared-Euclidean costs of 3-D Gaussian clouds divided by
their max, uniform(0.5, 1.5) marginals (the large dense EROT workload).
qrot_points: squared-Euclidean costs of uniform points in [0,1]^2 with
Dirichlet(1) marginals floored at 1e-6 (the large QROT workload).
"""
import math

import numpy as np


def _norm_pdf(x, loc, scale):
    return np.exp(-0.5 * ((x - loc) / scale) ** 2) / (scale * math.sqrt(2 * math.pi))


def readme_example(n=100, m=80):
    x1 = np.linspace(0.0, 5.0, num=n)
    x2 = np.linspace(0.0, 5.0, num=m)
    a = np.exp(-x1)  # Exponential(scale=1) pdf on x >= 0
    a = a / np.sum(a)
    b = 0.2 * _norm_pdf(x2, 1.0, 0.2) + 0.8 * _norm_pdf(x2, 3.0, 0.5)
    b = b / np.sum(b)
    M = np.square(x1.reshape(n, 1) - x2.reshape(1, m))
    return M, a, b


def erot_points(n, m, seed=0, dtype=np.float32):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 3))
    y = rng.standard_normal((m, 3)) + 0.5
    a = rng.uniform(0.5, 1.5, n)
    b = rng.uniform(0.5, 1.5, m)
    a /= a.sum()
    b /= b.sum()
    M = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    M /= M.max()
    return M.astype(dtype), a, b


def qrot_points(n, m, seed=1, dtype=np.float32):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, 1.0, (n, 2))
    y = rng.uniform(0.0, 1.0, (m, 2))
    a = np.maximum(rng.dirichlet(np.ones(n)), 1e-6)
    b = np.maximum(rng.dirichlet(np.ones(m)), 1e-6)
    a /= a.sum()
    b /= b.sum()
    M = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    return M.astype(dtype), a, b
