"""Seeded synthetic inputs of the benchmark workloads (the reference ships no data sets).

    burgers_config1()        500-cell Burgers, u0 = exp(-x^2) on [-5, 5]
                             (example/example1_burgers_1d_fv.f90:43-57, LF flux with alpha = 1)
    multi_gaussian_1d(n)     sum of 8 Gaussians on [-5, 5]: amplitudes U(0.2, 1), centres
                             U(-4, 4), widths U(0.05, 0.5), numpy default_rng(seed)
    large_burgers(n, k)      the 2^24-cell Burgers line: multi-Gaussian u0, LF flux with
                             alpha = max|u0|, copy boundaries, dt = CFL dx / max|u0|
    pbe_gaussian_2d(n1, n2)  Gaussian pulse at (0.2, 0.2), sigma 0.05 on [0, 1]^2, x1 fastest
                             (example/example2_pbe_2d_fv.f90:41-52)
    batched_config(nprob)    independent 1D problems: cell counts log-uniform in [64, 65536],
                             half Burgers, half linear advection a ~ U(-1, 1), k in {2, 3},
                             multi-Gaussian u0 in [0, 1], LF flux, per-problem dt at CFL 0.4
"""
from __future__ import annotations

import numpy as np

from .problems import burgers_1d, pbe_2d


def centres(n: int, xmin: float, xmax: float) -> np.ndarray:
    """Cell centres of grid1%linear (src/hrweno_grids.f90:60-79)."""
    return xmin + (xmax - xmin) / n * (np.arange(n) + 0.5)


def burgers_config1(numerics: str = "fast"):
    nc = 500
    prob = burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy",
                      numerics=numerics)
    return prob, np.exp(-centres(nc, -5.0, 5.0) ** 2)


def multi_gaussian_1d(n: int, seed: int = 1, xmin: float = -5.0, xmax: float = 5.0,
                      ngauss: int = 8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.2, 1.0, ngauss)
    cen = rng.uniform(-4.0, 4.0, ngauss)
    sig = rng.uniform(0.05, 0.5, ngauss)
    x = centres(n, xmin, xmax)
    u = np.zeros(n)
    for a, c, s in zip(amp, cen, sig):
        u += a * np.exp(-((x - c) / s) ** 2)
    return u


def large_burgers(n: int = 1 << 24, k: int = 3, cfl: float = 0.4, seed: int = 1,
                  numerics: str = "fast", u0: np.ndarray | None = None):
    """(problem, u0, dt) of the large 1D Burgers line."""
    if u0 is None:
        u0 = multi_gaussian_1d(n, seed)
    amax = float(np.max(np.abs(u0)))
    prob = burgers_1d(n, -5.0, 5.0, k=k, eps=1e-6, flux="lax_friedrichs", alpha=amax, bc="copy",
                      numerics=numerics)
    dt = cfl * (10.0 / n) / amax
    return prob, u0, dt


def pbe_gaussian_2d(n1: int, n2: int, sigma: float = 0.05, centre=(0.2, 0.2)) -> np.ndarray:
    """n0 on [0,1]^2, layout u((j-1)*n1 + i) (x1 fastest), as a flat array."""
    x1 = centres(n1, 0.0, 1.0)
    x2 = centres(n2, 0.0, 1.0)
    g = np.exp(-((x2[:, None] - centre[1]) ** 2 + (x1[None, :] - centre[0]) ** 2)
               / (2 * sigma ** 2))
    return np.ascontiguousarray(g.reshape(-1))


def pbe_config(n1: int, n2: int, cfl: float = 0.4, k: int = 3, bc: str = "zero_inflow",
               numerics: str = "fast"):
    """(problem, n0, dt) of the 2D population-balance case: g1 = 1 + 0.5 x1, g2 = 0.5."""
    prob = pbe_2d(n1, n2, g1=(1.0, 0.5), g2=(0.5, 0.0), k=k, flux="godunov", bc=bc,
                  numerics=numerics)
    dt = cfl / (1.5 * n1 + 0.5 * n2)
    return prob, pbe_gaussian_2d(n1, n2), dt


def batched_config(nprob: int = 4096, seed: int = 7, nmin: int = 64, nmax: int = 65536,
                   cfl: float = 0.4, numerics: str = "fast"):
    """(problems, initial lines, dt per problem) of the batched workload on [-5, 5]."""
    from .problems import Problem
    rng = np.random.default_rng(seed)
    ncs = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nprob)).astype(np.int64)
    probs, lines, dts = [], [], []
    for i in range(nprob):
        n = int(ncs[i])
        k = int(rng.integers(2, 4))
        ng = int(rng.integers(1, 5))
        x = centres(n, -5.0, 5.0)
        u = np.zeros(n)
        for _ in range(ng):
            u += rng.uniform(0.2, 1.0) * np.exp(-((x - rng.uniform(-4, 4)) / rng.uniform(0.1, 1.0)) ** 2)
        u *= 1.0 / max(1.0, float(u.max()))  # u0 in [0, 1]
        if i % 2 == 0:  # Burgers
            alpha = max(float(np.max(np.abs(u))), 1e-3)
            p = Problem(kind="fv1d", ncells=(n, 1), k=k, flux="lax_friedrichs",
                        fn=("burgers", "burgers"), alpha=(alpha, alpha), bc=("copy", "copy"),
                        xmin=(-5.0, 0.0), xmax=(5.0, 1.0), numerics=numerics)
        else:  # linear advection f = a u
            a = float(rng.uniform(-1.0, 1.0))
            alpha = max(abs(a), 1e-3)
            p = Problem(kind="fv1d", ncells=(n, 1), k=k, flux="lax_friedrichs",
                        fn=("linear", "linear"), coef_a=(a, 0.0), coef_b=(0.0, 0.0),
                        alpha=(alpha, alpha), bc=("copy", "copy"), xmin=(-5.0, 0.0),
                        xmax=(5.0, 1.0), numerics=numerics)
        probs.append(p)
        lines.append(u)
        dts.append(cfl * (10.0 / n) / alpha)
    return probs, lines, np.array(dts)
