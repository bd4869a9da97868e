"""The reference's example drivers on the GPU path, with their output files.

example1: 1D inviscid Burgers, 500 cells on [-5, 5], u0 = exp(-x^2), WENO5 (eps 1e-6), Godunov
flux, copy boundaries, rktvd order 3, dt = 1e-2, 101 output times to t = 12
(example/example1_burgers_1d_fv.f90:30-66).

example2: 2D population balance, 250^2 cells on [0, 10]^2, f1 = f2 = u (unit velocities),
WENO5, Godunov, closed boundaries, mstvd, dt = 5e-3, 101 output times to t = 5
(example/example2_pbe_2d_fv.f90:25-66).  The initial condition is the example's rectangular
pulse, u0 = 1 on [1, 3]^2 and 0 elsewhere (:157-168), unless the caller passes `u0`.

Each writes its grid files (x.txt; x1.txt and x2.txt) and u.txt in the examples' formats (hrweno.output) through an asynchronous
SnapshotWriter.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .output import SnapshotWriter
from .problems import Problem, burgers_1d
from .tvdode import mstvd, rktvd
from .workloads import centres


def example1(folder, numerics: str = "fast", flux: str = "godunov"):
    """Run example1 on the GPU; returns (t, u) at the end."""
    import torch
    nc = 500
    prob = burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux=flux, alpha=1.0, bc="copy",
                      numerics=numerics)
    x = centres(nc, -5.0, 5.0)
    width = np.full(nc, 10.0 / nc)
    u = torch.from_numpy(np.exp(-x ** 2)).cuda()
    ode = rktvd(prob, nc, 3)
    out = SnapshotWriter(Path(folder), [(x, width)])
    t = 0.0
    try:
        for ii in range(101):
            t = ode.integrate(u, t, 12.0 * ii / 100, 1e-2)
            out.snapshot(t, u)
    finally:
        out.close()
    return t, u.cpu().numpy()


def example2(folder, u0=None, numerics: str = "fast"):
    """Run example2 on the GPU; returns (t, u) at the end."""
    import torch
    n = 250
    prob = Problem(kind="fv2d", ncells=(n, n), k=3, eps=1e-6, flux="godunov",
                   fn=("linear", "linear"), coef_a=(1.0, 1.0), coef_b=(0.0, 0.0),
                   alpha=(1.0, 1.0), bc=("zero", "zero"), xmin=(0.0, 0.0), xmax=(10.0, 10.0),
                   numerics=numerics)
    x = centres(n, 0.0, 10.0)
    if u0 is None:  # u((j-1) n + i) = ic(x1(i), x2(j)), x1 fastest
        inside = (x >= 1.0) & (x <= 3.0)
        u0 = (inside[None, :] & inside[:, None]).astype(np.float64).reshape(-1)
    u = torch.from_numpy(np.ascontiguousarray(u0, dtype=np.float64)).cuda()
    ode = mstvd(prob, n * n)
    out = SnapshotWriter(Path(folder), [(x, np.full(n, 10.0 / n))] * 2)
    t = 0.0
    try:
        for ii in range(101):
            t = ode.integrate(u, t, 5.0 * ii / 100, 5e-3)
            out.snapshot(t, u)
    finally:
        out.close()
    return t, u.cpu().numpy()
