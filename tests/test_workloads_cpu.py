"""The seeded benchmark workloads are what the measurements say they are (CPU only): cell
counts, flux mix, orders, value ranges and time steps."""
import numpy as np

from hrweno import workloads


def test_batched_workload_definition():
    """4096 lines of log-uniform length in [64, 65536] (38.6M cells with seed 7), half Burgers
    and half linear advection with a in (-1, 1), k in {2, 3}, u0 in [0, 1], Lax-Friedrichs,
    copy boundaries, dt = 0.4 dx / alpha per problem."""
    probs, lines, dts = workloads.batched_config(4096, seed=7)
    n = np.array([p.ncells[0] for p in probs])
    assert n.sum() == 38611538 and n.min() >= 64 and n.max() < 65536
    assert [p.fn[0] for p in probs[:4]] == ["burgers", "linear", "burgers", "linear"]
    assert sum(p.fn[0] == "burgers" for p in probs) == 2048
    assert {p.k for p in probs} == {2, 3}
    assert all(p.flux == "lax_friedrichs" and p.bc == ("copy", "copy") for p in probs)
    assert all(abs(p.coef_a[0]) < 1.0 for p in probs if p.fn[0] == "linear")
    assert all(0.0 <= float(u.min()) and float(u.max()) <= 1.0 for u in lines)
    assert all(u.size == m for u, m in zip(lines, n))
    alpha = np.array([p.alpha[0] for p in probs])
    assert np.allclose(dts, 0.4 * (10.0 / n) / alpha, rtol=0, atol=0)


def test_large_line_workload_definition():
    """The 2^24-cell line: seeded 8-Gaussian u0 on [-5, 5], alpha = max|u0|, CFL 0.4."""
    prob, u0, dt = workloads.large_burgers(1 << 16)  # same construction, smaller line
    assert u0.size == 1 << 16 and prob.ncells[0] == 1 << 16
    assert prob.alpha[0] == float(np.max(np.abs(u0))) and dt == 0.4 * (10.0 / (1 << 16)) / prob.alpha[0]
    assert prob.flux == "lax_friedrichs" and prob.bc[0] == "copy" and prob.k == 3 and prob.eps == 1e-6
    # the same seeded Gaussians at any resolution: the coarse line samples the fine one
    fine = workloads.multi_gaussian_1d(1 << 18)
    coarse = workloads.multi_gaussian_1d(1 << 16)
    assert np.max(np.abs(fine.reshape(-1, 4).mean(1) - coarse)) < 1e-6


def test_pbe_workload_definition():
    """The 2D population balance: g1 = 1 + 0.5 x1, g2 = 0.5, upwind Godunov, zero inflow, a
    Gaussian pulse at (0.2, 0.2) with sigma 0.05, dt = 0.4 / (1.5 n1 + 0.5 n2)."""
    prob, n0, dt = workloads.pbe_config(64, 32)
    assert prob.kind == "fv2d" and prob.ncells == (64, 32) and prob.flux == "godunov"
    assert prob.coef_a == (1.0, 0.5) and prob.coef_b == (0.5, 0.0) and prob.bc == ("zero_inflow",) * 2
    assert dt == 0.4 / (1.5 * 64 + 0.5 * 32)
    g = n0.reshape(32, 64)  # x1 fastest
    j, i = np.unravel_index(np.argmax(g), g.shape)
    assert abs((i + 0.5) / 64 - 0.2) <= 1 / 64 and abs((j + 0.5) / 32 - 0.2) <= 1 / 32
