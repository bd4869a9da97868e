"""Full-size (2^24 cells) checks of the 1D path: oracle parity over a few steps, plus
size-independent properties over longer runs (conservation, invariance of constant states)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 24


def multi_gaussian(n, seed=1, xmin=-5.0, xmax=5.0):
    """u0 = sum of 8 Gaussians, amplitudes U(0.2,1), centres U(-4,4), widths U(0.05,0.5)."""
    rng = np.random.default_rng(seed)
    amp, cen, sig = rng.uniform(0.2, 1.0, 8), rng.uniform(-4, 4, 8), rng.uniform(0.05, 0.5, 8)
    x = xmin + (xmax - xmin) / n * (np.arange(n) + 0.5)
    u = np.zeros(n)
    for a, c, s in zip(amp, cen, sig):
        u += a * np.exp(-((x - c) / s) ** 2)
    return u


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def u0():
    return multi_gaussian(N)


@pytest.mark.parametrize("k", [2, 3])
def test_full_size_oracle_parity(hw, orc, u0, k):
    """Two RK3 steps at CFL 0.4 on 2^24 cells: STRICT bit-exact, FAST within 1e-12."""
    import torch
    alpha = float(np.max(np.abs(u0)))
    dt = 0.4 * (10.0 / N) / alpha
    for numerics in ("strict", "fast"):
        prob = hw.burgers_1d(N, -5.0, 5.0, k=k, alpha=alpha, numerics=numerics)
        ug = torch.from_numpy(u0).cuda()
        hw.rktvd(prob, N, 3).integrate(ug, 0.0, 1.5 * dt, dt)
        uo = u0.copy()
        orc.ODE(prob, N, 0, 3).integrate(uo, 0.0, 1.5 * dt, dt)
        got = ug.cpu().numpy()
        if numerics == "strict":
            assert np.array_equal(got, uo)
        else:
            assert nrel(got, uo) <= 1e-12


def test_full_size_conservation(hw, u0):
    """Zero boundary fluxes: sum(u) is conserved to rounding over 200 steps."""
    import torch
    alpha = float(np.max(np.abs(u0)))
    dt = 0.4 * (10.0 / N) / alpha
    prob = hw.burgers_1d(N, -5.0, 5.0, k=3, alpha=alpha, bc="zero")
    ug = torch.from_numpy(u0).cuda()
    m0 = float(ug.sum())
    hw.rktvd(prob, N, 3).integrate(ug, 0.0, 199.5 * dt, dt)
    m1 = float(ug.sum())
    assert abs(m1 - m0) <= 1e-11 * abs(m0), (m0, m1)


def test_full_size_constant_state(hw):
    import torch
    prob = hw.burgers_1d(N, -5.0, 5.0, k=3, alpha=1.0, bc="copy")
    ug = torch.full((N,), 0.37, dtype=torch.float64, device="cuda")
    hw.rktvd(prob, N, 3).integrate(ug, 0.0, 10.5e-7, 1e-7)
    # the stencils reproduce a constant only to rounding (11/6 - 7/6 + 1/3 is not exact)
    assert float((ug - 0.37).abs().max()) <= 1e-14
