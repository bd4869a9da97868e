"""A second, independent restatement of the reference's formulas -- vectorised numpy, written
from src/hrweno_weno.f90 and example/example1_burgers_1d_fv.f90 -- against the C++ oracle on
random inputs (CPU only).  The oracle is pinned to the reference's known-answer tests; this
checks it everywhere else, to rounding level (numpy sums in its own order)."""
import numpy as np
import pytest

# method constants (src/hrweno_weno.f90:12-21): linear weights d and stencil coefficients c(j, r),
# r = -1 .. k-1 (stored here at column r + 1)
D = {1: np.array([1.0]), 2: np.array([2 / 3, 1 / 3]), 3: np.array([0.3, 0.6, 0.1])}
C = {
    1: np.array([[1.0, 1.0]]),
    2: np.array([[3 / 2, 1 / 2, -1 / 2], [-1 / 2, 1 / 2, 3 / 2]]),
    3: np.array([[11 / 6, 1 / 3, -1 / 6, 1 / 3], [-7 / 6, 5 / 6, 5 / 6, -7 / 6], [1 / 3, -1 / 6, 1 / 3, 11 / 6]]),
}


def reconstruct_np(v, k, eps):
    """weno%reconstruct (src/hrweno_weno.f90:163-215): (vl, vr) of every cell."""
    nc = v.size
    ext = np.concatenate([np.full(k - 1, v[0]), v, np.full(k - 1, v[-1])])  # vext, ghosts replicate
    at = lambda o: ext[k - 1 + o: k - 1 + o + nc]  # noqa: E731  vext(i + o) for every cell i
    vrr = np.zeros((k, nc))
    vlr = np.zeros((k, nc))
    for r in range(k):
        for j in range(k):
            vrr[r] += C[k][j, r + 1] * at(j - r)
            vlr[r] += C[k][j, r] * at(j - r)
    if k == 1:
        beta = np.zeros((1, nc))
    elif k == 2:
        beta = np.array([(at(1) - at(0)) ** 2, (at(0) - at(-1)) ** 2])
    else:
        beta = np.array([
            13 / 12 * (at(0) - 2 * at(1) + at(2)) ** 2 + 1 / 4 * (3 * at(0) - 4 * at(1) + at(2)) ** 2,
            13 / 12 * (at(-1) - 2 * at(0) + at(1)) ** 2 + 1 / 4 * (at(-1) - at(1)) ** 2,
            13 / 12 * (at(-2) - 2 * at(-1) + at(0)) ** 2 + 1 / 4 * (at(-2) - 4 * at(-1) + 3 * at(0)) ** 2,
        ])
    s = (eps + beta) ** 2
    alfa = D[k][:, None] / s
    alfat = D[k][::-1, None] / s
    return (alfat * vlr).sum(0) / alfat.sum(0), (alfa * vrr).sum(0) / alfa.sum(0)


def rhs_burgers_np(v, xmin, xmax, k, eps, flux, alpha, bc):
    """example1's right-hand side (example/example1_burgers_1d_fv.f90:72-109) with its
    boundary rules and the fluxes of src/hrweno_fluxes.f90:43,67-74."""
    nc = v.size
    vl, vr = reconstruct_np(v, k, eps)
    f = lambda u: u * u / 2  # noqa: E731
    vm, vp = vr[:-1], vl[1:]
    if flux == "lax_friedrichs":
        inner = (f(vm) + f(vp) - alpha * (vp - vm)) / 2
    else:
        fm, fp = f(vm), f(vp)
        inner = np.where(vm <= vp, np.minimum(fm, fp), np.maximum(fm, fp))
    F = np.zeros(nc + 1)
    F[1:nc] = inner
    if bc == "copy" and nc > 1:
        F[0], F[nc] = F[1], F[nc - 1]
    elif bc == "zero_inflow":
        F[nc] = f(vr[-1])
    dx = (xmax - xmin) / nc
    return -(F[1:] - F[:-1]) / dx


def lines(nc, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, nc)
    yield np.sin(2 * x) + 0.5 * np.exp(-20 * x * x)          # smooth
    yield np.where(np.abs(x) < 0.4, 1.0, 0.1) + 0.01 * x      # discontinuous
    yield rng.standard_normal(nc)                             # rough, sign changes


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 3, 5, 64, 1001])
def test_reconstruct_matches_numpy(orc, k, nc):
    for v in lines(nc, nc + k):
        vl, vr = orc.reconstruct(v, k, 1e-6)
        nl, nr = reconstruct_np(v, k, 1e-6)
        scale = max(np.max(np.abs(v)), 1e-300)
        assert np.max(np.abs(vl - nl)) <= 1e-13 * scale and np.max(np.abs(vr - nr)) <= 1e-13 * scale


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
@pytest.mark.parametrize("nc", [2, 7, 500])
def test_burgers_rhs_matches_numpy(hw, orc, k, flux, bc, nc):
    for v in lines(nc, 3 * nc + k):
        prob = hw.burgers_1d(nc, -5.0, 5.0, k=k, eps=1e-6, flux=flux, alpha=1.3, bc=bc, numerics="strict")
        ref = orc.rhs(prob, v)
        got = rhs_burgers_np(v, -5.0, 5.0, k, 1e-6, flux, 1.3, bc)
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, (k, flux, bc, nc)
