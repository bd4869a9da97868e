"""The flux function registry beyond the examples' two: f(u, x) = u^2/2 + (a + b x) u
(HRW_FN_BURGERS_LINEAR), a convex flux carried by a velocity field, through every FP64 path
(single line, 2D, batched, adjoint), against the oracle: STRICT bit-identical, FAST to
rounding level."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_ONE = 1e-12


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def line(nc, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, nc)
    return 0.3 * np.sin(3 * x + rng.uniform(0, 6)) + 0.2 * rng.standard_normal(nc) * (np.abs(x) < 0.3)


def device_rhs(hw, prob, v):
    import ctypes as C

    import torch
    from hrweno import _abi as A
    tv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    out = torch.empty_like(tv)
    cp = prob.to_c()
    A.check(A.lib().hrw_rhs(C.byref(cp), A.HRW_F64, 0.0, tv.data_ptr(), out.data_ptr(), None))
    return out.cpu().numpy()


def problem(hw, nc, k, flux, bc, numerics, coef=(-0.3, 0.4), nd=1, n2=1):
    return hw.Problem(kind="fv2d" if nd == 2 else "fv1d", ncells=(nc, n2), k=k, flux=flux,
                      fn=("burgers_linear", "burgers_linear"), coef_a=(coef[0], 0.2), coef_b=(coef[1], -0.1),
                      alpha=(1.5, 1.5), bc=(bc, bc), xmin=(-1.0, 0.0), xmax=(1.0, 1.0), numerics=numerics)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
@pytest.mark.parametrize("nc", [1, 7, 1000])
def test_rhs_1d(hw, orc, k, flux, bc, nc):
    v = line(nc, nc + k)
    for numerics in ("strict", "fast"):
        prob = problem(hw, nc, k, flux, bc, numerics)
        ref = orc.rhs(prob, v)
        got = device_rhs(hw, prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref)
        else:
            assert nrel(got, ref) <= 10 * TOL_ONE


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("shape", [(5, 7), (64, 40), (31, 33)])
def test_rhs_2d(hw, orc, flux, shape):
    n1, n2 = shape
    v = line(n1 * n2, 3)
    for numerics in ("strict", "fast"):
        prob = problem(hw, n1, 3, flux, "zero", numerics, nd=2, n2=n2)
        ref = orc.rhs(prob, v)
        got = device_rhs(hw, prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref)
        else:
            assert nrel(got, ref) <= 10 * TOL_ONE


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_rktvd_integration(hw, orc, numerics):
    nc = 600
    prob = problem(hw, nc, 3, "godunov", "zero_inflow", numerics)
    u0 = line(nc, 5)
    dt = 0.3 * (2.0 / nc) / 1.5
    g, o = hw.rktvd(prob, nc, 3), orc.ODE(prob, nc, 0, 3)
    ug, uo = u0.copy(), u0.copy()
    tg = g.integrate(ug, 0.0, 149.5 * dt, dt)
    to = o.integrate(uo, 0.0, 149.5 * dt, dt)
    assert tg == to
    if numerics == "strict":
        assert np.array_equal(ug, uo)
    else:
        assert nrel(ug, uo) <= 1e-12


def test_batch_matches_single(hw):
    probs, lines, dts = [], [], []
    for i, n in enumerate((64, 300, 5000)):
        probs.append(problem(hw, n, 2 + i % 2, ("lax_friedrichs", "godunov")[i % 2], "copy", "fast"))
        lines.append(line(n, i))
        dts.append(0.3 * (2.0 / n) / 1.5)
    dts = np.array(dts)
    b = hw.batch(probs, order=3)
    u = b.pack(lines)
    b.advance(u, np.zeros(len(probs)), dts, 20)
    got = b.unpack(u)
    for i, p in enumerate(probs):
        v = lines[i].copy()
        hw.rktvd(p, p.ncells[0], 3).integrate(v, 0.0, 19.5 * dts[i], dts[i])
        assert np.array_equal(got[i], v), i


def test_adjoint_vs_tangent_linear(hw, orc):
    n, steps = 300, 40
    prob = problem(hw, n, 3, "lax_friedrichs", "copy", "fast")
    u0, target = line(n, 1), line(n, 2) * 0.9
    dt = 0.3 * (2.0 / n) / 1.5
    J, g = hw.adjoint(prob, checkpoint_every=7).gradient(u0, target, dt, steps)
    d = np.random.default_rng(0).standard_normal(n)
    Jo, dJ = orc.tl_misfit(prob, u0, d, target, dt, steps)
    assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
    assert abs(g @ d - dJ) <= 1e-10 * abs(dJ)
