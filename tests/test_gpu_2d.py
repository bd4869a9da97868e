"""GPU parity of the fused 2D stage kernel (example/example2_pbe_2d_fv.f90) against the oracle.

Tolerances: STRICT numerics bit-identical; FAST numerics max|gpu - oracle| / max|oracle|
<= 1e-12 for one right-hand side and for integrations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def device_rhs(prob, v):
    import ctypes as C

    import torch
    from hrweno import _abi as A
    tv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    out = torch.empty_like(tv)
    cp = prob.to_c()
    A.check(A.lib().hrw_rhs(C.byref(cp), A.HRW_F64, 0.0, tv.data_ptr(), out.data_ptr(), None))
    return out.cpu().numpy()


SHAPES = [(1, 1), (2, 3), (5, 7), (31, 33), (32, 32), (64, 40), (100, 37)]

PROBLEMS = {
    # upwind Godunov, g1 = 1 + 0.5 x1 > 0, g2 = 0.5 > 0: the vr-only specialisation
    "pbe_upwind": dict(flux="godunov", g1=(1.0, 0.5), g2=(0.5, 0.0), bc="zero_inflow"),
    # closed boundaries as the reference example (example2...f90:117-120)
    "pbe_closed": dict(flux="godunov", g1=(1.0, 0.5), g2=(0.5, 0.0), bc="zero"),
    # negative velocity in x2: general Godunov path
    "pbe_mixed": dict(flux="godunov", g1=(0.3, 0.5), g2=(-0.4, 0.0), bc="copy"),
    # Lax-Friedrichs
    "pbe_lf": dict(flux="lax_friedrichs", g1=(1.0, 0.5), g2=(0.5, 0.0), bc="zero_inflow"),
}


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("name", list(PROBLEMS))
def test_rhs_2d_linear(hw, orc, shape, k, name):
    n1, n2 = shape
    rng = np.random.default_rng(n1 * 131 + n2 + k)
    v = rng.uniform(0.0, 1.0, n1 * n2)
    kw = PROBLEMS[name]
    for numerics in ("strict", "fast"):
        prob = hw.pbe_2d(n1, n2, g1=kw["g1"], g2=kw["g2"], k=k, flux=kw["flux"], bc=kw["bc"],
                         numerics=numerics)
        ref = orc.rhs(prob, v)
        got = device_rhs(prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref), (name, shape, k)
        else:
            assert nrel(got, ref) <= TOL, (name, shape, k, nrel(got, ref))


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
def test_rhs_2d_burgers(hw, orc, flux):
    n1, n2 = 45, 70
    rng = np.random.default_rng(5)
    v = rng.uniform(-1.0, 1.0, n1 * n2)  # sign changes: both Godunov branches
    for numerics in ("strict", "fast"):
        prob = hw.Problem(kind="fv2d", ncells=(n1, n2), k=3, flux=flux,
                          fn=("burgers", "burgers"), alpha=(1.0, 1.0), bc=("copy", "zero"),
                          xmin=(-1.0, 0.0), xmax=(1.0, 2.0), numerics=numerics)
        ref = orc.rhs(prob, v)
        got = device_rhs(prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref)
        else:
            assert nrel(got, ref) <= TOL


def test_rhs_2d_widths(hw, orc):
    n1, n2 = 40, 24
    rng = np.random.default_rng(9)
    w1 = rng.uniform(0.5, 1.5, n1) / n1
    w2 = rng.uniform(0.5, 1.5, n2) / n2
    v = rng.uniform(0.0, 1.0, n1 * n2)
    for numerics in ("strict", "fast"):
        prob = hw.pbe_2d(n1, n2, numerics=numerics)
        prob.width = (w1, w2)
        ref = orc.rhs(prob, v)
        got = device_rhs(prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref)
        else:
            assert nrel(got, ref) <= TOL


def stretched_edges(n, x0, x1, ratio):
    """n + 1 edges on [x0, x1] with widths in geometric progression (a smooth stretched grid)."""
    w = ratio ** np.arange(n, dtype=np.float64)
    return x0 + (x1 - x0) * np.concatenate([[0.0], np.cumsum(w) / w.sum()])


def nonuniform_pbe(hw, n1, n2, k, name, which, numerics):
    kw = PROBLEMS[name]
    prob = hw.pbe_2d(n1, n2, g1=kw["g1"], g2=kw["g2"], k=k, flux=kw["flux"], bc=kw["bc"],
                     numerics=numerics)
    prob.xedges = (stretched_edges(n1, 0.0, 1.0, 1.02) if which in ("x1", "both") else None,
                   stretched_edges(n2, 0.0, 1.0, 0.97) if which in ("x2", "both") else None)
    return prob


@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (33, 31), (64, 40), (100, 37)])
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("which", ["x1", "x2", "both"])
@pytest.mark.parametrize("name", ["pbe_upwind", "pbe_mixed", "pbe_lf"])
def test_rhs_2d_nonuniform(hw, orc, shape, k, which, name):
    """Non-uniform lines in 2D ("any smooth grid can be used", example2...f90:36-39): each
    line's cells reconstruct with their own cnu, divide by their widths and evaluate g at
    the true edges; a uniform line of the same problem keeps the tables."""
    n1, n2 = shape
    rng = np.random.default_rng(n1 * 7 + n2 + k)
    v = rng.uniform(0.0, 1.0, n1 * n2)
    for numerics in ("strict", "fast"):
        prob = nonuniform_pbe(hw, n1, n2, k, name, which, numerics)
        ref = orc.rhs(prob, v)
        got = device_rhs(prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref), (name, shape, k, which)
        else:
            assert nrel(got, ref) <= TOL, (name, shape, k, which, nrel(got, ref))


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_mstvd_2d_nonuniform(hw, orc, numerics):
    from hrweno import workloads
    n1, n2 = 96, 80
    _, n0, dt = workloads.pbe_config(n1, n2, cfl=0.25)
    prob = nonuniform_pbe(hw, n1, n2, 3, "pbe_upwind", "both", numerics)
    g, o = hw.mstvd(prob, n1 * n2), orc.ODE(prob, n1 * n2, 1)
    ug, uo = n0.copy(), n0.copy()
    tg = to = 0.0
    for tout in (20 * dt, 61.5 * dt):
        tg = g.integrate(ug, tg, tout, dt)
        to = o.integrate(uo, to, tout, dt)
        assert tg == to and g.nsteps == o.info()[2]
        assert np.isfinite(uo).all()
        if numerics == "strict":
            assert np.array_equal(ug, uo)
        else:
            assert nrel(ug, uo) <= TOL


@pytest.mark.parametrize("numerics", ["strict", "fast"])
@pytest.mark.parametrize("bc", ["zero_inflow", "zero"])
def test_mstvd_2d_pbe(hw, orc, numerics, bc):
    """mstvd (src/hrweno_tvdode.f90:203-271) on the PBE problem: RK3 start, then 5-step."""
    from hrweno import workloads
    n1, n2 = 96, 80
    prob, n0, dt = workloads.pbe_config(n1, n2, bc=bc, numerics=numerics)
    g, o = hw.mstvd(prob, n1 * n2), orc.ODE(prob, n1 * n2, 1)
    ug, uo = n0.copy(), n0.copy()
    tg = to = 0.0
    for tout in (0.0, 20 * dt, 61.5 * dt):
        tg = g.integrate(ug, tg, tout, dt)
        to = o.integrate(uo, to, tout, dt)
        assert tg == to and g.nsteps == o.info()[2] and g.fevals == o.info()[0]
        if numerics == "strict":
            assert np.array_equal(ug, uo)
        else:
            assert nrel(ug, uo) <= TOL


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_rktvd_2d(hw, orc, numerics):
    from hrweno import workloads
    n1, n2 = 70, 50
    prob, n0, dt = workloads.pbe_config(n1, n2, numerics=numerics)
    g, o = hw.rktvd(prob, n1 * n2, 3), orc.ODE(prob, n1 * n2, 0, 3)
    ug, uo = n0.copy(), n0.copy()
    tg = g.integrate(ug, 0.0, 30.5 * dt, dt)
    to = o.integrate(uo, 0.0, 30.5 * dt, dt)
    assert tg == to
    if numerics == "strict":
        assert np.array_equal(ug, uo)
    else:
        assert nrel(ug, uo) <= TOL


def test_pbe_1024_strict_parity(hw, orc):
    """The 1024^2 configuration: the RK3 start and three multistep steps, bit-identical."""
    import torch
    from hrweno import workloads
    n = 1024
    prob, n0, dt = workloads.pbe_config(n, n, numerics="strict")
    ug = torch.from_numpy(n0.copy()).cuda()
    g, o = hw.mstvd(prob, n * n), orc.ODE(prob, n * n, 1)
    tg = g.integrate(ug, 0.0, 6.5 * dt, dt)
    uo = n0.copy()
    to = o.integrate(uo, 0.0, 6.5 * dt, dt)
    assert tg == to and g.nsteps == 7
    assert np.array_equal(ug.cpu().numpy(), uo)


def test_pbe_mass_balance(hw):
    """Closed boundaries (all edge fluxes zero): total mass is conserved to rounding."""
    import torch
    from hrweno import workloads
    n = 512
    prob, n0, dt = workloads.pbe_config(n, n, bc="zero")
    ug = torch.from_numpy(n0.copy()).cuda()
    m0 = float(ug.sum())
    hw.mstvd(prob, n * n).integrate(ug, 0.0, 200.5 * dt, dt)
    assert abs(float(ug.sum()) - m0) <= 1e-12 * m0
    # WENO is not positivity-preserving: small undershoots at the pulse foot only
    assert float(ug.min()) > -1e-4 * float(ug.max())
