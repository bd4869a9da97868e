"""GPU parity: the CUDA path through the C ABI against the oracle on the same inputs.

Tolerances:
  STRICT numerics  bit-identical to the oracle (same IEEE operations in the same order).
  FAST numerics    normwise relative error max|gpu - oracle| / max|oracle| <= 1e-12 for
                   integrations (the 1e-12 relative parity bound), <= 1e-13 for one reconstruction / rhs.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_INT = 1e-12
TOL_ONE = 1e-13


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rand_line(nc, seed, kind="smooth"):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, nc)
    if kind == "smooth":
        return np.sin(3 * x) + 0.3 * np.cos(7 * x) + 0.1 * rng.standard_normal(nc)
    if kind == "pulse":
        v = np.zeros(nc)
        v[nc // 3 - 1: 2 * nc // 3] = 1.0
        return v
    return rng.uniform(-1, 1, nc)


NCS = [1, 2, 3, 4, 5, 7, 8, 30, 1023, 1024, 1025, 5000]


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", NCS)
def test_reconstruct_uniform(hw, orc, k, nc):
    for seed, kind in [(1, "smooth"), (2, "pulse"), (3, "noise")]:
        v = rand_line(nc, seed, kind)
        rl, rr = orc.reconstruct(v, k=k, eps=1e-6)
        for numerics in ("strict", "fast"):
            w = hw.weno(nc, k, 1e-6, numerics=numerics)
            vl, vr = np.empty(nc), np.empty(nc)
            w.reconstruct(v, vl, vr)
            if numerics == "strict":
                assert np.array_equal(vl, rl) and np.array_equal(vr, rr), (k, nc, kind)
            else:
                assert nrel(vl, rl) <= TOL_ONE and nrel(vr, rr) <= TOL_ONE, (k, nc, kind)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_reconstruct_pulse_kat_gpu(hw, k):
    """test_weno_uniform / test_weno_nonuniform (test/test_hrweno.f90:29-161) on the GPU."""
    nc = 30
    v = rand_line(nc, 0, "pulse")
    for xedges in (None, (np.arange(nc + 1) / nc) ** 3):
        w = hw.weno(nc, k, 1e-6, xedges=xedges)
        vl, vr = np.empty(nc), np.empty(nc)
        w.reconstruct(v, vl, vr)
        assert np.all(np.abs(vl - v) <= 1e-6) and np.all(np.abs(vr - v) <= 1e-6)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 5, 30, 777])
def test_reconstruct_nonuniform(hw, orc, k, nc):
    rng = np.random.default_rng(nc + k)
    xedges = np.cumsum(np.concatenate([[0.0], rng.uniform(0.5, 1.5, nc)]))
    v = rand_line(nc, 4, "smooth")
    cref = orc.calc_cnu(nc, k, xedges)
    rl, rr = orc.reconstruct(v, k=k, eps=1e-6, xedges=xedges)
    for numerics in ("strict", "fast"):
        w = hw.weno(nc, k, 1e-6, xedges=xedges, numerics=numerics)
        assert np.array_equal(w.cnu, cref)
        vl, vr = np.empty(nc), np.empty(nc)
        w.reconstruct(v, vl, vr)
        if numerics == "strict":
            assert np.array_equal(vl, rl) and np.array_equal(vr, rr)
        else:
            assert nrel(vl, rl) <= TOL_ONE and nrel(vr, rr) <= TOL_ONE


def test_calc_cnu_kat_gpu(hw):
    """test_calc_cnu (test/test_hrweno.f90:69-112) on the GPU: uniform edges give c tables."""
    gold = json.loads((Path(__file__).parent / "golden" / "kat_reference.json").read_text())
    nc = 30
    xedges = 3.0 * np.arange(nc + 1) / nc
    for k in (1, 2, 3):
        cnu = hw.weno(nc, k, 1e-6, xedges=xedges).cnu
        cref = np.array(gold["c_tables"][str(k)])
        for i in range(nc):
            np.testing.assert_allclose(cnu[i], cref, rtol=1e-5)


def device_rhs(hw, prob, v):
    import ctypes as C

    import torch
    from hrweno import _abi as A
    tv = torch.from_numpy(v).cuda()
    out = torch.empty_like(tv)
    cp = prob.to_c()
    A.check(A.lib().hrw_rhs(C.byref(cp), A.HRW_F64, 0.0, tv.data_ptr(), out.data_ptr(), None))
    return out.cpu().numpy()


PROBS_1D = [
    dict(flux="lax_friedrichs", bc="copy"),
    dict(flux="godunov", bc="copy"),
    dict(flux="godunov", bc="zero"),
    dict(flux="lax_friedrichs", bc="zero_inflow"),
]


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("pi", range(len(PROBS_1D)))
@pytest.mark.parametrize("nc", [1, 2, 6, 1000, 2049])
def test_rhs_1d_burgers(hw, orc, k, pi, nc):
    v = rand_line(nc, 7, "noise")  # sign changes exercise both Godunov branches
    for numerics in ("strict", "fast"):
        prob = hw.burgers_1d(nc, k=k, alpha=1.2, numerics=numerics, **PROBS_1D[pi])
        ref = orc.rhs(prob, v)
        got = device_rhs(hw, prob, v)
        if numerics == "strict":
            assert np.array_equal(got, ref)
        else:
            assert nrel(got, ref) <= 10 * TOL_ONE


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("coef", [(0.7, 0.0), (-0.4, 0.0), (1.0, 0.5), (-0.2, 0.6)])
def test_rhs_1d_linear_and_widths(hw, orc, flux, coef):
    nc = 333
    rng = np.random.default_rng(11)
    width = rng.uniform(0.8, 1.2, nc) * (2.0 / nc)
    v = rand_line(nc, 8, "smooth")
    for numerics in ("strict", "fast"):
        for w in (None, width):
            prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux=flux, fn=("linear", "linear"),
                              coef_a=(coef[0], 0), coef_b=(coef[1], 0), alpha=(abs(coef[0]) + abs(coef[1]), 0),
                              bc=("zero_inflow", "copy"), xmin=(-1.0, 0), xmax=(1.0, 1), width=(w, None),
                              numerics=numerics)
            ref = orc.rhs(prob, v)
            got = device_rhs(hw, prob, v)
            if numerics == "strict":
                assert np.array_equal(got, ref)
            else:
                assert nrel(got, ref) <= 10 * TOL_ONE


def config1(hw, numerics):
    nc = 500
    x = -5.0 + (10.0 / nc) * (np.arange(nc) + 0.5)
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy",
                         numerics=numerics)
    return prob, np.exp(-x ** 2)


GOLD1 = json.loads((Path(__file__).parent / "golden" / "oracle_config1.json").read_text())


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_config1_burgers_rk3_full(hw, orc, numerics):
    """500 cells, LF alpha=1, WENO5, RK3, dt=1e-2, 101 output times to t=12 (1201 steps)."""
    prob, _ = config1(hw, numerics)
    u0 = np.array(GOLD1["u0"])
    g = hw.rktvd(prob, 500, 3)
    o = orc.ODE(prob, 500, 0, 3)
    ug, uo = u0.copy(), u0.copy()
    tg = to = 0.0
    worst = 0.0
    for ii in range(101):
        tout = 12.0 * ii / 100
        tg = g.integrate(ug, tg, tout, 1e-2)
        to = o.integrate(uo, to, tout, 1e-2)
        assert tg == to
        if numerics == "strict":
            assert np.array_equal(ug, uo), ii
        else:
            worst = max(worst, nrel(ug, uo))
    assert worst <= TOL_INT, worst
    assert tg == 12.009999999999788 and g.nsteps == 1201 and g.fevals == 3603 and g.istate == 2
    snap = GOLD1["snapshots"][-1]
    assert snap["t"] == tg
    assert nrel(ug, np.array(snap["u"])) <= (0 if numerics == "strict" else TOL_INT)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("k", [2, 3])
def test_rktvd_orders(hw, orc, order, k):
    nc = 1500
    x = np.linspace(-1, 1, nc)
    u0 = 0.5 + np.exp(-20 * x ** 2) * np.sign(np.sin(9 * x))
    for numerics in ("strict", "fast"):
        # outflow boundaries keep the local CFL number below 0.6 (a wall would pile mass into
        # the last cell until forward Euler blows up)
        prob = hw.burgers_1d(nc, -1.0, 1.0, k=k, flux="godunov", bc="copy", numerics=numerics)
        g, o = hw.rktvd(prob, nc, order), orc.ODE(prob, nc, 0, order)
        ug, uo = u0.copy(), u0.copy()
        # forward Euler is not stable with WENO (its amplification factor exceeds 1 on the
        # imaginary axis), so order 1 runs 20 steps only; orders 2 and 3 run 400
        tend = 0.2 if order > 1 else 0.01
        tg = g.integrate(ug, 0.0, tend, 5e-4)
        to = o.integrate(uo, 0.0, tend, 5e-4)
        assert tg == to and g.fevals == o.info()[0]
        assert np.all(np.isfinite(uo)) and np.max(np.abs(uo)) < 2.0
        if numerics == "strict":
            assert np.array_equal(ug, uo)
        else:
            assert nrel(ug, uo) <= TOL_INT


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_mstvd_1d(hw, orc, numerics):
    nc = 800
    x = np.linspace(0, 1, nc)
    u0 = np.exp(-((x - 0.3) / 0.05) ** 2)
    prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux="godunov", fn=("linear", "linear"),
                      coef_a=(1.0, 0), coef_b=(0.5, 0), alpha=(1.5, 0), bc=("zero_inflow", "copy"),
                      xmin=(0.0, 0), xmax=(1.0, 1), numerics=numerics)
    g, o = hw.mstvd(prob, nc), orc.ODE(prob, nc, 1)
    ug, uo = u0.copy(), u0.copy()
    tg = to = 0.0
    # CFL 0.24: at 0.48 the multistep method sits at its stability limit and rounding grows
    # (the FP64 and binary128 oracles then disagree completely); here they agree to 2e-15
    for tout in (0.0, 0.05, 0.1, 0.25):
        tg = g.integrate(ug, tg, tout, 2e-4)
        to = o.integrate(uo, to, tout, 2e-4)
        assert tg == to
        assert g.fevals == o.info()[0] and g.nsteps == o.info()[2]
        if numerics == "strict":
            assert np.array_equal(ug, uo)
        else:
            assert nrel(ug, uo) <= TOL_INT


RATES = np.array([-1.0 + (ii - 1) * 4.0 / 9 for ii in range(1, 11)])


@pytest.mark.parametrize("order,rtol", [(1, 2e-2), (2, 1e-3), (3, 1e-3)])
def test_rktvd_linear_kat_gpu(hw, orc, order, rtol):
    """test_rktvd (test/test_tvdode.f90:31-70) through the GPU integrator."""
    t0, tout = -1.3, 1.5
    dt = (tout - t0) / 3000
    for numerics in ("strict", "fast"):
        prob = hw.linear_ode(RATES, numerics=numerics)
        g = hw.rktvd(prob, 10, order)
        u = np.full(10, 0.1)
        t = g.integrate(u, t0, tout, dt)
        uref = 0.1 * np.exp(RATES * (t - t0))
        assert np.all(np.abs(u - uref) <= rtol * np.abs(uref))
        uo = np.full(10, 0.1)
        orc.ODE(prob, 10, 0, order).integrate(uo, t0, tout, dt)
        assert np.array_equal(u, uo) if numerics == "strict" else nrel(u, uo) <= TOL_INT


def test_mstvd_linear_kat_gpu(hw, orc):
    """test_mstvd (test/test_tvdode.f90:72-104) through the GPU integrator."""
    for numerics in ("strict", "fast"):
        prob = hw.linear_ode(RATES, numerics=numerics)
        g = hw.mstvd(prob, 10)
        u = np.full(10, 0.1)
        t = g.integrate(u, -1.3, 1.5, 1e-3)
        uref = 0.1 * np.exp(RATES * (t + 1.3))
        assert np.all(np.abs(u - uref) <= 1e-3 * np.abs(uref))
        uo = np.full(10, 0.1)
        orc.ODE(prob, 10, 1).integrate(uo, -1.3, 1.5, 1e-3)
        assert np.array_equal(u, uo) if numerics == "strict" else nrel(u, uo) <= TOL_INT


def test_device_memory_matches_host_memory(hw):
    import torch
    prob, u0 = config1(hw, "fast")
    a = hw.rktvd(prob, 500, 3)
    b = hw.rktvd(prob, 500, 3)
    uh = u0.copy()
    ud = torch.from_numpy(u0.copy()).cuda()
    th = a.integrate(uh, 0.0, 1.0, 1e-2)
    td = b.integrate(ud, 0.0, 1.0, 1e-2)
    assert th == td and np.array_equal(uh, ud.cpu().numpy())


def test_itask_single_step(hw, orc):
    prob, u0 = config1(hw, "strict")
    g, o = hw.rktvd(prob, 500, 3), orc.ODE(prob, 500, 0, 3)
    ug, uo = u0.copy(), u0.copy()
    tg = g.integrate(ug, 0.0, 5.0, 1e-2, itask=2)
    to = o.integrate(uo, 0.0, 5.0, 1e-2, itask=2)
    assert tg == to == 0.01 and g.nsteps == 1 and np.array_equal(ug, uo)


def test_integrate_already_done_is_noop(hw):
    prob, u0 = config1(hw, "fast")
    g = hw.rktvd(prob, 500, 3)
    u = u0.copy()
    t = g.integrate(u, 1.0, 0.5, 1e-2)  # (t - tout) * sign(dt) > 0: return at once (:127)
    assert t == 1.0 and np.array_equal(u, u0) and g.fevals == 0 and g.istate == 1


def test_invalid_memory_space_is_rejected(hw):
    """A memory-space flag other than HRW_MEM_HOST / HRW_MEM_DEVICE returns HRW_EINVAL before any
    copy or launch; u, t and the handle are untouched and the handle stays usable."""
    import ctypes as C
    from hrweno import _abi as A
    prob, u0 = config1(hw, "fast")
    g = hw.rktvd(prob, 500, 3)
    u = u0.copy()
    t = C.c_double(0.0)
    assert A.lib().hrw_integrate(g._h, 7, u.ctypes.data, C.byref(t), 1.0, 1e-2, 1) == A.HRW_EINVAL
    assert A.lib().hrw_last_error().decode() == "Invalid input 'mem'."
    assert t.value == 0.0 and np.array_equal(u, u0) and g.istate == 1 and g.nsteps == 0
    w = hw.weno(500)
    vl, vr = np.zeros(500), np.zeros(500)
    assert A.lib().hrw_weno_reconstruct(w._h, A.HRW_F64, -1, u.ctypes.data, vl.ctypes.data,
                                        vr.ctypes.data) == A.HRW_EINVAL
    assert not vl.any() and not vr.any()
    assert g.integrate(u, 0.0, 1.0, 1e-2) > 1.0 and g.istate == 2


def stretched_edges(nc, kind, seed=0):
    if kind == "cubic":  # test/test_hrweno.f90:123-128 stretches edges as (i/nc)^3
        return -1.0 + 2.0 * (np.arange(nc + 1) / nc) ** 3
    rng = np.random.default_rng(seed)
    return np.concatenate([[-1.0], -1.0 + np.cumsum(rng.uniform(0.5, 1.5, nc)) * (2.0 / nc)])


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 7, 300, 1000])
@pytest.mark.parametrize("kind", ["cubic", "random"])
def test_rhs_1d_nonuniform(hw, orc, k, nc, kind):
    """weno(ncells, k, eps, xedges) inside the fused stage: cnu coefficients, true widths and
    interface coordinates (src/hrweno_weno.f90:100-104,177; example1...f90:107)."""
    xe = stretched_edges(nc, kind, nc)
    v = rand_line(nc, 9, "smooth") + 1.0
    cases = [dict(flux="lax_friedrichs", fn="burgers", bc="copy", b=0.0),
             dict(flux="godunov", fn="burgers", bc="zero", b=0.0),
             dict(flux="godunov", fn="linear", bc="zero_inflow", b=0.4),
             dict(flux="lax_friedrichs", fn="linear", bc="copy", b=-0.3)]
    for c in cases:
        for numerics in ("strict", "fast"):
            prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, flux=c["flux"],
                              fn=(c["fn"], c["fn"]), coef_a=(0.8, 0), coef_b=(c["b"], 0),
                              alpha=(2.5, 2.5), bc=(c["bc"], c["bc"]), xedges=(xe, None),
                              numerics=numerics)
            ref = orc.rhs(prob, v)
            got = device_rhs(hw, prob, v)
            if numerics == "strict":
                assert np.array_equal(got, ref), (c, k, nc, kind)
            else:
                assert nrel(got, ref) <= 10 * TOL_ONE, (c, k, nc, kind)


@pytest.mark.parametrize("numerics", ["strict", "fast"])
@pytest.mark.parametrize("order", [2, 3])
def test_rktvd_nonuniform(hw, orc, numerics, order):
    nc = 700
    xe = stretched_edges(nc, "random", 3)
    xc = 0.5 * (xe[1:] + xe[:-1])
    u0 = 0.5 + np.exp(-30 * xc ** 2)
    prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux="lax_friedrichs",
                      fn=("burgers", "burgers"), alpha=(1.5, 1.5), bc=("copy", "copy"),
                      xedges=(xe, None), numerics=numerics)
    dt = 0.3 * np.min(np.diff(xe)) / 1.5
    g, o = hw.rktvd(prob, nc, order), orc.ODE(prob, nc, 0, order)
    ug, uo = u0.copy(), u0.copy()
    tg = g.integrate(ug, 0.0, 150.5 * dt, dt)
    to = o.integrate(uo, 0.0, 150.5 * dt, dt)
    assert tg == to
    if numerics == "strict":
        assert np.array_equal(ug, uo)
    else:
        assert nrel(ug, uo) <= TOL_INT
