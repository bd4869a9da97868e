"""Oracle properties the reference's semantics imply (CPU only)."""
import numpy as np
import pytest

from hrweno.problems import burgers_1d, linear_ode, pbe_2d


def config1_u0(nc=500):
    x = -5.0 + (10.0 / nc) * (np.arange(nc) + 0.5)
    return np.exp(-x ** 2)


def test_config1_step_count_and_time(orc):
    """101 output times to t=12 with dt=1e-2: 1201 steps, t ends at 12.009999999999788
    (is_done overshoot, src/hrweno_tvdode.f90:127,137-143,282)."""
    nc = 500
    prob = burgers_1d(nc, k=3, alpha=1.0)
    ode = orc.ODE(prob, nc, method=0, order=3)
    u, t = config1_u0(nc), 0.0
    for ii in range(101):
        t = ode.integrate(u, t, 12.0 * ii / 100, 1e-2)
    fe, st, ns = ode.info()
    assert ns == 1201 and fe == 3 * 1201 and st == 2
    assert t == 12.009999999999788


def test_quad_yardstick_config1(orc):
    """REAL64 oracle vs the REAL128 yardstick on the 500-cell shock case: the rounding-level
    sensitivity of the problem, which sets the scale of the 1e-12 parity tolerance."""
    nc = 500
    prob = burgers_1d(nc, k=3, alpha=1.0)
    res = {}
    for prec in (64, 128):
        ode = orc.ODE(prob, nc, method=0, order=3, prec=prec)
        u = config1_u0(nc)
        ode.integrate(u, 0.0, 3.0, 1e-2)
        res[prec] = u
    err = np.max(np.abs(res[64] - res[128])) / np.max(np.abs(res[128]))
    assert err < 1e-13, err


def test_conservation_zero_bc(orc):
    """With zero boundary fluxes the FV update conserves sum(u * width) to rounding."""
    nc = 200
    prob = burgers_1d(nc, k=3, alpha=1.5, bc="zero", flux="godunov")
    ode = orc.ODE(prob, nc, method=0, order=3)
    u = 0.5 + config1_u0(nc)
    m0 = u.sum()
    ode.integrate(u, 0.0, 1.0, 1e-2)
    assert abs(u.sum() - m0) <= 1e-12 * m0


def test_mstvd_fevals(orc):
    """mstvd counts the start's 12 RK3 evaluations, not the 4 extra rhs calls (:246)."""
    ode = orc.ODE(linear_ode(np.ones(3)), 3, method=1)
    u = np.ones(3)
    t = ode.integrate(u, 0.0, 0.1, 0.01)
    fe, st, ns = ode.info()
    assert st == 2
    # start: 4 steps to t=0.04; then steps while not is_done: t = 0.05 ... 0.11
    assert fe == 12 + (ns - 4)


def test_pbe2d_rhs_linear_in_n(orc):
    """The upwind 2D right-hand side is homogeneous of degree 1 in n (WENO weights are
    scale-invariant only up to eps, so use a scale where eps is negligible)."""
    n1 = n2 = 24
    prob = pbe_2d(n1, n2, flux="godunov", bc="zero_inflow")
    rng = np.random.default_rng(1)
    v = rng.uniform(1e4, 2e4, n1 * n2)  # beta >> eps
    a = orc.rhs(prob, v)
    b = orc.rhs(prob, 2.0 * v)
    np.testing.assert_allclose(b, 2.0 * a, rtol=1e-8, atol=1e-8 * np.abs(a).max())


@pytest.mark.parametrize("k", [1, 2, 3])
def test_reconstruct_constant_state(orc, k):
    v = np.full(17, 0.3)
    vl, vr = orc.reconstruct(v, k=k)
    assert np.all(vl == 0.3) or np.allclose(vl, 0.3, rtol=1e-15)
    assert np.allclose(vr, 0.3, rtol=1e-15)


def test_oracle_reproduces_golden_config1(orc):
    """The committed 500-cell snapshots (tests/golden/oracle_config1.json) are reproduced bit
    for bit from the stored u0: the oracle gives the same bits on every machine."""
    import json
    from pathlib import Path
    gold = json.loads((Path(__file__).parent / "golden" / "oracle_config1.json").read_text())
    nc = gold["nc"]
    prob = burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy")
    ode = orc.ODE(prob, nc, method=0, order=3)
    u = np.array(gold["u0"])
    t = 0.0
    for snap in gold["snapshots"]:
        t = ode.integrate(u, t, snap["tout"], gold["dt"])
        assert t == snap["t"]
        assert np.array_equal(u, np.array(snap["u"]))


def test_pbe_mstvd_stability_limit(orc):
    """The 2D multistep scheme is rounding-stable at CFL 0.3 (FP64 and binary128 oracles
    agree to 1e-14 after 300 steps) and unstable at the configuration's CFL 0.4 (they drift
    apart by orders of magnitude): accuracy checks of the 2D forms use CFL 0.3."""
    from hrweno import workloads
    n = 96
    drift = {}
    for cfl in (0.3, 0.4):
        p, n0, dt = workloads.pbe_config(n, n, cfl=cfl)
        out = []
        for prec in (64, 128):
            o = orc.ODE(p, n * n, 1, prec=prec)
            u = n0.copy()
            o.integrate(u, 0.0, 299.5 * dt, dt)
            out.append(u)
        drift[cfl] = np.abs(out[0] - out[1]).sum() / np.abs(out[1]).sum()
    assert drift[0.3] < 1e-14
    assert drift[0.4] > 1e3 * drift[0.3]


def test_flux_burgers_linear_consistency_and_upwinding(orc):
    """f(u, x) = u^2/2 + (a + b x) u in the reference's flux checks (test/test_fluxes.f90:27-71):
    h(v, v) = f(v) for both fluxes; Godunov takes the upwind state where f' keeps one sign."""
    from hrweno import _abi as A
    a, b, x = 0.5, 0.25, 2.0
    f = lambda u: u * u / 2 + (a + b * x) * u  # noqa: E731
    for v in (-3.0, 0.2, 1.7):
        for kind in (A.HRW_FLUX_LAX_FRIEDRICHS, A.HRW_FLUX_GODUNOV):
            h = orc.numflux(kind, A.HRW_FN_BURGERS_LINEAR, v, v, x, 0.0, alpha=5.0, a=a, b=b)
            assert abs(h - f(v)) <= 1e-15 * max(1.0, abs(f(v)))
    # f'(u) = u + 1 > 0 for u > -1: the flux from the left state
    vm, vp = 0.4, 0.9
    assert orc.numflux(A.HRW_FLUX_GODUNOV, A.HRW_FN_BURGERS_LINEAR, vm, vp, x, 0.0, a=a, b=b) == f(vm)
    assert orc.numflux(A.HRW_FLUX_GODUNOV, A.HRW_FN_BURGERS_LINEAR, vp, vm, x, 0.0, a=a, b=b) == f(vp)


def test_godunov_takes_the_endpoint_extremum(orc):
    """godunov (src/hrweno_fluxes.f90:67-74) takes min(f(vm), f(vp)) when vm <= vp and the max
    otherwise: the endpoints only, where Shu's eq. 2.70 takes the extremum over [vm, vp].  The
    two agree unless f has a critical point between the states; for Burgers that is a
    rarefaction across u = 0, where the reference gives min(vm^2, vp^2)/2 instead of f(0) = 0.
    The oracle and the GPU fluxes keep the reference's rule."""
    from hrweno import _abi as A
    g = lambda vm, vp: orc.numflux(A.HRW_FLUX_GODUNOV, A.HRW_FN_BURGERS, vm, vp, 0.0, 0.0)  # noqa: E731
    assert g(-1.0, 2.0) == 0.5          # rarefaction through the sonic point: eq. 2.70 gives 0
    assert g(2.0, -1.0) == 2.0          # shock: the max over [vp, vm] is at an endpoint
    assert g(0.5, 2.0) == 0.125         # f' > 0 on [vm, vp]: the upwind state
    assert g(-2.0, -0.5) == 0.125       # f' < 0: the downwind end is upwind


@pytest.mark.parametrize("k", [1, 2, 3])
def test_reconstruct_symmetries(orc, k):
    """Invariances of weno%reconstruct on a uniform grid that follow from its formulas
    (src/hrweno_weno.f90:163-215), to rounding:
      mirror     reversing the line swaps the roles of vl and vr (c and d are symmetric);
      shift      v + s reconstructs to vl + s, vr + s (beta sees differences only);
      scale      s v with eps s^2 reconstructs to s vl, s vr (beta scales with s^2)."""
    rng = np.random.default_rng(k)
    x = np.linspace(-1.0, 1.0, 257)
    for v in (np.sin(3 * x) + (x > 0.2), rng.standard_normal(257), np.exp(-30 * x * x)):
        vl, vr = orc.reconstruct(v, k, 1e-6)
        ml, mr = orc.reconstruct(v[::-1].copy(), k, 1e-6)
        scale = np.max(np.abs(v))
        assert np.max(np.abs(ml[::-1] - vr)) <= 1e-14 * scale
        assert np.max(np.abs(mr[::-1] - vl)) <= 1e-14 * scale
        sl, sr = orc.reconstruct(v + 3.0, k, 1e-6)
        assert np.max(np.abs(sl - (vl + 3.0))) <= 1e-13 * (scale + 3.0)
        assert np.max(np.abs(sr - (vr + 3.0))) <= 1e-13 * (scale + 3.0)
        for s in (1e-3, 7.0):
            ql, qr = orc.reconstruct(s * v, k, 1e-6 * s * s)
            assert np.max(np.abs(ql - s * vl)) <= 1e-14 * s * scale
            assert np.max(np.abs(qr - s * vr)) <= 1e-14 * s * scale


def test_numerical_fluxes_are_monotone(orc):
    """The fluxes are monotone (src/hrweno_fluxes.f90:22-76): h(vm, vp) does not decrease in vm
    nor increase in vp.  Lax-Friedrichs (alpha = max|f'| over the states) and Godunov for linear
    fluxes of either sign are monotone everywhere.  The reference's endpoint Godunov rule is
    monotone for Burgers on states of one sign only: across the sonic point u = 0,
    min(f(vm), f(vp)) grows as vm falls below -vp's magnitude (the true Godunov flux is 0 there)."""
    from hrweno import _abi as A

    def table(kind, fn, a, alpha, vs):
        return np.array([[orc.numflux(kind, fn, vm, vp, 0.0, 0.0, alpha=alpha, a=a, b=0.0)
                          for vp in vs] for vm in vs])

    def monotone(h):
        return bool(np.all(np.diff(h, axis=0) >= -1e-15) and np.all(np.diff(h, axis=1) <= 1e-15))

    vs = np.linspace(-2.0, 2.0, 41)
    for fn, a, alpha in [(A.HRW_FN_BURGERS, 1.0, 2.0), (A.HRW_FN_LINEAR, 0.7, 0.7),
                         (A.HRW_FN_LINEAR, -1.3, 1.3)]:
        assert monotone(table(A.HRW_FLUX_LAX_FRIEDRICHS, fn, a, alpha, vs)), (fn, a)
    for a in (0.7, -1.3):
        assert monotone(table(A.HRW_FLUX_GODUNOV, A.HRW_FN_LINEAR, a, 0.0, vs)), a
    burgers = lambda vs: table(A.HRW_FLUX_GODUNOV, A.HRW_FN_BURGERS, 1.0, 0.0, vs)  # noqa: E731
    assert monotone(burgers(np.linspace(0.0, 2.0, 21)))
    assert monotone(burgers(np.linspace(-2.0, 0.0, 21)))
    assert not monotone(burgers(vs))


@pytest.mark.parametrize("bc", ["copy", "zero_inflow"])
def test_tangent_linear_oracle_matches_central_differences(orc, bc):
    """The tangent-linear oracle (the restated forward map on dual numbers), which the GPU
    adjoint is checked against, agrees with the oracle's own forward solve: the same J, and dJ
    in a smooth random direction equal to 4th-order central differences of J.  The WENO weights
    make the map strongly nonlinear at this resolution (at h = 1e-3 the differences are still
    1e-3 off), so the step is 1e-5."""
    n, steps = 64, 20
    prob = burgers_1d(n, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.5, bc=bc,
                      numerics="strict")
    x = -5.0 + 10.0 / n * (np.arange(n) + 0.5)
    u0 = 0.3 + np.exp(-x ** 2)
    target = 0.8 * (0.3 + np.exp(-(x - 0.5) ** 2))
    dt = 0.4 * (10.0 / n) / 1.5
    rng = np.random.default_rng(3)
    xs = np.linspace(0.0, 1.0, n)
    d = sum(rng.standard_normal() * np.sin(np.pi * m * xs + rng.uniform(0.0, 6.28)) / m
            for m in range(1, 9))

    def J(u):
        o = orc.ODE(prob, n, 0, 3)
        uu = u.copy()
        o.integrate(uu, 0.0, (steps - 0.5) * dt, dt)
        return 0.5 * float(np.sum((uu - target) ** 2))

    J0, dJ = orc.tl_misfit(prob, u0, d, target, dt, steps)
    assert abs(J0 - J(u0)) <= 1e-13 * abs(J0)
    h = 1e-5
    fd = (8 * (J(u0 + h * d) - J(u0 - h * d)) - (J(u0 + 2 * h * d) - J(u0 - 2 * h * d))) / (12 * h)
    assert abs(fd - dJ) <= 1e-9 * abs(dJ), (fd, dJ)


def test_results_do_not_depend_on_the_thread_count(orc):
    """The oracle splits the reference's `do concurrent` cell loop (src/hrweno_weno.f90:174) and
    its elementwise stage combines over OpenMP threads; each element's arithmetic is unchanged,
    so 1 and several threads give the same bits (reconstruction, rktvd, mstvd, the 2D
    right-hand side)."""
    import os
    before = orc.set_threads(0)
    many = max(2, min(8, os.cpu_count() or 2))
    try:
        runs = []
        for threads in (1, many):
            assert orc.set_threads(threads) == threads
            rng = np.random.default_rng(5)
            v = rng.standard_normal(3001)
            out = list(orc.reconstruct(v, 3, 1e-6))
            prob = burgers_1d(3001, -5.0, 5.0, k=3, eps=1e-6, flux="godunov", alpha=1.0,
                              bc="zero_inflow", numerics="strict")
            for method in (0, 1):
                u = config1_u0(3001)
                orc.ODE(prob, 3001, method, 3).integrate(u, 0.0, 0.035, 1e-3)
                out.append(u)
            out.append(orc.rhs(pbe_2d(96, 80, k=3, numerics="strict"), np.abs(rng.standard_normal(96 * 80))))
            runs.append(out)
        for a, b in zip(*runs):
            assert np.array_equal(a, b)
    finally:
        orc.set_threads(before)


def test_real32_oracle_keeps_time_in_fp32(orc):
    """The oracle's float instantiation is a REAL32 build: t, tout and dt are FP32 and t
    advances by FP32 additions (src/hrweno_kinds.F90:9-10, src/hrweno_tvdode.f90:170-171), so
    the step count and the final t follow FP32 arithmetic, not FP64."""
    from hrweno import linear_ode
    prob = linear_ode(np.full(4, -1.0))
    for dt, tout in ((0.1, 1.0), (0.01, 12.0), (1e-3, 0.5)):
        o = orc.ODE(prob, 4, 0, 3, prec=32)
        u = np.ones(4)
        t = o.integrate(u, 0.0, tout, dt)
        t32, n = np.float32(0.0), 0
        while not (t32 - np.float32(tout)) > 0:
            t32 = np.float32(t32 + np.float32(dt))
            n += 1
        assert t == float(t32) and o.info()[2] == n
        o64 = orc.ODE(prob, 4, 0, 3, prec=64)
        t64 = o64.integrate(np.ones(4), 0.0, tout, dt)
        assert t64 != t  # FP64 time takes other values
