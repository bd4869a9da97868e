"""Pin the oracle against the reference's own known-answer tests (CPU only).

The reference stores no golden vectors; its unit tests are the known answers for this path:
  test/test_hrweno.f90:29-161   pulse reconstruction (uniform / non-uniform), cnu == c tables
  test/test_fluxes.f90:27-79    consistency and upwinding of lax_friedrichs / godunov
  test/test_tvdode.f90:31-118   rktvd orders 1-3 and mstvd against exp(a (t - t0))
Each test below restates one of them, with the reference's tolerances, on the oracle.
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "kat_reference.json").read_text())


def pulse(nc):
    # v = 0; v(nc/3:2*nc/3) = 1 (1-based, integer division)
    v = np.zeros(nc)
    v[nc // 3 - 1: 2 * nc // 3] = 1.0
    return v


@pytest.mark.parametrize("k", [1, 2, 3])
def test_weno_uniform_pulse(orc, k):
    """test_weno_uniform (test/test_hrweno.f90:29-67): vl = vr = v within 1e-6."""
    v = pulse(30)
    vl, vr = orc.reconstruct(v, k=k, eps=1e-6)
    assert np.all(np.abs(vl - v) <= 1e-6)
    assert np.all(np.abs(vr - v) <= 1e-6)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_calc_cnu_uniform_equals_tables(orc, k):
    """test_calc_cnu (test/test_hrweno.f90:69-112): uniform edges on [0,3] give c1/c2/c3."""
    nc = 30
    xedges = 0.0 + (3.0 - 0.0) * np.arange(nc + 1) / nc
    cnu = orc.calc_cnu(nc, k, xedges)
    cref = np.array(GOLDEN["c_tables"][str(k)])  # [k+1, k]: c(j, r) at [r+1, j]
    for i in range(nc):
        np.testing.assert_allclose(cnu[i], cref, rtol=1e-5, atol=0)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_weno_nonuniform_pulse(orc, k):
    """test_weno_nonuniform (test/test_hrweno.f90:114-161): cubic edges, default eps."""
    nc = 30
    xedges = (0.0 + (1.0 - 0.0) * np.arange(nc + 1) / nc) ** 3
    v = pulse(nc)
    vl, vr = orc.reconstruct(v, k=k, eps=1e-6, xedges=xedges)
    assert np.all(np.abs(vl - v) <= 1e-6)
    assert np.all(np.abs(vr - v) <= 1e-6)


def test_fluxes(orc):
    """test_allfluxes (test/test_fluxes.f90:27-71): f = u x t, alpha = x t, rtol 1e-8."""
    f = lambda u, x, t: u * x * t  # noqa: E731
    x, t, rtol = 3.0, 5.0, 1e-8
    for vm, vp, expect_from in [(2.0, 2.0, 2.0), (2.0, -4.0, 2.0), (-2.0, 4.0, -2.0)]:
        href = f(expect_from, x, t)
        for kind in (0, 1):
            h = orc.numflux(kind, orc.FLUX_TEST_UXT, vm, vp, x, t, alpha=x * t)
            assert abs(h - href) <= rtol * abs(href), (kind, vm, vp, h, href)


RATES = [-1.0 + (ii - 1) * 4.0 / 9 for ii in range(1, 11)]


@pytest.mark.parametrize("order,rtol", [(1, 2e-2), (2, 1e-3), (3, 1e-3)])
def test_rktvd_linear(orc, order, rtol):
    """test_rktvd (test/test_tvdode.f90:31-70): u' = a u, t0=-1.3, tout=1.5, dt=(tout-t0)/3000."""
    from hrweno.problems import linear_ode
    a = np.array(RATES)
    t0, tout = -1.3, 1.5
    dt = (tout - t0) / 3000
    ode = orc.ODE(linear_ode(a), 10, method=0, order=order)
    u = np.full(10, 0.1)
    t = ode.integrate(u, t0, tout, dt)
    uref = 0.1 * np.exp(a * (t - t0))
    assert np.all(np.abs(u - uref) <= rtol * np.abs(uref))


def test_mstvd_linear(orc):
    """test_mstvd (test/test_tvdode.f90:72-104): dt=1e-3, rtol 1e-3."""
    from hrweno.problems import linear_ode
    a = np.array(RATES)
    t0, tout = -1.3, 1.5
    ode = orc.ODE(linear_ode(a), 10, method=1)
    u = np.full(10, 0.1)
    t = ode.integrate(u, t0, tout, 1e-3)
    uref = 0.1 * np.exp(a * (t - t0))
    assert np.all(np.abs(u - uref) <= 1e-3 * np.abs(uref))


def test_tables_match_reference_literals():
    """The c/d tables of the fixture are the reference's literals (src/hrweno_weno.f90:11-21)."""
    c3 = np.array(GOLDEN["c_tables"]["3"])
    assert np.allclose(c3[0], [11 / 6, -7 / 6, 1 / 3]) and np.allclose(c3[3], [1 / 3, -7 / 6, 11 / 6])
    assert GOLDEN["d_tables"]["3"] == [0.3, 0.6, 0.1]


def test_fv_nonuniform_uniform_edges_match_uniform_line(orc):
    """A non-uniform line whose edges are uniform reproduces the uniform line to rounding:
    cnu equals the c tables (test/test_hrweno.f90:69-112) and the widths equal dx."""
    from hrweno.problems import burgers_1d
    nc = 64
    x = np.linspace(-1, 1, nc)
    v = 0.5 + np.exp(-10 * x ** 2)
    p_u = burgers_1d(nc, -1.0, 1.0, k=3, alpha=1.5)
    p_n = burgers_1d(nc, -1.0, 1.0, k=3, alpha=1.5)
    p_n.xedges = (-1.0 + 2.0 * np.arange(nc + 1) / nc, None)
    a, b = orc.rhs(p_u, v), orc.rhs(p_n, v)
    assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(a))
