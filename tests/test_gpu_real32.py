"""REAL32 (dtype "f32", HRW_F32): what a REAL32 build of the reference computes, against the
oracle's float instantiation on the same inputs.

A REAL32 build (src/hrweno_kinds.F90:9-10, rk = real32) holds every real in FP32: the state,
eps, the grid and cnu, every flux and stage, and the time t, tout and dt.  The GPU path runs the
reference's operation order in FP32, so the bar is bit-identical results, the same final t
(an FP32 value) and the same step count.
"""
import ctypes as C

import numpy as np
import pytest

from hrweno import workloads

pytestmark = pytest.mark.gpu


def f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def line(nc, seed, kind="smooth"):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, nc)
    if kind == "smooth":
        v = np.sin(3 * x) + 0.3 * np.cos(7 * x) + 0.1 * rng.standard_normal(nc)
    elif kind == "pulse":
        v = np.zeros(nc)
        v[nc // 3 - 1: 2 * nc // 3] = 1.0
    else:
        v = rng.uniform(-1, 1, nc)
    return f32(v)


def gpu_rhs32(prob, v):
    import torch
    from hrweno import _abi as A
    tv = torch.from_numpy(v).cuda()
    out = torch.empty_like(tv)
    cp = prob.to_c()
    A.check(A.lib().hrw_rhs(C.byref(cp), A.HRW_F32, 0.0, tv.data_ptr(), out.data_ptr(), None))
    return out.cpu().numpy()


NCS = [1, 2, 3, 5, 30, 1023, 1025, 5000, 80000]


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", NCS)
def test_reconstruct_uniform_f32(hw, orc, k, nc):
    import torch
    for seed, kind in [(1, "smooth"), (2, "pulse"), (3, "noise")]:
        v = line(nc, seed, kind)
        rl, rr = orc.reconstruct(v.astype(np.float64), k=k, eps=1e-6, prec=32)
        w = hw.weno(nc, k, 1e-6)
        vl, vr = np.empty(nc, np.float32), np.empty(nc, np.float32)
        w.reconstruct(v, vl, vr)
        assert np.array_equal(vl.astype(np.float64), rl) and np.array_equal(vr.astype(np.float64), rr)
        tv = torch.from_numpy(v).cuda()
        tl, tr = torch.empty_like(tv), torch.empty_like(tv)
        w.reconstruct(tv, tl, tr)
        assert np.array_equal(tl.cpu().numpy(), vl) and np.array_equal(tr.cpu().numpy(), vr)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 5, 30, 777])
def test_reconstruct_nonuniform_f32(hw, orc, k, nc):
    rng = np.random.default_rng(nc + k)
    xedges = np.cumsum(np.concatenate([[0.0], rng.uniform(0.5, 1.5, nc)])) / nc
    v = line(nc, 4)
    rl, rr = orc.reconstruct(v.astype(np.float64), k=k, eps=1e-6, xedges=xedges, prec=32)
    w = hw.weno(nc, k, 1e-6, xedges=xedges)
    vl, vr = np.empty(nc, np.float32), np.empty(nc, np.float32)
    w.reconstruct(v, vl, vr)
    assert np.array_equal(vl.astype(np.float64), rl) and np.array_equal(vr.astype(np.float64), rr)
    # the FP64 reconstruction of the same handle is unchanged by the REAL32 call
    v64 = v.astype(np.float64)
    dl, dr = np.empty(nc), np.empty(nc)
    w.reconstruct(v64, dl, dr)
    ol, orr = orc.reconstruct(v64, k=k, eps=1e-6, xedges=xedges)
    assert np.max(np.abs(dl - ol)) <= 1e-13 * max(1.0, np.max(np.abs(ol)))


def test_reconstruct_f32_eps_below_fp32_epsilon(hw):
    """eps = 1e-8 is valid for REAL64 but not for REAL32 (eps > epsilon(1._rk),
    src/hrweno_weno.f90:92): the REAL32 reconstruction refuses with the reference's message."""
    w = hw.weno(16, 3, 1e-8)
    v = np.zeros(16, np.float32)
    with pytest.raises(hw.HrwError, match="eps"):
        w.reconstruct(v, v.copy(), v.copy())


PROBS_1D = [
    dict(flux="lax_friedrichs", bc="copy"),
    dict(flux="godunov", bc="copy"),
    dict(flux="godunov", bc="zero"),
    dict(flux="lax_friedrichs", bc="zero_inflow"),
]


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("pi", range(len(PROBS_1D)))
@pytest.mark.parametrize("nc", [1, 2, 6, 1000, 2049, 320000])
def test_rhs_1d_burgers_f32(hw, orc, k, pi, nc):
    v = line(nc, 7, "noise")
    prob = hw.burgers_1d(nc, k=k, alpha=1.2, **PROBS_1D[pi])
    ref = orc.rhs(prob, v.astype(np.float64), prec=32)
    assert np.array_equal(gpu_rhs32(prob, v).astype(np.float64), ref)


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("fn,coef", [("linear", (0.7, 0.0)), ("linear", (-0.2, 0.6)),
                                     ("burgers_linear", (0.3, -0.4))])
@pytest.mark.parametrize("grid", ["uniform", "width", "xedges"])
def test_rhs_1d_flux_kinds_and_grids_f32(hw, orc, flux, fn, coef, grid):
    nc = 333
    rng = np.random.default_rng(11)
    v = line(nc, 8)
    p = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux=flux, fn=(fn, fn), coef_a=(coef[0], 0.0),
                   coef_b=(coef[1], 0.0), alpha=(abs(coef[0]) + abs(coef[1]) + 1.0, 1.0),
                   bc=("zero_inflow", "copy"), xmin=(-1.0, 0.0), xmax=(2.0, 1.0))
    if grid == "width":
        p.width = (rng.uniform(0.8, 1.2, nc) * (3.0 / nc), None)
    elif grid == "xedges":
        p.xedges = (-1.0 + 3.0 * np.linspace(0.0, 1.0, nc + 1) ** 1.5, None)
    ref = orc.rhs(p, v.astype(np.float64), prec=32)
    assert np.array_equal(gpu_rhs32(p, v).astype(np.float64), ref)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("n1,n2", [(1, 1), (5, 3), (64, 48), (100, 37), (130, 260)])
@pytest.mark.parametrize("flux", ["godunov", "lax_friedrichs"])
def test_rhs_2d_pbe_f32(hw, orc, k, n1, n2, flux):
    """n1 a multiple of 4 stages the tile by TMA (16-byte rows of floats), others by loads."""
    prob, n0, _ = workloads.pbe_config(n1, n2, k=k)
    prob.flux = flux
    v = f32(n0 + 0.01 * np.random.default_rng(3).standard_normal(n0.size))
    ref = orc.rhs(prob, v.astype(np.float64), prec=32)
    assert np.array_equal(gpu_rhs32(prob, v).astype(np.float64), ref)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("n1,n2", [(5, 3), (64, 48), (100, 37)])
def test_rhs_2d_nonuniform_f32(hw, orc, k, n1, n2):
    prob, n0, _ = workloads.pbe_config(n1, n2, k=k)
    w1 = 1.02 ** np.arange(n1)
    prob.xedges = (np.concatenate([[0.0], np.cumsum(w1) / w1.sum()]), None)
    v = f32(n0 + 0.01 * np.random.default_rng(5).standard_normal(n0.size))
    ref = orc.rhs(prob, v.astype(np.float64), prec=32)
    assert np.array_equal(gpu_rhs32(prob, v).astype(np.float64), ref)


def run_both(hw, orc, prob, n, u0, method, order, t0, tout, dt, itask=1, mem="device", graphs=True):
    import torch
    mk = (lambda: hw.rktvd(prob, n, order, dtype="f32")) if method == 0 else \
        (lambda: hw.mstvd(prob, n, dtype="f32"))
    ode = mk()
    ode.set_graphs(graphs)
    u = torch.from_numpy(u0.copy()).cuda() if mem == "device" else u0.copy()
    tg = ode.integrate(u, t0, tout, dt, itask)
    got = u.cpu().numpy() if mem == "device" else u
    o = orc.ODE(prob, n, method, order, prec=32)
    uo = u0.astype(np.float64)
    to = o.integrate(uo, t0, tout, dt, itask)
    assert np.isfinite(uo).all()
    return got.astype(np.float64), uo, tg, to, ode, o


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("mem", ["device", "host"])
def test_rktvd_config1_f32(hw, orc, order, mem):
    """The reference's example 1 (500 cells, CFL-limited dt, t to 12) in REAL32."""
    prob, u0 = workloads.burgers_config1()
    u0 = f32(u0)
    dt = 0.01
    got, ref, tg, to, ode, o = run_both(hw, orc, prob, 500, u0, 0, order, 0.0, 12.0, dt, mem=mem)
    assert tg == to and np.array_equal(got, ref)
    fe, st, ns = o.info()
    assert (ode.fevals, ode.istate, ode.nsteps) == (fe, st, ns)
    # t accumulates in FP32: t = t + dt with t, dt, tout rounded to FP32
    t32, d32, n32 = np.float32(0.0), np.float32(dt), 0
    while not (t32 - np.float32(12.0)) > 0:
        t32 = np.float32(t32 + d32)
        n32 += 1
    assert tg == float(t32) and ode.nsteps == n32


def test_rktvd_f32_driver_loop_and_graphs(hw, orc):
    """101 output calls of the example driver, graphs on and off, equal bits throughout."""
    import torch
    prob, u0 = workloads.burgers_config1()
    u0 = f32(u0)
    dt = 0.01
    outs = []
    for graphs in (True, False):
        ode = hw.rktvd(prob, 500, 3, dtype="f32")
        ode.set_graphs(graphs)
        u = torch.from_numpy(u0.copy()).cuda()
        t = 0.0
        snaps = []
        for i in range(1, 101):
            t = ode.integrate(u, t, 0.12 * i, dt)
            snaps.append(u.cpu().numpy().copy())
        outs.append((t, snaps))
    o = orc.ODE(prob, 500, 0, 3, prec=32)
    uo = u0.astype(np.float64)
    t = 0.0
    for i in range(1, 101):
        t = o.integrate(uo, t, 0.12 * i, dt)
        for tg, snaps in outs:
            assert np.array_equal(snaps[i - 1].astype(np.float64), uo), i
    assert outs[0][0] == outs[1][0] == t


@pytest.mark.parametrize("k", [2, 3])
def test_rktvd_large_line_f32(hw, orc, k):
    """A 2^20-cell line of the large 1D case for 50 steps (the 1024-cell tile shape)."""
    n = 1 << 20
    prob, u0, dt = workloads.large_burgers(n, k=k)
    got, ref, tg, to, _, _ = run_both(hw, orc, prob, n, f32(u0), 0, 3, 0.0, 49.5 * dt, dt)
    assert tg == to and np.array_equal(got, ref)


@pytest.mark.parametrize("mem", ["device", "host"])
def test_mstvd_pbe_f32(hw, orc, mem):
    n1, n2 = 96, 64
    prob, n0, dt = workloads.pbe_config(n1, n2, cfl=0.3)
    got, ref, tg, to, ode, o = run_both(hw, orc, prob, n1 * n2, f32(n0), 1, 3, 0.0, 60.5 * dt, dt,
                                        mem=mem)
    assert tg == to and np.array_equal(got, ref)
    assert (ode.fevals, ode.istate, ode.nsteps) == o.info()


def test_mstvd_1d_f32_two_calls(hw, orc):
    """mstvd keeps its history between calls (src/hrweno_tvdode.f90:228-249).  CFL 0.25: the
    5-step method is unstable at the example's CFL 0.5."""
    import torch
    prob, u0 = workloads.burgers_config1()
    u0 = f32(u0)
    dt = 0.005
    ode = hw.mstvd(prob, 500, dtype="f32")
    o = orc.ODE(prob, 500, 1, prec=32)
    u = torch.from_numpy(u0.copy()).cuda()
    uo = u0.astype(np.float64)
    t = to = 0.0
    for tout in (0.5, 1.0, 3.0):
        t = ode.integrate(u, t, tout, dt)
        to = o.integrate(uo, to, tout, dt)
        assert np.isfinite(uo).all()
        assert t == to and np.array_equal(u.cpu().numpy().astype(np.float64), uo)


@pytest.mark.parametrize("method,order", [(0, 1), (0, 2), (0, 3), (1, 3)])
def test_linear_ode_f32(hw, orc, method, order):
    rates = np.linspace(-2.0, -0.1, 64)
    prob = hw.linear_ode(rates)
    u0 = f32(np.linspace(1.0, 2.0, 64))
    got, ref, tg, to, _, _ = run_both(hw, orc, prob, 64, u0, method, order, 0.0, 1.0, 0.01)
    assert tg == to and np.array_equal(got, ref)


def test_f32_integrate_refuses_float64_and_stalled_dt(hw):
    import torch
    prob, u0 = workloads.burgers_config1()
    ode = hw.rktvd(prob, 500, 3, dtype="f32")
    with pytest.raises(TypeError):
        ode.integrate(torch.from_numpy(u0).cuda(), 0.0, 1.0, 0.01)
    u = torch.from_numpy(f32(u0)).cuda()
    # at t = 1e4 an FP32 step of 1e-4 leaves t unchanged: refused, as it would never end
    with pytest.raises(hw.HrwError, match="never reached"):
        ode.integrate(u, 1.0e4, 1.0e4 + 1.0, 1e-4)
    assert ode.istate == 1
