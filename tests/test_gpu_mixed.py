"""MIXED numerics (HRW_NUMERICS_MIXED: FP64 state, right-hand side in difference form on the
FP32 pipe) through the C ABI, against the oracle and against the FAST path.

Bar: max|gpu - oracle| / max|oracle| <= 1e-12 (normwise relative), as for FAST; the pointwise
relative error with a floor of 1e-3 max|oracle| is printed beside it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def prel(a, b):
    den = np.maximum(np.abs(b), 1e-3 * np.max(np.abs(b)))
    return float(np.max(np.abs(a - b) / den))


def diag():
    from hrweno import _abi as A
    L = A.lib()
    L.hrw_diag_mixed_soft.argtypes = [C.c_int]
    L.hrw_diag_mixed_soft.restype = C.c_int
    L.hrw_diag_mixed_hard_warps.argtypes = [C.POINTER(C.c_ulonglong), C.c_int]
    L.hrw_diag_mixed_hard_warps.restype = C.c_int
    return L


def hard_warps(reset=True):
    n = C.c_ulonglong()
    assert diag().hrw_diag_mixed_hard_warps(C.byref(n), int(reset)) == 0
    return n.value


def line(hw, n, k, fn, numerics):
    from hrweno import workloads
    prob, u0, dt = workloads.large_burgers(n, k=k, numerics=numerics)
    if fn == "linear":
        prob = hw.Problem(kind="fv1d", ncells=(n, 1), k=k, flux="lax_friedrichs", fn=("linear", "linear"),
                          coef_a=(-0.7, 0.0), coef_b=(0.0, 0.0), alpha=(1.0, 1.0), bc=("copy", "copy"),
                          xmin=(-5.0, 0.0), xmax=(5.0, 1.0), numerics=numerics)
        dt = 0.4 * (10.0 / n)
    return prob, u0, dt


@pytest.mark.parametrize("order", [3, 2, 1])
@pytest.mark.parametrize("fn", ["burgers", "linear"])
@pytest.mark.parametrize("k", [3, 2])
def test_mixed_vs_oracle(hw, orc, k, fn, order):
    import torch
    n, steps = 1 << 20, 41
    prob, u0, dt = line(hw, n, k, fn, "mixed")
    sprob, _, _ = line(hw, n, k, fn, "strict")
    ug = torch.from_numpy(u0).cuda()
    ode = hw.rktvd(prob, n, order)
    hard_warps()
    tg = ode.integrate(ug, 0.0, (steps - 0.5) * dt, dt)
    hw_ = hard_warps()
    uo = u0.copy()
    o = orc.ODE(sprob, n, 0, order)
    to = o.integrate(uo, 0.0, (steps - 0.5) * dt, dt)
    got = ug.cpu().numpy()
    assert tg == to and ode.nsteps == steps and ode.fevals == o.info()[0]
    e, p = nrel(got, uo), prel(got, uo)
    warps = (n // 128) * steps * order
    print(f"mixed k={k} {fn} order {order}: normwise {e:.3e}, pointwise {p:.3e}, "
          f"FP64-path warps {hw_ / warps:.3f}")
    assert e <= TOL
    assert hw_ < warps  # the FP32 path carried part of the line


def test_mixed_takes_the_fp32_path_on_a_resolved_line(hw):
    """On the 2^22-cell line almost every warp away from the line ends takes the FP32 path."""
    import torch
    n = 1 << 22
    prob, u0, dt = line(hw, n, 3, "burgers", "mixed")
    ug = torch.from_numpy(u0).cuda()
    hard_warps()
    hw.rktvd(prob, n, 3).integrate(ug, 0.0, 0.5 * dt, dt)
    frac = hard_warps() / (3 * (n // 128))
    print(f"2^22 cells: FP64-path warps {frac:.4f}")
    assert frac < 0.05


def test_mixed_fp64_path_alone(hw, orc):
    """With the FP32 path switched off, every warp runs the FAST arithmetic in increment form:
    still within 1e-12 of the oracle."""
    import torch
    L = diag()
    n, steps = 1 << 18, 30
    prob, u0, dt = line(hw, n, 3, "burgers", "mixed")
    sprob, _, _ = line(hw, n, 3, "burgers", "strict")
    assert L.hrw_diag_mixed_soft(0) == 0
    try:
        ug = torch.from_numpy(u0).cuda()
        hw.rktvd(prob, n, 3).integrate(ug, 0.0, (steps - 0.5) * dt, dt)
    finally:
        assert L.hrw_diag_mixed_soft(1) == 0
    uo = u0.copy()
    orc.ODE(sprob, n, 0, 3).integrate(uo, 0.0, (steps - 0.5) * dt, dt)
    assert nrel(ug.cpu().numpy(), uo) <= TOL


@pytest.mark.parametrize("steps", [5, 70, 129])
def test_mixed_graphs_host_and_device_bits(hw, steps):
    """Graph replay and direct launches, device and page-locked host arrays: the same bits
    (an odd step count ends in the second state buffer, copied back)."""
    import torch
    n = 1 << 17
    prob, u0, dt = line(hw, n, 3, "burgers", "mixed")
    res = []
    for graphs in (True, False):
        for host in (False, True):
            ode = hw.rktvd(prob, n, 3)
            ode.set_graphs(graphs)
            u = torch.from_numpy(u0.copy()).pin_memory() if host else torch.from_numpy(u0.copy()).cuda()
            ode.integrate(u, 0.0, (steps - 0.5) * dt, dt)
            res.append(u.cpu().numpy())
    for r in res[1:]:
        assert np.array_equal(r, res[0])


@pytest.mark.parametrize("n", [1 << 20, (1 << 20) + 777])
@pytest.mark.parametrize("steps", [1, 2, 5])
def test_mixed_host_pipeline_bits(hw, n, steps):
    """Page-locked host lines of at least 2 x SMs x 1024 cells take the chunked pipeline (the
    last step's second and third stages by chunks, each chunk copied back behind its third
    stage): the same bits as the device-array call, for one and several steps, a ragged last
    chunk, and single steps (itask = 2) in a row."""
    import torch
    prob, u0, dt = line(hw, n, 3, "burgers", "mixed")
    ode = hw.rktvd(prob, n, 3)
    ud = torch.from_numpy(u0.copy()).cuda()
    td = ode.integrate(ud, 0.0, (steps - 0.5) * dt, dt)
    oh = hw.rktvd(prob, n, 3)
    uh = torch.from_numpy(u0.copy()).pin_memory()
    th = oh.integrate(uh, 0.0, (steps - 0.5) * dt, dt)
    assert th == td and np.array_equal(uh.numpy(), ud.cpu().numpy())
    os_ = hw.rktvd(prob, n, 3)
    us = torch.from_numpy(u0.copy()).pin_memory()
    ts = 0.0
    for _ in range(steps):  # from the second call on, the pipelined step on the guessed scale
        ts = os_.integrate(us, ts, 1e9, dt, itask=2)
    assert ts == td and np.array_equal(us.numpy(), ud.cpu().numpy())


def test_mixed_host_pipeline_guess_missed(hw):
    """A driver that changes the host line between calls (here: scales it by 4 and by 1/3, which
    moves the exponent of max|u|, and by 1.01, which keeps it): a call whose guess of the scale
    misses takes the step again from the device copy of its input; every call gives the bits
    of the device-array path on the same input."""
    import torch
    n = (1 << 20) + 2048
    prob, u0, dt = line(hw, n, 3, "burgers", "mixed")
    prob.alpha = (4.0 * float(np.max(np.abs(u0))), 1.0)
    oh, od = hw.rktvd(prob, n, 3), hw.rktvd(prob, n, 3)
    uh = torch.from_numpy(u0.copy()).pin_memory()
    th = td = 0.0
    for factor in (1.0, 1.0, 4.0, 1.01, 1.0 / 3.0, 1.0):
        uh.mul_(factor)
        ud = uh.clone().cuda()
        th = oh.integrate(uh, th, 1e9, 0.25 * dt, itask=2)
        td = od.integrate(ud, td, 1e9, 0.25 * dt, itask=2)
        assert th == td and np.array_equal(uh.numpy(), ud.cpu().numpy()), factor


def test_mixed_elsewhere_runs_fast(hw):
    """Where the MIXED kernel does not apply (a short line, Godunov, mstvd, one right-hand side)
    MIXED gives FAST's bits."""
    import torch
    from hrweno import workloads
    cases = []
    p1, u1 = workloads.burgers_config1("mixed")
    f1, _ = workloads.burgers_config1("fast")
    cases.append(("rktvd", p1, f1, u1, 1e-2, 100))
    n = 1 << 17
    pg, ug0, dtg = workloads.large_burgers(n, k=3, numerics="mixed")
    fg, _, _ = workloads.large_burgers(n, k=3, numerics="fast")
    pg.flux = fg.flux = "godunov"
    cases.append(("rktvd", pg, fg, ug0, dtg, 20))
    cases.append(("mstvd", pg, fg, ug0, dtg, 20))
    for method, pm, pf, u0, dt, steps in cases:
        out = []
        for p in (pm, pf):
            u = torch.from_numpy(u0.copy()).cuda()
            ode = hw.rktvd(p, u0.size, 3) if method == "rktvd" else hw.mstvd(p, u0.size)
            ode.integrate(u, 0.0, (steps - 0.5) * dt, dt)
            out.append(u.cpu().numpy())
        assert np.array_equal(out[0], out[1]), method


def test_mixed_rejects_tiny_eps(hw):
    prob, _, _ = line(hw, 1 << 17, 3, "burgers", "mixed")
    prob.eps = 1e-9
    with pytest.raises(hw.HrwError, match="HRW_NUMERICS_MIXED needs eps >= 1e-8"):
        hw.rktvd(prob, 1 << 17, 3)
