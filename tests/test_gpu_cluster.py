"""The cluster path of short uniform 1D lines (stage1d_cluster.cu): every step of an integrate
call in one launch of one thread-block cluster, the line in distributed shared memory.

It runs the same reconstruction, flux and combine code as the stage-by-stage kernels, so the
bar is bit-identical results to those kernels (FAST) and to the oracle (STRICT), over the
tile shapes (32, 64 and 256 cells per CTA), a last CTA that owns fewer cells than the stencil
reaches, every order, flux and boundary kind, and the driver loop of the reference's example 1.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def line(nc, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1.0, 1.0, nc)
    return np.exp(-8 * x ** 2) + 0.05 * rng.standard_normal(nc) + np.where(x > 0.3, 0.5, 0.0)


def run(hw, prob, nc, order, u0, tout, dt, cluster, itask=1):
    import torch
    ode = hw.rktvd(prob, nc, order)
    ode.set_cluster(cluster)
    u = torch.from_numpy(u0.copy()).cuda()
    t = ode.integrate(u, 0.0, tout, dt, itask)
    return u.cpu().numpy(), t, ode


NCS = [6, 7, 31, 32, 33, 500, 511, 512, 513, 1000, 1024, 1025, 2049, 4095, 4096, 4097]
PROBS = [dict(flux="lax_friedrichs", bc="copy"), dict(flux="godunov", bc="zero"),
         dict(flux="godunov", bc="zero_inflow")]


@pytest.mark.parametrize("nc", NCS)
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("pi", range(len(PROBS)))
def test_cluster_equals_stage_launches_and_oracle(hw, orc, nc, k, pi):
    u0 = line(nc, nc + k)
    dt = 0.3 * (10.0 / nc) / 1.6
    tout = 7.5 * dt
    for numerics in ("strict", "fast"):
        prob = hw.burgers_1d(nc, k=k, alpha=1.6, numerics=numerics, **PROBS[pi])
        uc, tc, oc = run(hw, prob, nc, 3, u0, tout, dt, True)
        us, ts, _ = run(hw, prob, nc, 3, u0, tout, dt, False)
        assert tc == ts and oc.nsteps == 8
        assert np.array_equal(uc, us), (nc, k, numerics)
        if numerics == "strict":
            uo = u0.copy()
            to = orc.ODE(prob, nc, 0, 3).integrate(uo, 0.0, tout, dt)
            assert to == tc and np.array_equal(uc, uo)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("nc", [33, 700, 3000])
def test_cluster_orders_and_linear_flux(hw, orc, order, nc):
    """Orders 1 and 2 (order 1 alternates its two buffers), and g(x) = a + b x at the interfaces."""
    u0 = line(nc, 3)
    p = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux="godunov", fn=("linear", "linear"),
                   coef_a=(0.4, 0.0), coef_b=(0.3, 0.0), alpha=(0.7, 1.0), bc=("zero_inflow", "copy"),
                   xmin=(-1.0, 0.0), xmax=(1.0, 1.0), numerics="strict")
    dt = 0.2 * (2.0 / nc) / 0.7
    for steps in (1, 9):
        uc, tc, _ = run(hw, p, nc, order, u0, (steps - 0.5) * dt, dt, True)
        us, ts, _ = run(hw, p, nc, order, u0, (steps - 0.5) * dt, dt, False)
        uo = u0.copy()
        to = orc.ODE(p, nc, 0, order).integrate(uo, 0.0, (steps - 0.5) * dt, dt)
        assert tc == ts == to
        assert np.array_equal(uc, uo) and np.array_equal(us, uo)


@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_cluster_example1_driver_loop(hw, orc, numerics):
    """The reference's example 1: 101 integrate calls to the output times, 1201 steps."""
    import torch
    from hrweno import workloads
    prob, u0 = workloads.burgers_config1(numerics=numerics)
    outs = {}
    for cluster in (True, False):
        ode = hw.rktvd(prob, 500, 3)
        ode.set_cluster(cluster)
        u = torch.from_numpy(u0.copy()).cuda()
        t, snaps = 0.0, []
        for i in range(101):
            t = ode.integrate(u, t, 12.0 * i / 100, 1e-2)
            snaps.append(u.cpu().numpy().copy())
        assert ode.nsteps == 1201 and t == 12.009999999999788
        outs[cluster] = snaps
    for a, b in zip(outs[True], outs[False]):
        assert np.array_equal(a, b)
    if numerics == "strict":
        uo = u0.copy()
        o = orc.ODE(prob, 500, 0, 3)
        t = 0.0
        for i in range(101):
            t = o.integrate(uo, t, 12.0 * i / 100, 1e-2)
        assert np.array_equal(outs[True][-1], uo)


def test_cluster_single_steps_and_host_arrays(hw, orc):
    """itask = 2 (one step per call) and host arrays take the same path."""
    prob, u0 = None, None
    from hrweno import workloads
    prob, u0 = workloads.burgers_config1(numerics="strict")
    ode = hw.rktvd(prob, 500, 3)
    u = u0.copy()
    o = orc.ODE(prob, 500, 0, 3)
    uo = u0.copy()
    t = to = 0.0
    for _ in range(5):
        t = ode.integrate(u, t, 1.0, 1e-2, itask=2)
        to = o.integrate(uo, to, 1.0, 1e-2, itask=2)
        assert t == to and np.array_equal(u, uo)
