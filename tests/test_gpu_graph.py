"""Graph replay of integrate loops gives the same bits as launching every stage directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(ode, u, t0, touts, dt):
    t = t0
    for tout in touts:
        t = ode.integrate(u, t, tout, dt)
    return t


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("dtype", ["f64", "f32c"])
def test_rktvd_graphs_bitwise(hw, order, dtype):
    from hrweno import workloads
    n = 3000
    prob, u0, dt = workloads.large_burgers(n, k=3)
    touts = [dt * s for s in (0.5, 13.5, 26.5, 39.5, 150.5, 151.5, 280.5)]  # 1, 13, 13, 13, 111, 1, 129 steps
    if order == 1:
        touts = touts[:4]
    res = []
    for graphs in (True, False):
        ode = hw.rktvd(prob, n, order, dtype=dtype)
        ode.set_graphs(graphs)
        u = u0.copy()
        t = run(ode, u, 0.0, touts, dt)
        res.append((t, u, ode.nsteps, ode.fevals))
    assert res[0][0] == res[1][0] and res[0][2:] == res[1][2:]
    assert np.array_equal(res[0][1], res[1][1])


def test_config1_graphs_vs_oracle(hw, orc):
    """The 500-cell driver loop (101 output times, 12 steps per call) replays one graph per
    call; STRICT numerics stay bit-identical to the oracle."""
    from hrweno import workloads
    prob, u0 = workloads.burgers_config1(numerics="strict")
    g, o = hw.rktvd(prob, 500, 3), orc.ODE(prob, 500, 0, 3)
    ug, uo = u0.copy(), u0.copy()
    tg = to = 0.0
    for ii in range(101):
        tout = 12.0 * ii / 100
        tg = g.integrate(ug, tg, tout, 1e-2)
        to = o.integrate(uo, to, tout, 1e-2)
    assert tg == to and np.array_equal(ug, uo)


def test_mstvd_graphs_bitwise(hw):
    from hrweno import workloads
    n1 = n2 = 48
    prob, n0, dt = workloads.pbe_config(n1, n2)
    res = []
    for graphs in (True, False):
        ode = hw.mstvd(prob, n1 * n2)
        ode.set_graphs(graphs)
        u = n0.copy()
        t = run(ode, u, 0.0, [dt * s for s in (0.5, 30.5, 95.5, 97.5, 180.5)], dt)
        res.append((t, u, ode.nsteps))
    assert res[0][0] == res[1][0] and res[0][2] == res[1][2]
    assert np.array_equal(res[0][1], res[1][1])
