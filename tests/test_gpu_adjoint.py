"""The discrete adjoint (hrw_adjoint_*) against the tangent-linear oracle and finite differences.

  grad . d  vs  the oracle's tangent-linear dJ(d) (dual numbers through the reference-order
            forward map): relative difference <= 1e-10
  J         vs  the oracle's forward solve: relative difference <= 1e-12
  central finite differences on the GPU forward map: relative difference <= 1e-6
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def line(n, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-5, 5, n)
    u = np.zeros(n)
    for _ in range(4):
        u += rng.uniform(0.2, 1.0) * np.exp(-((x - rng.uniform(-4, 4)) / rng.uniform(0.3, 1.0)) ** 2)
    return u


def smooth_direction(n, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, n)
    d = np.zeros(n)
    for m in range(1, 9):
        d += rng.standard_normal() * np.sin(np.pi * m * x + rng.uniform(0, 6.28)) / m
    return d


CASES = [
    dict(k=3, fn="burgers", bc="copy"), dict(k=2, fn="burgers", bc="zero"),
    dict(k=1, fn="burgers", bc="zero_inflow"), dict(k=3, fn="linear", bc="zero_inflow"),
    dict(k=3, fn="burgers", bc="zero_inflow"), dict(k=2, fn="linear", bc="copy"),
]


def problem(hw, n, k, fn, bc):
    a, b = (0.7, 0.1) if fn == "linear" else (1.0, 0.0)
    return hw.Problem(kind="fv1d", ncells=(n, 1), k=k, eps=1e-6, flux="lax_friedrichs",
                      fn=(fn, fn), coef_a=(a, 0), coef_b=(b, 0), alpha=(1.5, 1.5), bc=(bc, bc),
                      xmin=(-5.0, 0.0), xmax=(5.0, 1.0))


@pytest.mark.parametrize("case", range(len(CASES)))
def test_adjoint_vs_tangent_linear(hw, orc, case):
    n, steps = 400, 60
    prob = problem(hw, n, **CASES[case])
    u0 = line(n, case)
    target = line(n, case + 100) * 0.8
    dt = 0.4 * (10.0 / n) / 1.5
    adj = hw.adjoint(prob, checkpoint_every=7)
    J, g = adj.gradient(u0, target, dt, steps)
    for s in range(3):
        d = np.random.default_rng(s).standard_normal(n) if s else smooth_direction(n, s)
        Jo, dJ = orc.tl_misfit(prob, u0, d, target, dt, steps)
        assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
        assert abs(g @ d - dJ) <= 1e-10 * max(abs(dJ), 1e-30), (case, s, g @ d, dJ)
    assert adj.forward_steps == steps + (steps - steps % 7 if steps % 7 else steps - 7)


def stretched_edges(n, seed):
    """Edges on [-5, 5] with random widths in a 1:3 range."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.5, 1.5, n)
    return np.concatenate([[-5.0], -5.0 + np.cumsum(w) * (10.0 / w.sum())])


NU_CASES = CASES + [dict(k=3, fn="burgers_linear", bc="copy"), dict(k=2, fn="burgers", bc="zero_inflow")]


@pytest.mark.parametrize("case", range(len(NU_CASES)))
def test_adjoint_nonuniform_vs_tangent_linear(hw, orc, case):
    """weno(ncells, k, eps, xedges) in the adjoint: each cell's coefficients in the candidates
    and their transposes, the cells' own widths in the flux adjoints, g at the true edges."""
    n, steps = 400, 60
    c = NU_CASES[case]
    a, b = (0.7, 0.1) if c["fn"] != "burgers" else (1.0, 0.0)
    xe = stretched_edges(n, case)
    prob = hw.Problem(kind="fv1d", ncells=(n, 1), k=c["k"], eps=1e-6, flux="lax_friedrichs",
                      fn=(c["fn"], c["fn"]), coef_a=(a, 0), coef_b=(b, 0), alpha=(1.5, 1.5),
                      bc=(c["bc"], c["bc"]), xedges=(xe, None))
    xc = 0.5 * (xe[1:] + xe[:-1])
    u0 = np.interp(xc, np.linspace(-5, 5, n), line(n, case))
    target = np.interp(xc, np.linspace(-5, 5, n), line(n, case + 100)) * 0.8
    dt = 0.4 * np.min(np.diff(xe)) / 2.0
    adj = hw.adjoint(prob, checkpoint_every=7)
    J, g = adj.gradient(u0, target, dt, steps)
    assert adj.tape_bytes[1] == 0  # the reverse recomputes the non-uniform maps
    for s in range(3):
        d = np.random.default_rng(s).standard_normal(n) if s else smooth_direction(n, s)
        Jo, dJ = orc.tl_misfit(prob, u0, d, target, dt, steps)
        assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
        assert abs(g @ d - dJ) <= 1e-10 * max(abs(dJ), 1e-30), (case, s, g @ d, dJ)


def test_adjoint_nonuniform_forward_and_batch(hw):
    """The adjoint's forward map on a non-uniform line is hrw_integrate's (same bits), and a
    batch of segments on the same edges matches one-segment solves."""
    n, nseg, steps = 256, 3, 40
    xe = stretched_edges(n, 11)
    prob = hw.Problem(kind="fv1d", ncells=(n, 1), k=3, eps=1e-6, flux="lax_friedrichs",
                      fn=("burgers", "burgers"), alpha=(1.5, 1.5), bc=("zero_inflow", "zero_inflow"),
                      xedges=(xe, None))
    dt = 0.4 * np.min(np.diff(xe)) / 1.5
    u0 = np.concatenate([line(n, s) for s in range(nseg)])
    tg = np.concatenate([line(n, 50 + s) * 0.9 for s in range(nseg)])
    _, uT = hw.adjoint(prob).forward(u0[:n], None, dt, steps, uT=np.empty(n))
    ui = u0[:n].copy()
    hw.rktvd(prob, n, 3).integrate(ui, 0.0, (steps - 0.5) * dt, dt)
    assert np.array_equal(uT, ui)
    Jb, gb = hw.adjoint(prob, nseg=nseg, checkpoint_every=9).gradient(u0, tg, dt, steps)
    for s in range(nseg):
        sl = slice(s * n, (s + 1) * n)
        J1, g1 = hw.adjoint(prob, checkpoint_every=9).gradient(u0[sl], tg[sl], dt, steps)
        assert np.array_equal(gb[sl], g1)
        assert abs(Jb[s] - J1[0]) <= 1e-13 * J1[0]


def test_adjoint_checkpoint_interval_invariant(hw):
    n, steps = 300, 50
    prob = problem(hw, n, 3, "burgers", "copy")
    u0, target = line(n, 1), line(n, 2) * 0.9
    dt = 0.4 * (10.0 / n) / 1.5
    ref = None
    for every in (1, 6, 50, 1000, 0):
        J, g = hw.adjoint(prob, checkpoint_every=every).gradient(u0, target, dt, steps)
        if ref is None:
            ref = (J, g)
        assert np.array_equal(g, ref[1]) and abs(J[0] - ref[0][0]) <= 1e-14 * ref[0][0]


def test_adjoint_weno_tape_used(hw, orc):
    """The pass that records a segment keeps the WENO tape (20 doubles per cell and stage for
    k = 3, 12 for k = 2, none for k = 1); the gradient through it agrees with the tangent-linear
    oracle as the recompute path does."""
    n, steps = 256, 20
    for k, nq in ((3, 20), (2, 12), (1, 0)):
        prob = problem(hw, n, k, "burgers", "copy")
        u0, target = line(n, 7), line(n, 8) * 0.9
        dt = 0.4 * (10.0 / n) / 1.5
        adj = hw.adjoint(prob, checkpoint_every=5)
        J, g = adj.gradient(u0, target, dt, steps)
        sb, wb = adj.tape_bytes
        assert sb == 8 * n * (3 * 5 + 1) and wb == 8 * n * nq * 3 * 5
        d = smooth_direction(n, 3)
        _, dJ = orc.tl_misfit(prob, u0, d, target, dt, steps)
        assert abs(g @ d - dJ) <= 1e-10 * abs(dJ)


def test_adjoint_batch_matches_single(hw):
    n, nseg, steps = 256, 5, 40
    prob = problem(hw, n, 3, "burgers", "zero_inflow")
    dt = 0.4 * (10.0 / n) / 1.5
    u0 = np.concatenate([line(n, s) for s in range(nseg)])
    tg = np.concatenate([line(n, 50 + s) * 0.9 for s in range(nseg)])
    Jb, gb = hw.adjoint(prob, nseg=nseg, checkpoint_every=9).gradient(u0, tg, dt, steps)
    for s in range(nseg):
        sl = slice(s * n, (s + 1) * n)
        J1, g1 = hw.adjoint(prob, checkpoint_every=9).gradient(u0[sl], tg[sl], dt, steps)
        assert np.array_equal(gb[sl], g1)
        assert abs(Jb[s] - J1[0]) <= 1e-13 * J1[0]


def test_adjoint_central_differences(hw):
    """Central finite differences of the GPU forward map in 6 directions."""
    import torch
    n, steps = 1 << 14, 200
    prob = problem(hw, n, 3, "burgers", "copy")
    u0 = torch.from_numpy(line(n, 3)).cuda()
    tg = torch.from_numpy(line(n, 4) * 0.9).cuda()
    dt = 0.4 * (10.0 / n) / 1.5
    adj = hw.adjoint(prob, checkpoint_every=15)
    J, g = adj.gradient(u0, tg, dt, steps)
    for s in range(6):
        d = torch.from_numpy(smooth_direction(n, 10 + s)).cuda()
        h = 1e-5 * float(u0.abs().max()) / float(d.abs().max())
        Jp, _ = adj.forward(u0 + h * d, tg, dt, steps)
        Jm, _ = adj.forward(u0 - h * d, tg, dt, steps)
        fd = (Jp[0] - Jm[0]) / (2 * h)
        gd = float((g * d).sum())
        assert abs(fd - gd) <= 1e-6 * abs(gd), (s, fd, gd)


def test_torch_autograd_op(hw):
    """loss = 0.5 ||weno_solve(u0) - target||^2; loss.backward() gives the adjoint gradient,
    and a general upstream gradient matches the tangent-linear oracle."""
    import torch
    n, steps = 512, 80
    prob = problem(hw, n, 3, "burgers", "copy")
    dt = 0.4 * (10.0 / n) / 1.5
    u0 = torch.from_numpy(line(n, 5)).cuda().requires_grad_(True)
    tg = torch.from_numpy(line(n, 6) * 0.9).cuda()
    uT = hw.weno_solve(u0, prob, dt, steps)
    loss = 0.5 * ((uT - tg) ** 2).sum()
    loss.backward()
    J, g = hw.adjoint(prob, checkpoint_every=0).gradient(u0.detach(), tg, dt, steps)
    assert abs(loss.item() - J[0]) <= 1e-13 * J[0]
    assert torch.equal(u0.grad, g)
    # batched lines with a weighted loss
    u0b = torch.from_numpy(np.stack([line(n, 7), line(n, 8)])).cuda().requires_grad_(True)
    w = torch.linspace(0.5, 2.0, n, dtype=torch.float64, device="cuda")
    (hw.weno_solve(u0b, prob, dt, steps) * w).sum().backward()
    g1 = hw.adjoint(prob).vjp(u0b.detach()[1].contiguous(), w.contiguous(), dt, steps)
    assert torch.equal(u0b.grad[1], g1)


def test_torch_autograd_op_nonuniform(hw, orc):
    """The autograd op on a non-uniform line: the forward is hrw_integrate's, the backward the
    non-uniform adjoint; d(loss)/du0 . d matches the tangent-linear oracle."""
    import torch
    n, steps = 384, 50
    xe = stretched_edges(n, 21)
    prob = hw.Problem(kind="fv1d", ncells=(n, 1), k=3, eps=1e-6, flux="lax_friedrichs",
                      fn=("burgers", "burgers"), alpha=(1.5, 1.5), bc=("copy", "copy"), xedges=(xe, None))
    dt = 0.4 * np.min(np.diff(xe)) / 1.5
    u0n, tgn = line(n, 9), line(n, 10) * 0.9
    u0 = torch.from_numpy(u0n).cuda().requires_grad_(True)
    tg = torch.from_numpy(tgn).cuda()
    uT = hw.weno_solve(u0, prob, dt, steps)
    ui = u0n.copy()
    hw.rktvd(prob, n, 3).integrate(ui, 0.0, (steps - 0.5) * dt, dt)
    assert np.array_equal(uT.detach().cpu().numpy(), ui)
    (0.5 * ((uT - tg) ** 2).sum()).backward()
    d = smooth_direction(n, 4)
    _, dJ = orc.tl_misfit(prob, u0n, d, tgn, dt, steps)
    assert abs(float(u0.grad.cpu().numpy() @ d) - dJ) <= 1e-10 * abs(dJ)
    # edges edited in place (same array, same address): the op builds a new handle
    xe[1:-1] = 0.5 * (xe[1:-1] + np.linspace(-5.0, 5.0, n + 1)[1:-1])
    uT2 = hw.weno_solve(u0.detach(), prob, dt, steps)
    ui = u0n.copy()
    hw.rktvd(prob, n, 3).integrate(ui, 0.0, (steps - 0.5) * dt, dt)
    assert np.array_equal(uT2.cpu().numpy(), ui)


def test_torch_op_follows_an_edited_problem(hw):
    """weno_solve keeps one adjoint handle per problem; editing the problem between calls gives
    the edited problem's solve, not the cached handle's."""
    import torch
    n, steps = 256, 20
    prob = problem(hw, n, 3, "burgers", "copy")
    dt = 0.4 * (10.0 / n) / 2.0
    u0 = torch.from_numpy(line(n, 9)).cuda()
    a = hw.weno_solve(u0, prob, dt, steps)
    prob.alpha = (2.0, 2.0)
    b = hw.weno_solve(u0, prob, dt, steps)
    _, ref = hw.adjoint(prob).forward(u0, None, dt, steps, uT=torch.empty_like(u0))
    assert torch.equal(b, ref) and not torch.equal(a, b)
