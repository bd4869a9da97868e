"""A second, independent restatement of the reference's formulas -- vectorised numpy, written
from src/hrweno_weno.f90, src/hrweno_fluxes.f90, src/hrweno_tvdode.f90 and the two example
drivers -- against the C++ oracle on random and generated inputs (CPU only).  The oracle is
pinned to the reference's known-answer tests; this checks it everywhere else, to rounding level
(numpy sums in its own order).

The same restatement also carries the rearranged algebra the GPU kernels use (the FAST product
form, the compensated FP32 difference form, the adjoint's transposes), so that each
rearrangement is shown equal to the reference's formulas independently of the kernels' own
rounding, which the GPU tests check."""
import numpy as np
import pytest

# method constants (src/hrweno_weno.f90:12-21): linear weights d and stencil coefficients c(j, r),
# r = -1 .. k-1 (stored here at column r + 1)
D = {1: np.array([1.0]), 2: np.array([2 / 3, 1 / 3]), 3: np.array([0.3, 0.6, 0.1])}
C = {
    1: np.array([[1.0, 1.0]]),
    2: np.array([[3 / 2, 1 / 2, -1 / 2], [-1 / 2, 1 / 2, 3 / 2]]),
    3: np.array([[11 / 6, 1 / 3, -1 / 6, 1 / 3], [-7 / 6, 5 / 6, 5 / 6, -7 / 6], [1 / 3, -1 / 6, 1 / 3, 11 / 6]]),
}


def reconstruct_np(v, k, eps, cn=None, weights=None):
    """weno%reconstruct (src/hrweno_weno.f90:163-215): (vl, vr) of every cell.  cn: per-cell
    coefficients [nc, k+1, k] of a non-uniform grid (cell i's c(j, r) at cn[i-1, r+1, j]),
    used as the reference uses cnu(:, :, i) (:170,177-181); None: the uniform tables.
    weights: optional map applied to the normalised weights (w, w~) before the sums."""
    nc = v.size
    ext = np.concatenate([np.full(k - 1, v[0]), v, np.full(k - 1, v[-1])])  # vext, ghosts replicate
    at = lambda o: ext[k - 1 + o: k - 1 + o + nc]  # noqa: E731  vext(i + o) for every cell i
    coef = (lambda j, col: C[k][j, col]) if cn is None else (lambda j, col: cn[:, col, j])  # noqa: E731
    vrr = np.zeros((k, nc), dtype=np.result_type(v, float))  # complex lines: complex-step tests
    vlr = np.zeros_like(vrr)
    for r in range(k):
        for j in range(k):
            vrr[r] += coef(j, r + 1) * at(j - r)
            vlr[r] += coef(j, r) * at(j - r)
    if k == 1:
        beta = np.zeros((1, nc))
    elif k == 2:
        beta = np.array([(at(1) - at(0)) ** 2, (at(0) - at(-1)) ** 2])
    else:
        beta = np.array([
            13 / 12 * (at(0) - 2 * at(1) + at(2)) ** 2 + 1 / 4 * (3 * at(0) - 4 * at(1) + at(2)) ** 2,
            13 / 12 * (at(-1) - 2 * at(0) + at(1)) ** 2 + 1 / 4 * (at(-1) - at(1)) ** 2,
            13 / 12 * (at(-2) - 2 * at(-1) + at(0)) ** 2 + 1 / 4 * (at(-2) - 4 * at(-1) + 3 * at(0)) ** 2,
        ])
    s = (eps + beta) ** 2
    alfa = D[k][:, None] / s
    alfat = D[k][::-1, None] / s
    if weights is not None:
        w, wt = weights(alfa / alfa.sum(0), alfat / alfat.sum(0))
        return (wt * vlr).sum(0), (w * vrr).sum(0)
    return (alfat * vlr).sum(0) / alfat.sum(0), (alfa * vrr).sum(0) / alfa.sum(0)


def rhs_burgers_np(v, xmin, xmax, k, eps, flux, alpha, bc):
    """example1's right-hand side (example/example1_burgers_1d_fv.f90:72-109) with its
    boundary rules and the fluxes of src/hrweno_fluxes.f90:43,67-74."""
    nc = v.size
    vl, vr = reconstruct_np(v, k, eps)
    f = lambda u: u * u / 2  # noqa: E731
    vm, vp = vr[:-1], vl[1:]
    if flux == "lax_friedrichs":
        inner = (f(vm) + f(vp) - alpha * (vp - vm)) / 2
    else:
        fm, fp = f(vm), f(vp)
        inner = np.where(vm <= vp, np.minimum(fm, fp), np.maximum(fm, fp))
    F = np.zeros(nc + 1)
    F[1:nc] = inner
    if bc == "copy" and nc > 1:
        F[0], F[nc] = F[1], F[nc - 1]
    elif bc == "zero_inflow":
        F[nc] = f(vr[-1])
    dx = (xmax - xmin) / nc
    return -(F[1:] - F[:-1]) / dx


def lines(nc, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, nc)
    yield np.sin(2 * x) + 0.5 * np.exp(-20 * x * x)          # smooth
    yield np.where(np.abs(x) < 0.4, 1.0, 0.1) + 0.01 * x      # discontinuous
    yield rng.standard_normal(nc)                             # rough, sign changes


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 3, 5, 64, 1001])
def test_reconstruct_matches_numpy(orc, k, nc):
    for v in lines(nc, nc + k):
        vl, vr = orc.reconstruct(v, k, 1e-6)
        nl, nr = reconstruct_np(v, k, 1e-6)
        scale = max(np.max(np.abs(v)), 1e-300)
        assert np.max(np.abs(vl - nl)) <= 1e-13 * scale and np.max(np.abs(vr - nr)) <= 1e-13 * scale


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
@pytest.mark.parametrize("nc", [2, 7, 500])
def test_burgers_rhs_matches_numpy(hw, orc, k, flux, bc, nc):
    for v in lines(nc, 3 * nc + k):
        prob = hw.burgers_1d(nc, -5.0, 5.0, k=k, eps=1e-6, flux=flux, alpha=1.3, bc=bc, numerics="strict")
        ref = orc.rhs(prob, v)
        got = rhs_burgers_np(v, -5.0, 5.0, k, 1e-6, flux, 1.3, bc)
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.max(np.abs(got - ref)) <= 1e-12 * scale, (k, flux, bc, nc)


def numflux_np(flux, f, vm, vp, alpha):
    """lax_friedrichs / godunov (src/hrweno_fluxes.f90:43,67-74), elementwise."""
    if flux == "lax_friedrichs":
        return (f(vm) + f(vp) - alpha * (vp - vm)) / 2
    fm, fp = f(vm), f(vp)
    return np.where(vm <= vp, np.minimum(fm, fp), np.maximum(fm, fp))


def sweep_np(lines_, k, eps, flux, alpha, bc, g_at, dx):
    """One direction of example2's right-hand side (example/example2_pbe_2d_fv.f90:96-120) for a
    stack of lines [m, n]: -dF/dx of f = g(x) u with g at the interfaces (g_at(e), e = 0..n)."""
    m, n = lines_.shape
    out = np.empty_like(lines_)
    ge = g_at(np.arange(n + 1))
    for r in range(m):
        vl, vr = reconstruct_np(lines_[r], k, eps)
        F = np.zeros(n + 1)
        g = ge[1:n]
        F[1:n] = numflux_np(flux, lambda u: g * u, vr[:-1], vl[1:], alpha)  # noqa: B023
        if bc == "copy" and n > 1:
            F[0], F[n] = F[1], F[n - 1]
        elif bc == "zero_inflow":
            F[n] = ge[n] * vr[-1]
        out[r] = -(F[1:] - F[:-1]) / dx
    return out


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["zero", "zero_inflow", "copy"])
@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (40, 24)])
def test_pbe_rhs_matches_numpy(hw, orc, flux, bc, shape):
    """example2's dimension-by-dimension right-hand side, u((j-1) n1 + i): x1 rows, then x2
    columns, vdot = -dF1/dx1 - dF2/dx2 (:123-127)."""
    n1, n2 = shape
    g1, g2 = (1.0, 0.5), (0.5, -0.2)
    prob = hw.pbe_2d(n1, n2, g1=g1, g2=g2, k=3, flux=flux, bc=bc, numerics="strict")
    rng = np.random.default_rng(n1 + n2)
    v = np.abs(rng.standard_normal(n1 * n2)) + 0.1
    ref = orc.rhs(prob, v)
    u = v.reshape(n2, n1)
    dx1, dx2 = 1.0 / n1, 1.0 / n2
    a1 = sweep_np(u, 3, 1e-6, flux, abs(g1[0]) + abs(g1[1]), bc,
                  lambda e: g1[0] + g1[1] * (e * dx1), dx1)
    a2 = sweep_np(u.T.copy(), 3, 1e-6, flux, abs(g2[0]) + abs(g2[1]), bc,
                  lambda e: g2[0] + g2[1] * (e * dx2), dx2).T
    got = (a1 + a2).reshape(-1)
    scale = max(np.max(np.abs(ref)), 1e-300)
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale


def rk3_step(u, dt, L):
    """src/hrweno_tvdode.f90:160-171 (the stage formulas as written)."""
    u1 = u + dt * L(u)
    u2 = (3 * u + u1 + dt * L(u1)) / 4
    return (u + 2 * u2 + 2 * dt * L(u2)) / 3


def test_rktvd3_and_mstvd_match_numpy(hw, orc):
    """rktvd(3) steps and mstvd (its RK3 start and equation 4.26 with the history shift,
    src/hrweno_tvdode.f90:236-265) restated in numpy on example1's right-hand side."""
    nc, dt = 200, 5e-3
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy",
                         numerics="strict")
    x = -5.0 + 10.0 / nc * (np.arange(nc) + 0.5)
    u0 = np.exp(-x * x)
    L = lambda u: rhs_burgers_np(u, -5.0, 5.0, 3, 1e-6, "lax_friedrichs", 1.0, "copy")  # noqa: E731
    # rktvd(3), 12 steps
    u = u0.copy()
    for _ in range(12):
        u = rk3_step(u, dt, L)
    o = orc.ODE(prob, nc, 0, 3)
    uo = u0.copy()
    o.integrate(uo, 0.0, 11.5 * dt, dt)
    assert np.max(np.abs(uo - u)) <= 1e-12 * np.max(np.abs(u))
    # mstvd: 4 RK3 start steps recording u and L(u) (oldest first), then 10 multistep steps
    u = u0.copy()
    hu, hl = [], []
    for _ in range(4):
        hu.append(u.copy())
        hl.append(L(u))
        u = rk3_step(u, dt, L)
    for _ in range(10):
        ud = L(u)
        ui = (25 * u + 50 * dt * ud + 7 * hu[0] + 10 * dt * hl[0]) / 32
        hu = hu[1:] + [u.copy()]
        hl = hl[1:] + [ud]
        u = ui
    o = orc.ODE(prob, nc, 1)
    uo = u0.copy()
    o.integrate(uo, 0.0, 13.5 * dt, dt)
    assert np.max(np.abs(uo - u)) <= 1e-12 * np.max(np.abs(u))


# ---- non-uniform grids ------------------------------------------------------------------------
def cnu_moments(xe, k):
    """c(j, r) of every cell of the grid with edges xe(0:nc), found without Shu's eq. 2.20: the
    polynomial p of degree k-1 whose averages over cells i-r .. i-r+k-1 are the given values is
    solved for from the averages of the monomials ((x - x_{i+1/2}) / h)^q, and c(j, r) is the
    weight of cell i-r+j in p(x_{i+1/2}).  Edges beyond the line continue the end cells' widths
    (src/hrweno_weno.f90:245-255).  Returns [nc, k+1, k] (cell i's c(j, r) at [i-1, r+1, j])."""
    nc, ng = xe.size - 1, k + 1
    ext = np.concatenate([xe[0] - (xe[1] - xe[0]) * np.arange(ng, 0, -1), xe,
                          xe[-1] + (xe[-1] - xe[-2]) * np.arange(1, ng + 1)])
    edge = lambda e: ext[e + ng]  # noqa: E731  x_{e+1/2}; cell m spans [edge(m-1), edge(m)]
    out = np.empty((nc, k + 1, k))
    q = np.arange(k)
    for i in range(1, nc + 1):
        x0 = edge(i)
        for r in range(-1, k):
            cells = i - r + np.arange(k)
            h = edge(cells[-1]) - edge(cells[0] - 1)
            sl = (np.array([edge(m - 1) for m in cells]) - x0) / h
            sr = (np.array([edge(m) for m in cells]) - x0) / h
            # M[a, q]: average of s^q over cell a of the stencil
            M = (sr[:, None] ** (q + 1) - sl[:, None] ** (q + 1)) / ((q + 1) * (sr - sl)[:, None])
            out[i - 1, r + 1] = np.linalg.solve(M.T, np.eye(k)[0])  # p(x0) = a_0 = e0 . M^-1 v
    return out


def grids(nc, seed):
    rng = np.random.default_rng(seed)
    yield "cubic", -1.0 + 2.0 * (np.arange(nc + 1) / nc) ** 3  # test/test_hrweno.f90:123-128
    yield "random", np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, nc))])
    yield "geometric", np.concatenate([[0.0], np.cumsum(1.1 ** np.arange(nc))])


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 5, 40])
def test_cnu_matches_moment_solve(orc, k, nc):
    """weno_calc_cnu (src/hrweno_weno.f90:221-297) against coefficients found by a linear solve
    instead of Shu's closed form, ghost edges included."""
    for name, xe in grids(nc, nc + k):
        ref = orc.calc_cnu(nc, k, xe)
        got = cnu_moments(xe, k)
        assert np.max(np.abs(got - ref)) <= 1e-11 * max(1.0, np.max(np.abs(ref))), (name, k, nc)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 3, 40, 301])
def test_nonuniform_reconstruct_matches_numpy(orc, k, nc):
    for name, xe in grids(nc, 7 * nc + k):
        cn = cnu_moments(xe, k)
        for v in lines(nc, nc + k):
            vl, vr = orc.reconstruct(v, k, 1e-6, xe)
            nl, nr = reconstruct_np(v, k, 1e-6, cn)
            scale = max(np.max(np.abs(v)), 1e-300)
            assert np.max(np.abs(vl - nl)) <= 1e-11 * scale, (name, k, nc)
            assert np.max(np.abs(vr - nr)) <= 1e-11 * scale, (name, k, nc)


def test_nonuniform_left_states_use_cell_i_coefficients(orc):
    """On a non-uniform grid the reference forms vl(i) with cell i's coefficients c(:, r-1, i)
    (src/hrweno_weno.f90:170,181); the set that reproduces polynomials exactly at x_{i-1/2} is
    cell i-1's.  The oracle keeps the reference's choice (the GPU path matches the oracle bit for
    bit), so vl is exact for polynomials of degree k-1 only where the two sets coincide: on
    grids with a constant ratio of neighbouring widths (uniform, geometric and logarithmic
    grids: the stencils of cells i and i-1 are scaled copies of each other).  vr is exact on
    every grid.  Cell averages of p(x) = 1 + 2x - 0.3x^2, k = 3, cells away from the ends."""
    nc, k = 40, 3
    P = lambda x: x + x ** 2 - 0.1 * x ** 3  # noqa: E731  a primitive of p
    p = lambda x: 1 + 2 * x - 0.3 * x ** 2  # noqa: E731
    inner = slice(4, nc - 4)
    for name, xe in [("uniform", np.linspace(0.0, 4.0, nc + 1))] + list(grids(nc, 3)):
        v = (P(xe[1:]) - P(xe[:-1])) / np.diff(xe)
        vl, vr = orc.reconstruct(v, k, 1e-6, xe)
        assert np.max(np.abs(vr[inner] - p(xe[1:][inner]))) <= 1e-10 * np.max(np.abs(v)), name
        cn = cnu_moments(xe, k)
        shifted = np.concatenate([cn[:1], cn[:-1]])  # cell i-1's coefficients for cell i
        left = np.stack([sum(shifted[:, r, j] * np.concatenate([v[:1]] * 2 + [v] + [v[-1:]] * 2)[2 - r + j: 2 - r + j + nc]
                             for j in range(k)) for r in range(k)])
        assert np.max(np.abs(left[:, inner] - p(xe[:-1][inner]))) <= 1e-10 * np.max(np.abs(v)), name
        err = np.max(np.abs(vl[inner] - p(xe[:-1][inner])))
        if name in ("uniform", "geometric"):
            assert err <= 1e-10 * np.max(np.abs(v)), (name, err)
        else:
            assert err > 1e-6, (name, err)


def rktvd_np(u, t, tout, dt, order, L, itask=1):
    """rktvd_integrate (src/hrweno_tvdode.f90:122-178): the stage formulas as written, t = t + dt
    per step and the stopping test is_done (:282); returns (u, t, fevals)."""
    done = lambda tt: (tt - tout) * np.copysign(1.0, dt) > 0  # noqa: E731
    if done(t):
        return u, t, 0
    fe = 0
    while True:
        if order == 1:
            u = u + dt * L(u)
        elif order == 2:
            ui = u + dt * L(u)
            u = (u + ui + dt * L(ui)) / 2
        else:
            u = rk3_step(u, dt, L)
        t = t + dt
        fe += order
        if done(t) or itask == 2:
            return u, t, fe


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("itask", [1, 2])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_rktvd_orders_times_and_fevals_match_numpy(hw, orc, order, itask, sign):
    """Every rktvd order, one step (itask 2) or a run to tout (itask 1), forward and backward in
    time: the oracle's u, t and fevals against the numpy restatement of the time loop."""
    nc = 120
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="godunov", alpha=1.0, bc="zero_inflow",
                         numerics="strict")
    x = -5.0 + 10.0 / nc * (np.arange(nc) + 0.5)
    u0 = 0.2 + np.exp(-x * x)
    L = lambda u: rhs_burgers_np(u, -5.0, 5.0, 3, 1e-6, "godunov", 1.0, "zero_inflow")  # noqa: E731
    dt, t0 = sign * 2e-3, 0.1
    tout = t0 + sign * 0.0137  # not a multiple of dt: the last step passes tout
    un, tn, fen = rktvd_np(u0.copy(), t0, tout, dt, order, L, itask)
    o = orc.ODE(prob, nc, 0, order)
    uo = u0.copy()
    to = o.integrate(uo, t0, tout, dt, itask)
    assert to == tn and o.info()[0] == fen
    assert np.max(np.abs(uo - un)) <= 1e-12 * np.max(np.abs(un))


def test_weights_need_more_than_fp32_precision():
    """How precisely must the nonlinear weights be computed to keep the 1e-12 agreement?  The
    large 1D configuration's problem (seeded 8-Gaussian u0, WENO5, Lax-Friedrichs, copy
    boundaries, RK3 at CFL 0.4) on 2^12 cells for 600 steps, with every weight perturbed by a
    random relative error of at most rel and renormalised: at rel = 2^-44 (float-pair
    arithmetic) the solution stays at the rounding floor, at rel = 2^-24 (FP32 weights) it
    leaves 1e-12 as the shocks form.  Weights in plain FP32 are therefore no route to a faster
    FP64 stage."""
    nc, steps = 1 << 12, 600
    x = -5.0 + 10.0 / nc * (np.arange(nc) + 0.5)
    rng0 = np.random.default_rng(1)
    u0 = np.zeros(nc)
    for _ in range(8):
        a, c, w = rng0.uniform(0.2, 1.0), rng0.uniform(-4.0, 4.0), rng0.uniform(0.05, 0.5)
        u0 += a * np.exp(-((x - c) / w) ** 2)
    alpha = float(np.max(np.abs(u0)))
    dx = 10.0 / nc
    dt = 0.4 * dx / alpha
    f = lambda u: u * u / 2  # noqa: E731

    def rhs(v, weights):
        vl, vr = reconstruct_np(v, 3, 1e-6, weights=weights)
        F = np.zeros(nc + 1)
        F[1:nc] = (f(vr[:-1]) + f(vl[1:]) - alpha * (vl[1:] - vr[:-1])) / 2
        F[0], F[nc] = F[1], F[nc - 1]
        return -(F[1:] - F[:-1]) / dx

    def run(rel):
        rng = np.random.default_rng(0)

        def perturb(w, wt):
            w = w * (1.0 + rel * rng.uniform(-1.0, 1.0, w.shape))
            wt = wt * (1.0 + rel * rng.uniform(-1.0, 1.0, wt.shape))
            return w / w.sum(0), wt / wt.sum(0)

        u = u0.copy()
        for _ in range(steps):
            u = rk3_step(u, dt, lambda v: rhs(v, perturb if rel else None))  # noqa: B023
        return u

    exact = run(0.0)
    err = {rel: np.max(np.abs(run(rel) - exact)) / np.max(np.abs(exact)) for rel in (2.0 ** -44, 2.0 ** -24)}
    assert err[2.0 ** -44] <= 1e-13, err
    assert err[2.0 ** -24] > 1e-11, err


def test_reconstruct_matches_numpy_on_generated_lines(orc):
    """Generated cases: line lengths 1..300, every k, eps from 1e-12 to 1e-2, values spread over
    twelve decades and of either sign, uniform and non-uniform grids."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=150, deadline=None, derandomize=True)
    @hyp.given(nc=st.integers(1, 300), k=st.integers(1, 3), log_eps=st.floats(-12.0, -2.0),
               log_scale=st.floats(-6.0, 6.0), seed=st.integers(0, 2 ** 31 - 1),
               nonuniform=st.booleans())
    def check(nc, k, log_eps, log_scale, seed, nonuniform):
        rng = np.random.default_rng(seed)
        eps = 10.0 ** log_eps
        v = 10.0 ** log_scale * rng.standard_normal(nc) * np.where(rng.random(nc) < 0.1, 100.0, 1.0)
        xe = np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, nc))]) if nonuniform else None
        vl, vr = orc.reconstruct(v, k, eps, xe)
        nl, nr = reconstruct_np(v, k, eps, cnu_moments(xe, k) if nonuniform else None)
        scale = np.max(np.abs(v))
        tol = (1e-11 if nonuniform else 1e-13) * scale
        assert np.max(np.abs(vl - nl)) <= tol and np.max(np.abs(vr - nr)) <= tol

    check()


def rhs1d_np(v, k, eps, flux, fn, a, b, alpha, bc, edges, width, cn=None):
    """example1's right-hand side generalised as the problem descriptor describes it
    (example/example1_burgers_1d_fv.f90:72-109): fluxes at the interior edges x_{i+1/2} with
    f = u^2/2, (a + b x) u or their sum, the boundary rule, and -dF / width.  Returns (vdot, F)."""
    nc = v.size
    vl, vr = reconstruct_np(v, k, eps, cn)

    def f(u, x):
        if fn == "burgers":
            return u * u / 2
        if fn == "linear":
            return (a + b * x) * u
        return u * u / 2 + (a + b * x) * u

    F = np.zeros(nc + 1)
    xi = edges[1:nc]
    F[1:nc] = numflux_np(flux, lambda u: f(u, xi), vr[:-1], vl[1:], alpha)
    if bc == "copy":
        F[0], F[nc] = F[1], F[nc - 1]
    elif bc == "zero_inflow":
        F[nc] = f(vr[-1], edges[nc])
    return -(F[1:] - F[:-1]) / width, F


def test_rhs_matches_numpy_on_generated_problems(hw, orc):
    """Generated 1D problems: every flux function (with x-dependent velocity), numerical flux and
    boundary rule, on uniform grids, uniform grids with given widths, and non-uniform edges."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=200, deadline=None, derandomize=True)
    @hyp.given(nc=st.integers(2, 200), k=st.integers(1, 3),
               fn=st.sampled_from(["burgers", "linear", "burgers_linear"]),
               flux=st.sampled_from(["lax_friedrichs", "godunov"]),
               bc=st.sampled_from(["copy", "zero", "zero_inflow"]),
               grid=st.sampled_from(["uniform", "width", "xedges"]), seed=st.integers(0, 2 ** 31 - 1))
    def check(nc, k, fn, flux, bc, grid, seed):
        rng = np.random.default_rng(seed)
        a, b, alpha = rng.uniform(-1.0, 1.0), rng.uniform(-0.5, 0.5), 1.7
        xmin, xmax = -2.0, 3.0
        v = rng.standard_normal(nc) * np.where(rng.random(nc) < 0.2, 3.0, 0.3)
        rx = (xmax - xmin) / nc
        edges = xmin + rx * np.arange(nc + 1)
        width = np.full(nc, rx)
        kw = {}
        cn = None
        if grid == "width":
            width = rng.uniform(0.5, 1.5, nc) * rx
            kw["width"] = (width, None)
        elif grid == "xedges":
            edges = xmin + np.concatenate([[0.0], np.cumsum(rng.uniform(0.5, 1.5, nc))]) * rx
            width = np.diff(edges)
            kw["xedges"] = (edges, None)
            cn = orc.calc_cnu(nc, k, edges)
        prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, eps=1e-6, flux=flux, fn=(fn, fn),
                          coef_a=(a, 0.0), coef_b=(b, 0.0), alpha=(alpha, alpha), bc=(bc, bc),
                          xmin=(xmin, 0.0), xmax=(xmax, 1.0), numerics="strict", **kw)
        ref = orc.rhs(prob, v)
        got, F = rhs1d_np(v, k, 1e-6, flux, fn, a, b, alpha, bc, edges, width, cn)
        scale = max(np.max(np.abs(F)) / np.min(width), 1e-300)
        assert np.max(np.abs(got - ref)) <= 1e-13 * scale, (nc, k, fn, flux, bc, grid)

    check()


def test_2d_rhs_matches_numpy_on_generated_problems(hw, orc):
    """Generated 2D problems (example2's dimension-by-dimension right-hand side,
    example/example2_pbe_2d_fv.f90:96-127): per direction its own flux function, velocity
    a + b x_d at the interfaces and boundary rule; rectangular grids of 2..40 cells a side."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    fns = st.sampled_from(["burgers", "linear", "burgers_linear"])
    bcs = st.sampled_from(["copy", "zero", "zero_inflow"])

    @hyp.settings(max_examples=100, deadline=None, derandomize=True)
    @hyp.given(n1=st.integers(2, 40), n2=st.integers(2, 40), k=st.integers(1, 3), fn1=fns, fn2=fns,
               bc1=bcs, bc2=bcs, flux=st.sampled_from(["lax_friedrichs", "godunov"]),
               seed=st.integers(0, 2 ** 31 - 1))
    def check(n1, n2, k, fn1, fn2, bc1, bc2, flux, seed):
        rng = np.random.default_rng(seed)
        a, b = rng.uniform(-1.0, 1.0, 2), rng.uniform(-0.5, 0.5, 2)
        alpha = (1.3, 0.9)
        xmin, xmax = (0.0, -1.0), (2.0, 1.5)
        v = rng.standard_normal(n1 * n2) * 0.5 + 1.0
        prob = hw.Problem(kind="fv2d", ncells=(n1, n2), k=k, eps=1e-6, flux=flux, fn=(fn1, fn2),
                          coef_a=tuple(a), coef_b=tuple(b), alpha=alpha, bc=(bc1, bc2),
                          xmin=xmin, xmax=xmax, numerics="strict")
        ref = orc.rhs(prob, v)
        u = v.reshape(n2, n1)  # u((j-1) n1 + i): rows are x1 lines
        got = np.zeros_like(u)
        scale = 0.0
        for d, (n, fn, bc, lines_) in enumerate([(n1, fn1, bc1, u), (n2, fn2, bc2, u.T)]):
            rx = (xmax[d] - xmin[d]) / n
            edges = xmin[d] + rx * np.arange(n + 1)
            part = np.empty_like(lines_)
            for r in range(lines_.shape[0]):
                part[r], F = rhs1d_np(lines_[r].copy(), k, 1e-6, flux, fn, a[d], b[d], alpha[d], bc,
                                      edges, np.full(n, rx))
                scale = max(scale, np.max(np.abs(F)) / rx)
            got += part if d == 0 else part.T
        assert np.max(np.abs(got.reshape(-1) - ref)) <= 1e-13 * max(scale, 1e-300), \
            (n1, n2, k, fn1, fn2, bc1, bc2, flux)

    check()


def mstvd_np(state, u, t, tout, dt, L):
    """mstvd_integrate (src/hrweno_tvdode.f90:203-271): on the first call four RK3 start steps
    record u and L(u) (run even past tout), then equation 4.26 until is_done, shifting the
    history.  state carries the history and fevals between calls; returns (u, t)."""
    done = lambda tt: (tt - tout) * np.copysign(1.0, dt) > 0  # noqa: E731
    if done(t):
        return u, t
    if not state:
        state.update(hu=[], hl=[], fe=0)
        for _ in range(4):
            state["hu"].append(u.copy())
            state["hl"].append(L(u))
            u = rk3_step(u, dt, L)
            t = t + dt
        state["fe"] = 12
    while not done(t):
        ud = L(u)
        ui = (25 * u + 50 * dt * ud + 7 * state["hu"][0] + 10 * dt * state["hl"][0]) / 32
        t = t + dt
        state["fe"] += 1
        state["hu"] = state["hu"][1:] + [u.copy()]
        state["hl"] = state["hl"][1:] + [ud]
        u = ui
    return u, t


def test_time_loops_match_numpy_on_generated_calls(hw, orc):
    """Generated call sequences of the integrators on the linear test ODE u_i' = a_i u_i
    (test/test_tvdode.f90:107-111): start time, two output times, dt of either sign and size,
    itask, rktvd orders 1-3 and mstvd across two integrate calls.  The oracle's u, t and fevals
    against the numpy restatement of the reference's time loops."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=150, deadline=None, derandomize=True)
    @hyp.given(t0=st.floats(-2.0, 2.0), d1=st.floats(-0.4, 0.4), d2=st.floats(-0.4, 0.4),
               h=st.floats(1e-3, 0.05), sign=st.sampled_from([1.0, -1.0]),
               method=st.sampled_from(["rk1", "rk2", "rk3", "ms"]), itask=st.sampled_from([1, 2]))
    def check(t0, d1, d2, h, sign, method, itask):
        rates = np.linspace(-1.0, 3.0, 10)
        prob = hw.linear_ode(rates, numerics="strict")
        L = lambda u: rates * u  # noqa: E731
        dt = sign * h
        ms = method == "ms"
        order = 3 if ms else int(method[-1])
        o = orc.ODE(prob, rates.size, 1 if ms else 0, order)
        uo, un = np.full(10, 0.1), np.full(10, 0.1)
        to = tn = t0
        fe, state = 0, {}
        for tout in (t0 + d1, t0 + d1 + d2):
            to = o.integrate(uo, to, tout, dt, 1 if ms else itask)
            if ms:
                un, tn = mstvd_np(state, un, tn, tout, dt, L)
                fe = state.get("fe", 0)
            else:
                un, tn, f = rktvd_np(un, tn, tout, dt, order, L, itask)
                fe += f
            assert to == tn and o.info()[0] == fe, (method, to, tn, o.info(), fe)
            assert np.max(np.abs(uo - un)) <= 1e-13 * np.max(np.abs(un))

    check()


def reconstruct_product_form_np(v, k, eps):
    """The FAST kernels' algebra for k = 2, 3, restated in numpy with true divisions: candidates
    scaled to integer stencils, the k = 3 indicators from per-centre terms D, eps + 13/12 D^2 and
    H (E0(j) = D(j+1) + H(j+1), E1(j) = H(j), E2(j) = D(j-1) - H(j-1)), and the weights in product
    form w_r = d_r P_r / sum d_q P_q with P_r the product of the other (eps + beta)^2."""
    nc = v.size
    ext = np.concatenate([np.full(k - 1, v[0]), v, np.full(k - 1, v[-1])])
    at = lambda o: ext[k - 1 + o: k - 1 + o + nc]  # noqa: E731
    if k == 2:
        V0, V1 = at(0) + at(1), 3 * at(0) - at(-1)
        W0, W1 = 3 * at(0) - at(1), at(-1) + at(0)
        s0 = (eps + (at(1) - at(0)) ** 2) ** 2
        s1 = (eps + (at(0) - at(-1)) ** 2) ** 2
        den, dent = 2 * s1 + s0, s1 + 2 * s0
        return (s1 * W0 + 2 * s0 * W1) / (2 * dent), (2 * s1 * V0 + s0 * V1) / (2 * den)
    D = lambda o: at(o - 1) - 2 * at(o) + at(o + 1)  # noqa: E731
    H = lambda o: 0.5 * (at(o - 1) - at(o + 1))  # noqa: E731
    A = lambda o: eps + 13 / 12 * D(o) ** 2  # noqa: E731
    e0 = (D(1) + H(1)) ** 2 + A(1)
    e1 = H(0) ** 2 + A(0)
    e2 = (D(-1) - H(-1)) ** 2 + A(-1)
    s0, s1, s2 = e0 ** 2, e1 ** 2, e2 ** 2
    P0, P1, P2 = s1 * s2, s0 * s2, s0 * s1
    V0 = 2 * at(0) + 5 * at(1) - at(2)
    V1 = -at(-1) + 5 * at(0) + 2 * at(1)
    V2 = 2 * at(-2) - 7 * at(-1) + 11 * at(0)
    W0 = 11 * at(0) - 7 * at(1) + 2 * at(2)
    W1 = 2 * at(-1) + 5 * at(0) - at(1)
    W2 = -at(-2) + 5 * at(-1) + 2 * at(0)
    den, dent = 3 * P0 + 6 * P1 + P2, P0 + 6 * P1 + 3 * P2
    return ((3 * P2 * W2 + 6 * P1 * W1 + P0 * W0) / (6 * dent),
            (3 * P0 * V0 + 6 * P1 * V1 + P2 * V2) / (6 * den))


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("nc", [1, 2, 5, 64, 1001])
def test_product_form_algebra_matches_the_oracle(orc, k, nc):
    """The FAST kernels compute the reference's reconstruction in a rearranged but equal form;
    restated in exact-division numpy, that form agrees with the oracle to rounding level on
    smooth, discontinuous and rough lines (the kernels' own rounding is checked on the GPU)."""
    for v in lines(nc, 11 * nc + k):
        vl, vr = orc.reconstruct(v, k, 1e-6)
        fl, fr = reconstruct_product_form_np(v, k, 1e-6)
        scale = max(np.max(np.abs(v)), 1e-300)
        assert np.max(np.abs(fl - vl)) <= 1e-13 * scale and np.max(np.abs(fr - vr)) <= 1e-13 * scale


def offsets_np(v, k, eps):
    """(rl, rr) = (vl - v, vr - v) of every cell from the neighbour differences d_m = v_{m+1} - v_m,
    as the compensated FP32 kernels form them (candidates and indicators as linear and quadratic
    forms in the differences, product-form weights), here in float64 with true divisions."""
    nc = v.size
    if k == 1:
        return np.zeros(nc), np.zeros(nc)
    ext = np.concatenate([np.full(2, v[0]), v, np.full(2, v[-1])])
    dd = np.diff(ext)  # dd[q] = d_{q-2}
    at = lambda o: dd[2 + o: 2 + o + nc]  # noqa: E731  d_{j+o}, j = 0 .. nc-1
    dmm, dm, d0, d1 = at(-2), at(-1), at(0), at(1)
    if k == 2:
        s0, s1 = (eps + d0 ** 2) ** 2, (eps + dm ** 2) ** 2
        return (-0.5 * (s1 * d0 + 2 * s0 * dm) / (s1 + 2 * s0),
                0.5 * (2 * s1 * d0 + s0 * dm) / (2 * s1 + s0))
    e0 = eps + 13 / 12 * (d1 - d0) ** 2 + 0.25 * (d1 - 3 * d0) ** 2
    e1 = eps + 13 / 12 * (d0 - dm) ** 2 + 0.25 * (dm + d0) ** 2
    e2 = eps + 13 / 12 * (dm - dmm) ** 2 + 0.25 * (3 * dm - dmm) ** 2
    s0, s1, s2 = e0 ** 2, e1 ** 2, e2 ** 2
    P0, P1, P2 = s1 * s2, s0 * s2, s0 * s1
    R0, R1, R2 = 4 * d0 - d1, 2 * d0 + dm, 5 * dm - 2 * dmm
    L0, L1, L2 = 2 * d1 - 5 * d0, -(2 * dm + d0), dmm - 4 * dm
    rr = (3 * P0 * R0 + 6 * P1 * R1 + P2 * R2) / (6 * (3 * P0 + 6 * P1 + P2))
    rl = (P0 * L0 + 6 * P1 * L1 + 3 * P2 * L2) / (6 * (P0 + 6 * P1 + 3 * P2))
    return rl, rr


def rhs_difference_form_np(v, k, eps, flux, fn, a, b, alpha, bc, xmin, xmax):
    """example1's right-hand side in the compensated kernels' difference form: per cell j,
    F_{j+1/2} - F_{j-1/2} = G_R - G_L (+ (g_R - g_L) v_j for f = g(x) u), G = F - f_base(v_j)
    evaluated from the offsets, so the O(1) part cancels exactly; boundary cells in full."""
    nc = v.size
    rx = (xmax - xmin) / nc
    rl, rr = offsets_np(v, k, eps)
    d = np.append(np.diff(v), 0.0)  # d_j = v_{j+1} - v_j (0 past the end: ghosts replicate)
    lin = fn == "linear"
    g = (a + b * (xmin + rx * np.arange(nc + 1))) if lin else np.zeros(nc + 1)

    def G(vj, am, bp, gg):  # F(vj + am, vj + bp) - f_base(vj)
        if flux == "lax_friedrichs":
            if lin:
                return 0.5 * ((gg + alpha) * am + (gg - alpha) * bp)
            return 0.25 * (am * (2 * vj + am + 2 * alpha) + bp * (2 * vj + bp - 2 * alpha))
        fa, fb = (gg * am, gg * bp) if lin else (0.5 * am * (2 * vj + am), 0.5 * bp * (2 * vj + bp))
        return np.where(am <= bp, np.minimum(fa, fb), np.maximum(fa, fb))

    rr_m = np.concatenate([[rr[0]], rr[:-1]])
    d_m = np.concatenate([[0.0], d[:-1]])
    rl_p = np.append(rl[1:], rl[-1])
    GL = G(v, rr_m - d_m, rl, g[:-1])
    GR = G(v, rr, d + rl_p, g[1:])
    dF = GR - GL + ((g[1:] - g[:-1]) * v if lin else 0.0)
    for j in {0, nc - 1}:  # boundary cells, fluxes in full
        fb = (lambda e, vv: g[e] * vv) if lin else (lambda e, vv: 0.5 * vv * vv)  # noqa: E731
        FL, FR = fb(j, v[j]) + GL[j], fb(j + 1, v[j]) + GR[j]
        if bc == "copy":
            dF[j] = 0.0
            continue
        if j == 0:
            FL = 0.0
        if j == nc - 1:
            FR = 0.0 if bc == "zero" else fb(nc, v[j] + rr[j])
        dF[j] = FR - FL
    return -dF / rx


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("fn", ["burgers", "linear"])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
def test_difference_form_matches_the_oracle(hw, orc, k, fn, flux, bc):
    """The compensated FP32 kernels' difference form of the right-hand side (offsets from the
    neighbour differences, G-form flux differences, boundary cells in full) is the reference's
    right-hand side rearranged: restated in float64 it agrees with the oracle to rounding level
    (the kernels' FP32 rounding is checked against FP64 on the GPU)."""
    a, b, alpha = (0.6, 0.3, 1.6) if fn == "linear" else (0.0, 0.0, 1.3)
    for nc in (2, 3, 9, 400):
        for v in lines(nc, 5 * nc + k):
            prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, eps=1e-6, flux=flux, fn=(fn, fn),
                              coef_a=(a, 0.0), coef_b=(b, 0.0), alpha=(alpha, alpha), bc=(bc, bc),
                              xmin=(-1.0, 0.0), xmax=(2.0, 1.0), numerics="strict")
            ref = orc.rhs(prob, v)
            got = rhs_difference_form_np(v, k, 1e-6, flux, fn, a, b, alpha, bc, -1.0, 2.0)
            scale = (1.0 + np.max(np.abs(v))) ** 2 * nc / 3.0
            assert np.max(np.abs(got - ref)) <= 1e-13 * scale, (nc, k, fn, flux, bc)


def offsets_nu_np(v, k, eps, cnu):
    """(rl, rr) of every cell of a non-uniform line as the compensated kernels form them
    (recon_diff_nu): a candidate minus v_j is sum_q c(q, r) (v_{j-r+q} - v_j) with the cell's
    own coefficients cnu [nc, k+1, k] (cnu(q, r) at [j, r+1, q]); indicators and weights as on
    a uniform line (float64, true divisions)."""
    nc = v.size
    if k == 1:
        return np.zeros(nc), np.zeros(nc)
    ext = np.concatenate([np.full(k - 1, v[0]), v, np.full(k - 1, v[-1])])
    S = lambda m: ext[k - 1 + m: k - 1 + m + nc] - v  # noqa: E731  v_{j+m} - v_j
    R, Lc = [], []
    for r in range(k):
        R.append(sum(cnu[:, r + 1, q] * S(q - r) for q in range(k) if q != r))
        Lc.append(sum(cnu[:, r, q] * S(q - r) for q in range(k) if q != r))
    d = lambda o: S(o + 1) - S(o)  # noqa: E731  d_{j+o} = v_{j+o+1} - v_{j+o}
    if k == 2:
        s0, s1 = (eps + d(0) ** 2) ** 2, (eps + d(-1) ** 2) ** 2
        return ((s1 * Lc[0] + 2 * s0 * Lc[1]) / (s1 + 2 * s0),
                (2 * s1 * R[0] + s0 * R[1]) / (2 * s1 + s0))
    dmm, dm, d0, d1 = d(-2), d(-1), d(0), d(1)
    e0 = eps + 13 / 12 * (d1 - d0) ** 2 + 0.25 * (d1 - 3 * d0) ** 2
    e1 = eps + 13 / 12 * (d0 - dm) ** 2 + 0.25 * (dm + d0) ** 2
    e2 = eps + 13 / 12 * (dm - dmm) ** 2 + 0.25 * (3 * dm - dmm) ** 2
    s0, s1, s2 = e0 ** 2, e1 ** 2, e2 ** 2
    P0, P1, P2 = s1 * s2, s0 * s2, s0 * s1
    return ((P0 * Lc[0] + 6 * P1 * Lc[1] + 3 * P2 * Lc[2]) / (P0 + 6 * P1 + 3 * P2),
            (3 * P0 * R[0] + 6 * P1 * R[1] + P2 * R[2]) / (3 * P0 + 6 * P1 + P2))


def random_edges(nc, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([[-1.0], -1.0 + np.cumsum(rng.uniform(0.5, 1.5, nc)) * (3.0 / nc)])


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 5, 64, 1001])
def test_nonuniform_offsets_match_the_oracle(orc, k, nc):
    """The compensated kernels' non-uniform reconstruction (offsets from per-cell coefficients
    and neighbour differences) is the reference's weno(ncells, k, eps, xedges) rearranged:
    v + offsets agree with the oracle's vl, vr to rounding level."""
    xe = random_edges(nc, nc + k)
    cnu = orc.calc_cnu(nc, k, xe)
    for v in lines(nc, 3 * nc + k):
        vl, vr = orc.reconstruct(v, k, 1e-6, xedges=xe)
        rl, rr = offsets_nu_np(v, k, 1e-6, cnu)
        scale = max(np.max(np.abs(v)), 1e-300)
        assert np.max(np.abs(v + rl - vl)) <= 1e-13 * scale and np.max(np.abs(v + rr - vr)) <= 1e-13 * scale


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("fn", ["burgers", "linear"])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
def test_nonuniform_difference_form_matches_the_oracle(hw, orc, k, fn, flux, bc):
    """The compensated kernels' difference form on a non-uniform line: g at the true edges, the
    linear flux's (g_R - g_L) v as b width_j v, each cell divided by its own width; restated in
    float64 it agrees with the oracle's right-hand side to rounding level."""
    a, b, alpha = (0.6, 0.3, 1.6) if fn == "linear" else (0.0, 0.0, 1.3)
    for nc in (2, 3, 9, 400):
        xe = random_edges(nc, 7 * nc + k)
        w = np.diff(xe)
        cnu = orc.calc_cnu(nc, k, xe)
        for v in lines(nc, 5 * nc + k):
            prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, eps=1e-6, flux=flux, fn=(fn, fn),
                              coef_a=(a, 0.0), coef_b=(b, 0.0), alpha=(alpha, alpha), bc=(bc, bc),
                              xedges=(xe, None), numerics="strict")
            ref = orc.rhs(prob, v)
            rl, rr = offsets_nu_np(v, k, 1e-6, cnu)
            d = np.append(np.diff(v), 0.0)
            lin = fn == "linear"
            g = (a + b * xe) if lin else np.zeros(nc + 1)

            def G(vj, am, bp, gg):  # F(vj + am, vj + bp) - f_base(vj), as rhs_difference_form_np
                if flux == "lax_friedrichs":
                    if lin:
                        return 0.5 * ((gg + alpha) * am + (gg - alpha) * bp)
                    return 0.25 * (am * (2 * vj + am + 2 * alpha) + bp * (2 * vj + bp - 2 * alpha))
                fa, fb = (gg * am, gg * bp) if lin else (0.5 * am * (2 * vj + am), 0.5 * bp * (2 * vj + bp))
                return np.where(am <= bp, np.minimum(fa, fb), np.maximum(fa, fb))

            rr_m = np.concatenate([[rr[0]], rr[:-1]])
            d_m = np.concatenate([[0.0], d[:-1]])
            rl_p = np.append(rl[1:], rl[-1])
            GL, GR = G(v, rr_m - d_m, rl, g[:-1]), G(v, rr, d + rl_p, g[1:])
            dF = GR - GL + (b * w * v if lin else 0.0)
            for j in {0, nc - 1}:
                fb = (lambda e, vv: g[e] * vv) if lin else (lambda e, vv: 0.5 * vv * vv)  # noqa: E731
                FL, FR = fb(j, v[j]) + GL[j], fb(j + 1, v[j]) + GR[j]
                if bc == "copy":
                    dF[j] = 0.0
                    continue
                if j == 0:
                    FL = 0.0
                if j == nc - 1:
                    FR = 0.0 if bc == "zero" else fb(nc, v[j] + rr[j])
                dF[j] = FR - FL
            got = -dF / w
            scale = (1.0 + np.max(np.abs(v))) ** 2 / np.min(w)
            assert np.max(np.abs(got - ref)) <= 1e-13 * scale, (nc, k, fn, flux, bc)


def _beta_forms(k):
    """Smoothness indicators as sums of weighted squares of linear forms in v(i-2 .. i+2):
    beta_r = sum (c, coefficients) over its terms (src/hrweno_weno.f90:189-202)."""
    if k == 1:
        return [[]]
    if k == 2:
        return [[(1.0, {1: 1.0, 0: -1.0})], [(1.0, {0: 1.0, -1: -1.0})]]
    return [[(13 / 12, {0: 1.0, 1: -2.0, 2: 1.0}), (1 / 4, {0: 3.0, 1: -4.0, 2: 1.0})],
            [(13 / 12, {-1: 1.0, 0: -2.0, 1: 1.0}), (1 / 4, {-1: 1.0, 1: -1.0})],
            [(13 / 12, {-2: 1.0, -1: -2.0, 0: 1.0}), (1 / 4, {-2: 1.0, -1: -4.0, 0: 3.0})]]


def weno_vjp_np(v, k, eps, ar, al):
    """d(sum ar vr + al vl)/dv through the WENO map, by the identities the adjoint kernels use:
    the candidates are linear, d vr/d beta_s = -2 w_s (q_s - vr)/(eps + beta_s) (and likewise for
    vl with the mirrored weights), the indicators are quadratic forms; ghost cells replicate the
    end values, so their sensitivities land on v(1) and v(nc)."""
    nc = v.size
    ext = np.concatenate([np.full(k - 1, v[0]), v, np.full(k - 1, v[-1])])
    at = lambda o: ext[k - 1 + o: k - 1 + o + nc]  # noqa: E731
    q = [sum(C[k][j, r + 1] * at(j - r) for j in range(k)) for r in range(k)]
    p = [sum(C[k][j, r] * at(j - r) for j in range(k)) for r in range(k)]
    forms = _beta_forms(k)
    beta = [sum(c * sum(w * at(o) for o, w in lin.items()) ** 2 for c, lin in forms[r]) if forms[r]
            else np.zeros(nc) for r in range(k)]
    alfa = [D[k][r] / (eps + beta[r]) ** 2 for r in range(k)]
    alft = [D[k][k - 1 - r] / (eps + beta[r]) ** 2 for r in range(k)]
    w = [a / sum(alfa) for a in alfa]
    wt = [a / sum(alft) for a in alft]
    vr = sum(w[r] * q[r] for r in range(k))
    vl = sum(wt[r] * p[r] for r in range(k))
    gext = np.zeros(nc + 2 * (k - 1))

    def push(o, coef):  # add coef (per cell) at offset o of every cell
        gext[k - 1 + o: k - 1 + o + nc] += coef

    for r in range(k):
        for j in range(k):
            push(j - r, ar * w[r] * C[k][j, r + 1] + al * wt[r] * C[k][j, r])
        g_beta = (ar * -2 * w[r] * (q[r] - vr) + al * -2 * wt[r] * (p[r] - vl)) / (eps + beta[r])
        for c, lin in forms[r]:
            val = sum(wt_ * at(o) for o, wt_ in lin.items())
            for o, wt_ in lin.items():
                push(o, g_beta * 2 * c * val * wt_)
    grad = gext[k - 1: k - 1 + nc].copy()
    grad[0] += gext[:k - 1].sum()
    grad[-1] += gext[k - 1 + nc:].sum()
    return grad


def lf_burgers_rhs_vjp_np(v, k, eps, alpha, bc, dx, mu):
    """J(v)^T mu of example1's right-hand side with the fixed-alpha Lax-Friedrichs flux: flux
    adjoints phi_e = (mu_e - mu_{e-1})/dx with the boundary rules transposed, then the states'
    adjoints ar, al and the reverse WENO map."""
    nc = v.size
    vl, vr = reconstruct_np(v, k, eps)
    m = np.concatenate([[0.0], mu, [0.0]])
    phi = (m[1:] - m[:-1]) / dx  # phi[e], e = 0 .. nc: faces
    if bc == "copy" and nc >= 2:
        phi[1] += phi[0]
        phi[nc - 1] += phi[nc]
    ar, al = np.zeros(nc), np.zeros(nc)
    ar[:-1] += phi[1:nc] * (vr[:-1] + alpha) / 2  # dF/dvm, f' = u
    al[1:] += phi[1:nc] * (vl[1:] - alpha) / 2    # dF/dvp
    if bc == "zero_inflow":
        ar[-1] += phi[nc] * vr[-1]                # F_nc = f(vr(nc))
    return weno_vjp_np(v, k, eps, ar, al)


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
def test_rk3_step_adjoint_identities(hw, k, bc):
    """The transposed RK3 step of the adjoint kernels (A3: l2 = 2/3 (l' + dt J(u2)^T l'), A2:
    l1 = 1/4 (l2 + dt J(u1)^T l2), A1: l = acc + l1 + dt J(u)^T l1 with acc = l'/3 + 3/4 l2) with
    the flux and WENO transposes above: <l, d> equals <l', J_step d> computed by complex-step
    differentiation of the numpy forward step, to rounding level."""
    nc, eps, alpha = 40, 1e-6, 1.5
    dx = 10.0 / nc
    dt = 0.4 * dx / alpha
    x = -5.0 + dx * (np.arange(nc) + 0.5)
    u = 0.3 + np.exp(-x ** 2) + 0.05 * np.sin(3 * x)
    rng = np.random.default_rng(k)
    d, lam = rng.standard_normal(nc), rng.standard_normal(nc)

    def L(v):
        vl, vr = reconstruct_np(v, k, eps)
        f = lambda z: z * z / 2  # noqa: E731
        F = np.zeros(nc + 1, dtype=np.result_type(v, float))
        F[1:nc] = (f(vr[:-1]) + f(vl[1:]) - alpha * (vl[1:] - vr[:-1])) / 2
        if bc == "copy":
            F[0], F[nc] = F[1], F[nc - 1]
        elif bc == "zero_inflow":
            F[nc] = f(vr[-1])
        return -(F[1:] - F[:-1]) / dx

    h = 1e-30
    jd = np.imag(rk3_step(u + 1j * h * d, dt, L)) / h  # J_step d, exact to rounding
    u1 = u + dt * L(u)
    u2 = (3 * u + u1 + dt * L(u1)) / 4
    JT = lambda v, mu: lf_burgers_rhs_vjp_np(v, k, eps, alpha, bc, dx, mu)  # noqa: E731
    l2 = 2 / 3 * (lam + dt * JT(u2, lam))
    acc = lam / 3 + 3 / 4 * l2
    l1 = 1 / 4 * (l2 + dt * JT(u1, l2))
    lu = acc + l1 + dt * JT(u, l1)
    assert abs(lu @ d - lam @ jd) <= 1e-12 * abs(lam @ jd)


def test_increment_form_stages_match_the_reference_formulas():
    """The compensated kernels store stage values as increments relative to u and add the last
    one to (hi, lo): E1 d1 = dt L(u); RK3B d2 = (d1 + dt L(u + d1))/4; RK3C u' = u + 2/3 (d2 +
    dt L(u + d2)); RK2B u' = u + (d1 + dt L(u + d1))/2; multistep u' = u + (7 (u4 - u) +
    50 dt L(u) + 10 dt L4)/32.  These equal the reference's formulas
    (src/hrweno_tvdode.f90:139-167,257) to rounding level."""
    nc, dt = 300, 4e-3
    L = lambda u: rhs_burgers_np(u, -5.0, 5.0, 3, 1e-6, "lax_friedrichs", 1.0, "copy")  # noqa: E731
    rng = np.random.default_rng(2)
    x = -5.0 + 10.0 / nc * (np.arange(nc) + 0.5)
    u = np.exp(-x * x) + 0.1 * rng.standard_normal(nc)
    u4 = u + 0.01 * rng.standard_normal(nc)
    L4 = L(u4)
    tol = lambda ref: 1e-14 * np.max(np.abs(ref))  # noqa: E731
    d1 = dt * L(u)
    d2 = (d1 + dt * L(u + d1)) / 4
    ref = rk3_step(u, dt, L)
    assert np.max(np.abs(u + 2 / 3 * (d2 + dt * L(u + d2)) - ref)) <= tol(ref)
    ui = u + dt * L(u)
    ref2 = (u + ui + dt * L(ui)) / 2
    assert np.max(np.abs(u + (d1 + dt * L(u + d1)) / 2 - ref2)) <= tol(ref2)
    refm = (25 * u + 50 * dt * L(u) + 7 * u4 + 10 * dt * L4) / 32
    assert np.max(np.abs(u + (7 * (u4 - u) + 50 * dt * L(u) + 10 * dt * L4) / 32 - refm)) <= tol(refm)
