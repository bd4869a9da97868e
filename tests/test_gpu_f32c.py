"""The compensated FP32 form (HRW_F32C) against the FP64 oracle.

The FP32 form is a different precision of the same method, so it is judged by its error
against FP64, not by parity:
  one right-hand side   max|L32 - L64| <= 2e-6 max|L64|
  integrations          relative L1 error sum|u32 - u64| / sum|u64| <= 1e-6 (the stated
                        bound of the FP32 form); the Linf error is reported by bench.py.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


def rhs_f32c(prob, v):
    import torch
    from hrweno import _abi as A
    tv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    out = torch.empty_like(tv)
    cp = prob.to_c()
    A.check(A.lib().hrw_rhs(C.byref(cp), A.HRW_F32C, 0.0, tv.data_ptr(), out.data_ptr(), None))
    return out.cpu().numpy()


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("nc", [1, 2, 7, 1000, 1 << 16, 1 << 20])
@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
@pytest.mark.parametrize("bc", ["copy", "zero", "zero_inflow"])
def test_rhs_f32c_burgers(hw, orc, k, nc, flux, bc):
    from hrweno import workloads
    u = workloads.multi_gaussian_1d(nc, seed=nc + k) if nc > 8 else np.linspace(0.2, 0.9, nc)
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=k, flux=flux, bc=bc, alpha=float(np.max(np.abs(u))))
    ref = orc.rhs(prob, u)
    got = rhs_f32c(prob, u)
    scale = max(np.max(np.abs(ref)), 1e-30)
    assert np.max(np.abs(got - ref)) <= 2e-6 * scale, np.max(np.abs(got - ref)) / scale


@pytest.mark.parametrize("flux", ["lax_friedrichs", "godunov"])
def test_rhs_f32c_linear_and_widths(hw, orc, flux):
    nc = 5000
    rng = np.random.default_rng(4)
    width = rng.uniform(0.8, 1.2, nc) * (2.0 / nc)
    x = np.linspace(-1, 1, nc)
    v = np.exp(-30 * x ** 2) + 0.2
    for w in (None, width):
        prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux=flux, fn=("linear", "linear"),
                          coef_a=(0.6, 0), coef_b=(0.3, 0), alpha=(0.9, 0),
                          bc=("zero_inflow", "copy"), xmin=(-1.0, 0), xmax=(1.0, 1), width=(w, None))
        ref = orc.rhs(prob, v)
        got = rhs_f32c(prob, v)
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))


def stretched(nc, kind, seed=0):
    """Edges on [-1, 1]: cubic (i / nc)^3 stretching (test/test_hrweno.f90:123-128) or random
    widths in a 1:3 range."""
    if kind == "cubic":
        return -1.0 + 2.0 * (np.arange(nc + 1) / nc) ** 3
    rng = np.random.default_rng(seed)
    return np.concatenate([[-1.0], -1.0 + np.cumsum(rng.uniform(0.5, 1.5, nc)) * (2.0 / nc)])


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("kind,nc", [(kd, n) for kd in ("cubic", "random") for n in (1, 2, 7, 300, 1000)]
                         + [("random", 1 << 16)])
def test_rhs_f32c_nonuniform(hw, orc, k, nc, kind):
    """weno(ncells, k, eps, xedges) in the compensated form: per-cell coefficients rounded from
    the FP64 ones, FP64 widths, g at the edges; against the FP64 oracle's stage.

    The float pair holds the state to about 2^-48 of its size, so a cell's right-hand side is
    resolved while its width is well above 2^-48 max|v| / 2e-6 (about 1e-9 here): the cubic
    line stops at 1000 cells (smallest cell 2e-9); at 2^16 cells its first cells are 7e-15
    wide, where the float pair (and even FP64, to about 1%) no longer resolves the
    differences of v."""
    xe = stretched(nc, kind, nc)
    xc = 0.5 * (xe[1:] + xe[:-1])
    v = 1.0 + 0.5 * np.sin(3.0 * xc) + 0.3 * np.exp(-40.0 * xc ** 2)
    cases = [dict(flux="lax_friedrichs", fn="burgers", bc="copy", b=0.0),
             dict(flux="godunov", fn="burgers", bc="zero", b=0.0),
             dict(flux="godunov", fn="linear", bc="zero_inflow", b=0.4),
             dict(flux="lax_friedrichs", fn="linear", bc="copy", b=-0.3)]
    for c in cases:
        prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, flux=c["flux"], fn=(c["fn"], c["fn"]),
                          coef_a=(0.8, 0), coef_b=(c["b"], 0), alpha=(2.5, 2.5),
                          bc=(c["bc"], c["bc"]), xedges=(xe, None))
        ref = orc.rhs(prob, v)
        got = rhs_f32c(prob, v)
        scale = max(np.max(np.abs(ref)), 1e-30)
        assert np.max(np.abs(got - ref)) <= 2e-6 * scale, (c, np.max(np.abs(got - ref)) / scale)


@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (33, 31), (64, 40), (100, 37)])
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("which", ["x1", "x2", "both"])
@pytest.mark.parametrize("name", ["pbe_upwind", "pbe_mixed", "pbe_lf"])
def test_rhs_f32c_2d_nonuniform(hw, orc, shape, k, which, name):
    """Non-uniform lines in 2D in the compensated form: the cells of a line with edges
    reconstruct with their own coefficients, divide by their widths and see g at the true
    edges; a uniform line of the same grid keeps the tables (the FP64 cases of
    test_gpu_2d.py against the FP64 oracle, within the compensated form's bound)."""
    import test_gpu_2d as T2
    n1, n2 = shape
    v = np.random.default_rng(n1 * 7 + n2 + k).uniform(0.0, 1.0, n1 * n2)
    prob = T2.nonuniform_pbe(hw, n1, n2, k, name, which, "fast")
    ref = orc.rhs(prob, v)
    got = rhs_f32c(prob, v)
    assert np.max(np.abs(got - ref)) <= 2e-6 * max(np.max(np.abs(ref)), 1e-30), \
        np.max(np.abs(got - ref)) / np.max(np.abs(ref))


@pytest.mark.parametrize("method", ["rktvd", "mstvd"])
def test_f32c_2d_nonuniform_integrate(hw, orc, method):
    import test_gpu_2d as T2
    from hrweno import workloads
    n1, n2 = 96, 80
    _, n0, dt = workloads.pbe_config(n1, n2, cfl=0.25)
    prob = T2.nonuniform_pbe(hw, n1, n2, 3, "pbe_upwind", "both", "fast")
    if method == "rktvd":
        g, o = hw.rktvd(prob, n1 * n2, 3, dtype="f32c"), orc.ODE(prob, n1 * n2, 0, 3)
    else:
        g, o = hw.mstvd(prob, n1 * n2, dtype="f32c"), orc.ODE(prob, n1 * n2, 1)
    u32, u64 = n0.copy(), n0.copy()
    t32 = g.integrate(u32, 0.0, 61.5 * dt, dt)
    t64 = o.integrate(u64, 0.0, 61.5 * dt, dt)
    assert t32 == t64 and g.nsteps == o.info()[2]
    assert rel_l1(u32, u64) <= 1e-6, rel_l1(u32, u64)


def jumpy(n, seed, amp=(3e3, 3e4)):
    """A state of plateaus with jumps of |amp[0]| .. |amp[1]|: the WENO indicators' squares
    then span 1e13 .. 1e20, across the bound between the weights' product and division forms."""
    rng = np.random.default_rng(seed)
    u = np.zeros(n)
    for p in np.sort(rng.choice(np.arange(5, n - 5), size=max(n // 50, 2), replace=False)):
        u[p:] += rng.choice([-1.0, 1.0]) * np.exp(rng.uniform(np.log(amp[0]), np.log(amp[1])))
    return u - u.min() + 1.0 + 50.0 * np.sin(np.linspace(0.0, 6.0, n))


@pytest.mark.parametrize("k", [2, 3])
def test_rhs_f32c_large_jumps(hw, orc, k):
    """Differences of 1e3 .. 3e4 between neighbours: the weights' product form stays finite
    (the fast branch is taken only while the indicators' squares are below 1e16), so the
    compensated right-hand side matches FP64 as on O(1) data.  Uniform and non-uniform lines
    and a 2D grid."""
    n = 1000
    u = jumpy(n, k)
    amax = float(np.max(np.abs(u)))
    xe = stretched(n, "random", 3)
    cases = [hw.burgers_1d(n, -5.0, 5.0, k=k, flux="lax_friedrichs", alpha=amax),
             hw.burgers_1d(n, -5.0, 5.0, k=k, flux="godunov", bc="zero"),
             hw.Problem(kind="fv1d", ncells=(n, 1), k=k, flux="lax_friedrichs", fn=("burgers", "burgers"),
                        alpha=(amax, amax), xedges=(xe, None))]
    for prob in cases:
        ref = orc.rhs(prob, u)
        got = rhs_f32c(prob, u)
        assert np.isfinite(got).all()
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref)), np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    from hrweno import workloads
    n1 = n2 = 96
    prob, _, _ = workloads.pbe_config(n1, n2)
    v = np.stack([jumpy(n1, 10 + r) for r in range(n2)]).ravel()
    v += np.repeat(jumpy(n2, 99), n1)
    ref = orc.rhs(prob, v)
    got = rhs_f32c(prob, v)
    assert np.isfinite(got).all()
    assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))


@pytest.mark.parametrize("method", ["rktvd", "mstvd"])
@pytest.mark.parametrize("kind", ["cubic", "random"])
def test_f32c_nonuniform_integrate(hw, orc, method, kind):
    nc = 2000
    xe = stretched(nc, kind, 5)
    xc = 0.5 * (xe[1:] + xe[:-1])
    u0 = 0.5 + np.exp(-30 * xc ** 2)
    prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux="godunov", fn=("burgers", "burgers"),
                      alpha=(1.5, 1.5), bc=("copy", "copy"), xedges=(xe, None))
    dt = 0.2 * np.min(np.diff(xe)) / 1.5
    steps = 300 if kind == "random" else 40  # the cubic line's smallest cell is 2 / nc^3 wide
    if method == "rktvd":
        g, o = hw.rktvd(prob, nc, 3, dtype="f32c"), orc.ODE(prob, nc, 0, 3)
    else:
        g, o = hw.mstvd(prob, nc, dtype="f32c"), orc.ODE(prob, nc, 1)
    u32, u64 = u0.copy(), u0.copy()
    t32 = g.integrate(u32, 0.0, (steps - 0.5) * dt, dt)
    t64 = o.integrate(u64, 0.0, (steps - 0.5) * dt, dt)
    assert t32 == t64 and g.nsteps == o.info()[2]
    assert rel_l1(u32, u64) <= 1e-6, rel_l1(u32, u64)


@pytest.mark.parametrize("k", [2, 3])
def test_f32c_large_burgers_vs_oracle(hw, orc, k):
    """2^16 cells, 8-Gaussian u0, LF, RK3 at CFL 0.4 for 1000 steps."""
    from hrweno import workloads
    n = 1 << 16
    prob, u0, dt = workloads.large_burgers(n, k=k)
    u32 = u0.copy()
    t32 = hw.rktvd(prob, n, 3, dtype="f32c").integrate(u32, 0.0, 999.5 * dt, dt)
    u64 = u0.copy()
    t64 = orc.ODE(prob, n, 0, 3).integrate(u64, 0.0, 999.5 * dt, dt)
    assert t32 == t64
    assert rel_l1(u32, u64) <= 1e-6, rel_l1(u32, u64)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_f32c_orders(hw, orc, order):
    from hrweno import workloads
    n = 4096
    prob, u0, dt = workloads.large_burgers(n, k=3)
    steps = 20 if order == 1 else 300
    u32, u64 = u0.copy(), u0.copy()
    g = hw.rktvd(prob, n, order, dtype="f32c")
    t32 = g.integrate(u32, 0.0, (steps - 0.5) * dt, dt)
    t64 = orc.ODE(prob, n, 0, order).integrate(u64, 0.0, (steps - 0.5) * dt, dt)
    assert t32 == t64 and g.nsteps == steps and g.fevals == order * steps
    assert rel_l1(u32, u64) <= 1e-6


def test_f32c_mstvd(hw, orc):
    nc = 2048
    x = np.linspace(0, 1, nc)
    u0 = np.exp(-((x - 0.3) / 0.05) ** 2)
    prob = hw.Problem(kind="fv1d", ncells=(nc, 1), k=3, flux="godunov", fn=("linear", "linear"),
                      coef_a=(1.0, 0), coef_b=(0.5, 0), alpha=(1.5, 0), bc=("zero_inflow", "copy"),
                      xmin=(0.0, 0), xmax=(1.0, 1))
    dt = 0.16 / nc  # CFL 0.24; at 0.375 the multistep method is past its stability limit
    g, o = hw.mstvd(prob, nc, dtype="f32c"), orc.ODE(prob, nc, 1)
    u32, u64 = u0.copy(), u0.copy()
    t32 = t64 = 0.0
    for tout in (0.0, 0.05, 0.2):
        t32 = g.integrate(u32, t32, tout, dt)
        t64 = o.integrate(u64, t64, tout, dt)
        assert t32 == t64 and g.nsteps == o.info()[2] and g.fevals == o.info()[0]
    assert rel_l1(u32, u64) <= 1e-6


def test_f32c_full_size_vs_fp64_gpu(hw):
    """2^24 cells, 1000 RK3 steps: compensated FP32 against the FP64 GPU path (itself within
    1e-12 of the oracle), relative L1 <= 1e-6."""
    import torch
    from hrweno import workloads
    n = 1 << 24
    prob, u0, dt = workloads.large_burgers(n, k=3)
    a = torch.from_numpy(u0.copy()).cuda()
    b = torch.from_numpy(u0.copy()).cuda()
    hw.rktvd(prob, n, 3).integrate(a, 0.0, 999.5 * dt, dt)
    hw.rktvd(prob, n, 3, dtype="f32c").integrate(b, 0.0, 999.5 * dt, dt)
    l1 = float((a - b).abs().sum() / a.abs().sum())
    assert l1 <= 1e-6, l1
    # the same integration conserves sum(u) to the FP32 increment rounding: copy boundaries
    # with zero flux difference at both boundary cells


# rows of a multiple of 4 floats take the TMA tile loader, the others the gathering loader
@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (31, 33), (64, 40), (100, 37), (4, 9), (36, 70),
                                   (128, 3)])
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("bc", ["zero_inflow", "zero", "copy"])
def test_rhs_f32c_2d(hw, orc, shape, k, bc):
    n1, n2 = shape
    rng = np.random.default_rng(n1 + 7 * n2 + k)
    from hrweno import workloads
    v = workloads.pbe_gaussian_2d(n1, n2, sigma=0.2, centre=(0.4, 0.5)) + 0.01 * rng.random(n1 * n2)
    for flux in ("godunov", "lax_friedrichs"):
        prob = hw.pbe_2d(n1, n2, k=k, flux=flux, bc=bc)
        ref = orc.rhs(prob, v)
        got = rhs_f32c(prob, v)
        scale = max(np.max(np.abs(ref)), 1e-30)
        assert np.max(np.abs(got - ref)) <= 2e-6 * scale, (shape, k, bc, flux)


@pytest.mark.parametrize("shape", [(96, 80), (90, 70)])
def test_f32c_mstvd_2d_vs_oracle(hw, orc, shape):
    from hrweno import workloads
    n1, n2 = shape
    prob, n0, dt = workloads.pbe_config(n1, n2)
    g, o = hw.mstvd(prob, n1 * n2, dtype="f32c"), orc.ODE(prob, n1 * n2, 1)
    u32, u64 = n0.copy(), n0.copy()
    t32 = t64 = 0.0
    for tout in (0.0, 20 * dt, 61.5 * dt):
        t32 = g.integrate(u32, t32, tout, dt)
        t64 = o.integrate(u64, t64, tout, dt)
        assert t32 == t64 and g.nsteps == o.info()[2]
    assert rel_l1(u32, u64) <= 1e-6, rel_l1(u32, u64)


def test_f32c_pbe1024_vs_fp64_gpu(hw):
    """1024^2 PBE, mstvd, 500 steps: compensated FP32 against the FP64 GPU path.  CFL 0.3:
    at 0.4 the multistep method is unstable on this problem and rounding differences of any
    two implementations (FP64 and binary128 oracles included) grow without bound."""
    import torch
    from hrweno import workloads
    n = 1024
    prob, n0, dt = workloads.pbe_config(n, n, cfl=0.3)
    a = torch.from_numpy(n0.copy()).cuda()
    b = torch.from_numpy(n0.copy()).cuda()
    hw.mstvd(prob, n * n).integrate(a, 0.0, 499.5 * dt, dt)
    hw.mstvd(prob, n * n, dtype="f32c").integrate(b, 0.0, 499.5 * dt, dt)
    l1 = float((a - b).abs().sum() / a.abs().sum())
    assert l1 <= 1e-6, l1


# ---- the 2D upwind specialisation gives the general path's bits --------------------------------
@pytest.mark.parametrize("n1,n2", [(64, 48), (128, 96), (100, 37)])
@pytest.mark.parametrize("bc", ["zero_inflow", "zero", "copy"])
def test_pbe_2d_upwind_same_bits(hw, n1, n2, bc):
    """Godunov's flux of g(x) u with g > 0 everywhere: the upwind kernels reconstruct only the
    left state of each interface (F = g vm exactly).  Handles created with the specialisation
    off (hrw_diag_upwind(0)) take the general flux path: the compensated FP32 mstvd and
    right-hand side, and the FP64 STRICT rktvd, give the same bits either way (n1 a multiple of
    4: TMA tiles; 100: gathered).  (FP64 FAST's upwind pass takes one reciprocal per cell of its
    own, so it agrees with the general pass to rounding only.)"""
    import torch
    from hrweno import _abi as A, workloads
    L = A.lib()
    L.hrw_diag_upwind.argtypes = [C.c_int]
    prob, n0, dt = workloads.pbe_config(n1, n2, cfl=0.3, bc=bc)
    sprob, _, _ = workloads.pbe_config(n1, n2, cfl=0.3, bc=bc, numerics="strict")
    outs = []
    try:
        for enable in (1, 0):
            assert L.hrw_diag_upwind(enable) == 0
            res = []
            for ode in (hw.mstvd(prob, n1 * n2, dtype="f32c"), hw.rktvd(sprob, n1 * n2, 3)):
                u = torch.from_numpy(n0.copy()).cuda()
                ode.integrate(u, 0.0, 30.5 * dt, dt)
                res.append(u.cpu().numpy())
            res.append(rhs_f32c(prob, n0))
            outs.append(res)
    finally:
        L.hrw_diag_upwind(1)
    for name, a, b in zip(("f32c mstvd", "f64 strict rktvd", "f32c rhs"), *outs):
        assert np.array_equal(a, b), (name, float(np.max(np.abs(a - b))))
