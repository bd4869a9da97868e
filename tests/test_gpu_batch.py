"""Batched solves (hrw_batch_*) against the oracle and against one-problem-at-a-time solves.

Tolerances: STRICT numerics bit-identical to the oracle; FAST numerics bit-identical to the
single-problem FAST path (same per-cell arithmetic whatever the launch shape) and within
1e-12 (normwise relative) of the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def nrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mixed_problems(hw, numerics, sizes=(1, 2, 3, 5, 8, 31, 64, 200, 511, 512, 600, 1000, 4095,
                                          4096, 5000, 9000, 20000)):
    """Every flux, flux function, boundary kind and k across sizes that cross the classes."""
    rng = np.random.default_rng(5)
    probs, lines, dts = [], [], []
    combos = [("lax_friedrichs", "burgers", "copy"), ("godunov", "burgers", "zero"),
              ("lax_friedrichs", "linear", "zero_inflow"), ("godunov", "linear", "copy")]
    for i, n in enumerate(sizes):
        flux, fn, bc = combos[i % 4]
        k = 1 + i % 3
        x = np.linspace(-1, 1, n)
        u = 0.3 + 0.5 * np.exp(-10 * x ** 2) * np.sign(np.sin(7 * x + i)) + 0.01 * rng.standard_normal(n)
        a = float(rng.uniform(-1, 1))
        p = hw.Problem(kind="fv1d", ncells=(n, 1), k=k, flux=flux, fn=(fn, fn),
                       coef_a=(a, 0.0), coef_b=(0.2 if fn == "linear" and i % 3 == 0 else 0.0, 0.0),
                       alpha=(1.5, 1.5), bc=(bc, bc), xmin=(-1.0, 0.0), xmax=(1.0, 1.0),
                       numerics=numerics)
        probs.append(p)
        lines.append(u)
        dts.append(0.3 * (2.0 / n) / 1.5)
    return probs, lines, np.array(dts)


@pytest.mark.parametrize("numerics", ["strict", "fast"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_batch_vs_oracle(hw, orc, numerics, order):
    probs, lines, dts = mixed_problems(hw, numerics)
    b = hw.batch(probs, order=order)
    u = b.pack(lines)
    t = np.zeros(len(probs))
    steps = 8 if order == 1 else 40
    tout = 1e9  # itask=2 semantics below: exactly `steps` steps per problem
    b.integrate(u, t, tout, dts, itask=2)
    b.advance(u, t, dts, steps - 1)
    assert np.all(b.steps_done == steps)
    got = b.unpack(u)
    for i, (p, v) in enumerate(zip(probs, lines)):
        o = orc.ODE(p, p.ncells[0], 0, order)
        uo = v.copy()
        to = 0.0
        for _ in range(steps):
            to = o.integrate(uo, to, tout, dts[i], itask=2)
        assert t[i] == to
        if numerics == "strict":
            assert np.array_equal(got[i], uo), (i, p.ncells[0])
        else:
            assert nrel(got[i], uo) <= 1e-12, (i, p.ncells[0], nrel(got[i], uo))


def test_batch_fast_equals_single_problem_path(hw):
    """The batched FAST kernel and the single-problem FAST kernel give the same bits."""
    import torch
    from hrweno import workloads
    probs, lines, dts = workloads.batched_config(96, seed=3, nmax=20000)
    b = hw.batch(probs, order=3)
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    b.integrate(u, t, 25.5 * dts.max(), dts)  # itask 1: each problem to its own step count
    got = b.unpack(u)
    for i, p in enumerate(probs):
        ug = torch.from_numpy(lines[i].copy()).cuda()
        ts = hw.rktvd(p, p.ncells[0], 3).integrate(ug, 0.0, 25.5 * dts.max(), dts[i])
        assert ts == t[i]
        assert np.array_equal(got[i], ug.cpu().numpy()), i


def test_batch_shapes_agree_and_tuner_caches(hw, tmp_path):
    """Every candidate shape gives the same bits; the tuner's cache is reused."""
    import torch
    from hrweno import workloads
    probs, lines, dts = workloads.batched_config(64, seed=11, nmax=12000)
    u0 = workloads  # noqa: F841
    ref = None
    cache = str(tmp_path / "tune.txt")
    b = hw.batch(probs, order=3)
    packed = b.pack(lines)
    shapes = b.tune(packed, dts, probe_steps=2, cache_path=cache)
    assert len(shapes) == 3
    text = open(cache).read()
    assert text.count("\n") >= 1
    b2 = hw.batch(probs, order=3)
    assert b2.tune(packed, dts, probe_steps=2, cache_path=cache) == shapes
    for bb in (b, b2):
        u = torch.from_numpy(packed.copy()).cuda()
        t = np.zeros(len(probs))
        bb.integrate(u, t, 10.5 * dts.max(), dts)
        if ref is None:
            ref = u.cpu().numpy()
        assert np.array_equal(u.cpu().numpy(), ref)


def test_batch_validation(hw):
    from hrweno import HrwError
    ok = hw.burgers_1d(10)
    with pytest.raises(HrwError, match="non-uniform lines as xedges"):
        hw.batch([ok, hw.burgers_1d(10, width=np.full(10, 0.1))])
    with pytest.raises(HrwError, match="one numerics mode"):
        hw.batch([ok, hw.burgers_1d(10, numerics="strict")])
    with pytest.raises(HrwError, match="FV1D"):
        hw.batch([ok, hw.pbe_2d(4, 4)])


def test_batch_f32c_vs_fp64(hw):
    """Compensated-FP32 batches against FP64 batches: relative L1 <= 1e-6 over the batch and
    <= 1e-5 per problem.  (A coarse line whose profile changes by O(1) per step carries an
    FP32 error of about eps * sqrt(steps) of its values: the compensation helps where the
    increments are small against the state.)"""
    import torch
    from hrweno import workloads
    probs, lines, dts = workloads.batched_config(128, seed=21, nmax=30000)
    res = {}
    for dtype in ("f64", "f32c"):
        b = hw.batch(probs, order=3, dtype=dtype)
        u = torch.from_numpy(b.pack(lines)).cuda()
        t = np.zeros(len(probs))
        b.advance(u, t, dts, 60)
        res[dtype] = b.unpack(u)
        assert np.all(b.steps_done == 60)
    num = den = 0.0
    for a, c in zip(res["f64"], res["f32c"]):
        assert np.sum(np.abs(a - c)) <= 1e-5 * np.sum(np.abs(a))
        num += np.sum(np.abs(a - c))
        den += np.sum(np.abs(a))
    assert num <= 1e-6 * den


@pytest.mark.parametrize("order", [1, 2, 3])
def test_batch_f32c_vs_single_f32c(hw, order):
    """A compensated-FP32 batch and single compensated-FP32 solves agree to the FP32 form's
    own accuracy (the shapes differ, the arithmetic per cell does not)."""
    probs, lines, dts = mixed_problems(hw, "fast", sizes=(8, 64, 300, 600, 5000, 9000))
    b = hw.batch(probs, order=order, dtype="f32c")
    u = b.pack(lines)
    t = np.zeros(len(probs))
    steps = 6 if order == 1 else 30
    b.advance(u, t, dts, steps)
    got = b.unpack(u)
    for i, p in enumerate(probs):
        v = lines[i].copy()
        hw.rktvd(p, p.ncells[0], order, dtype="f32c").integrate(v, 0.0, (steps - 0.5) * dts[i], dts[i])
        assert np.array_equal(got[i], v), i


# ---- mstvd batches ---------------------------------------------------------------------------
@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_mstvd_batch_matches_single_solves(hw, orc, numerics):
    """A batch of mstvd solves (src/hrweno_tvdode.f90:180-271) of uneven lines, over several
    integrate calls: each problem bit-identical to its own single-problem mstvd handle (FAST)
    and to the oracle (STRICT), with the same t and step count; the history carries across
    calls, and a problem whose first call takes no step starts later."""
    import torch
    from hrweno import workloads
    probs, lines, dts = workloads.batched_config(24, seed=3, nmin=40, nmax=3000, numerics=numerics,
                                                 cfl=0.2)
    b = hw.batch(probs, dtype="f64", method="mstvd")
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    t[5] = 1.0  # problem 5 is past the first tout: it takes no step on the first call
    singles = [hw.mstvd(p, int(p.ncells[0])) for p in probs]
    us = [torch.from_numpy(v.copy()).cuda() for v in lines]
    ts = [float(x) for x in t]
    orcs = [orc.ODE(p, int(p.ncells[0]), 1) for p in probs]
    uo = [v.copy() for v in lines]
    to = [float(x) for x in t]
    for tout in (0.05, 0.2, 1.5):
        b.integrate(u, t, tout, dts)
        got = b.unpack(u)
        for i, p in enumerate(probs):
            ts[i] = singles[i].integrate(us[i], ts[i], tout, dts[i])
            assert t[i] == ts[i], i
            assert np.array_equal(got[i], us[i].cpu().numpy()), (i, tout)
            if numerics == "strict":
                to[i] = orcs[i].integrate(uo[i], to[i], tout, dts[i])
                assert to[i] == t[i] and np.array_equal(got[i], uo[i]), (i, tout)
        assert list(b.steps_done) == [s.nsteps for s in singles]


def test_mstvd_batch_advance_and_tune(hw, orc):
    """advance: the start on the first call (4 steps), then exactly nsteps multistep steps; the
    autotuner leaves the histories as they are."""
    import torch
    from hrweno import workloads
    probs, lines, dts = workloads.batched_config(16, seed=4, nmin=64, nmax=5000, numerics="strict",
                                                 cfl=0.2)
    b = hw.batch(probs, method="mstvd")
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    b.advance(u, t, dts, 10)
    b.tune(u, dts, probe_steps=2)
    b.advance(u, t, dts, 7)
    got = b.unpack(u)
    for i, p in enumerate(probs):
        o = orc.ODE(p, int(p.ncells[0]), 1)
        uo = lines[i].copy()
        tt = o.integrate(uo, 0.0, (4 + 17 - 0.5) * dts[i], dts[i])
        assert tt == t[i] and np.array_equal(got[i], uo), i
    assert list(b.steps_done) == [21] * len(probs)


# ---- non-uniform lines in batches ----------------------------------------------------------------
def nonuniform_mix(hw, n, numerics, seed):
    """Uneven lines, every other one on a stretched grid (xedges), fluxes and k varied."""
    rng = np.random.default_rng(seed)
    probs, lines, dts = [], [], []
    for i in range(n):
        nc = int(rng.integers(20, 3000))
        k = int(rng.integers(1, 4))
        x = np.linspace(-1.0, 1.0, nc)
        u = np.exp(-((x - rng.uniform(-0.5, 0.5)) / 0.2) ** 2)
        if i % 3 == 0:
            p = hw.burgers_1d(nc, -1.0, 1.0, k=k, alpha=1.0, flux="godunov", bc="copy", numerics=numerics)
        else:
            p = hw.Problem(kind="fv1d", ncells=(nc, 1), k=k, flux="godunov" if i % 2 else "lax_friedrichs",
                           fn=("linear", "linear"), coef_a=(0.6, 0.0), coef_b=(0.3, 0.0), alpha=(0.9, 1.0),
                           bc=("zero_inflow", "copy"), xmin=(-1.0, 0.0), xmax=(1.0, 1.0), numerics=numerics)
        hmin = 2.0 / nc
        if i % 2 == 0:
            w = 1.001 ** np.arange(nc)
            e = -1.0 + 2.0 * np.concatenate([[0.0], np.cumsum(w) / w.sum()])
            p.xedges = (e, None)
            hmin = float(np.min(np.diff(e)))
        probs.append(p)
        lines.append(u)
        dts.append(0.2 * hmin)
    return probs, lines, np.array(dts)


@pytest.mark.parametrize("method", ["rktvd", "mstvd"])
@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_nonuniform_batch_matches_single_solves(hw, orc, method, numerics):
    """A batch whose lines are partly non-uniform (xedges: per-cell cnu, widths and true edges):
    every problem bit-identical to its own single-problem handle (FAST: the same recon_nu,
    flux and combine code), and to the oracle (STRICT), over two calls."""
    import torch
    probs, lines, dts = nonuniform_mix(hw, 18, numerics, 11)
    b = hw.batch(probs, method=method)
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    mk = (lambda p: hw.rktvd(p, int(p.ncells[0]), 3)) if method == "rktvd" else \
        (lambda p: hw.mstvd(p, int(p.ncells[0])))
    singles = [mk(p) for p in probs]
    us = [torch.from_numpy(v.copy()).cuda() for v in lines]
    ts = [0.0] * len(probs)
    orcs = [orc.ODE(p, int(p.ncells[0]), 0 if method == "rktvd" else 1, 3) for p in probs]
    uo = [v.copy() for v in lines]
    to = [0.0] * len(probs)
    for tout in (0.02, 0.06):
        b.integrate(u, t, tout, dts)
        got = b.unpack(u)
        for i, p in enumerate(probs):
            ts[i] = singles[i].integrate(us[i], ts[i], tout, dts[i])
            assert t[i] == ts[i]
            assert np.array_equal(got[i], us[i].cpu().numpy()), (i, tout)
            if numerics == "strict":
                to[i] = orcs[i].integrate(uo[i], to[i], tout, dts[i])
                assert to[i] == t[i] and np.array_equal(got[i], uo[i]), (i, tout)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_nonuniform_batch_f32c_matches_single_solves(hw, orc, order):
    """Compensated FP32 batches with non-uniform lines: every problem bit-identical to its own
    compensated single-problem handle (the same warp pass with per-cell coefficients), over two
    calls, and within the compensated form's bound of the FP64 oracle."""
    import torch
    probs, lines, dts = nonuniform_mix(hw, 18, "fast", 12)
    b = hw.batch(probs, order=order, dtype="f32c")
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    singles = [hw.rktvd(p, int(p.ncells[0]), order, dtype="f32c") for p in probs]
    us = [torch.from_numpy(v.copy()).cuda() for v in lines]
    ts = [0.0] * len(probs)
    for tout in (0.02, 0.06):
        b.integrate(u, t, tout, dts)
        got = b.unpack(u)
        for i in range(len(probs)):
            ts[i] = singles[i].integrate(us[i], ts[i], tout, dts[i])
            assert t[i] == ts[i]
            assert np.array_equal(got[i], us[i].cpu().numpy()), (i, tout)
    for i, p in enumerate(probs):
        uo = lines[i].copy()
        orc.ODE(p, int(p.ncells[0]), 0, order).integrate(uo, 0.0, 0.06, dts[i])
        assert np.sum(np.abs(got[i] - uo)) <= 1e-6 * np.sum(np.abs(uo)), i


@pytest.mark.parametrize("mix", ["uniform", "nonuniform"])
def test_mstvd_batch_f32c_matches_single_solves(hw, mix):
    """Compensated FP32 mstvd batches: every problem bit-identical to its own compensated mstvd
    handle over several integrate calls (the float-pair history carries across calls; problem 5
    starts on the second call), uniform and non-uniform lines, and the autotuner between calls
    leaves the histories as they are."""
    import torch
    from hrweno import workloads
    if mix == "uniform":
        probs, lines, dts = workloads.batched_config(24, seed=3, nmin=40, nmax=3000, cfl=0.2)
        touts = (0.05, 0.2, 1.5)
    else:
        probs, lines, dts = nonuniform_mix(hw, 18, "fast", 13)
        touts = (0.005, 0.01, 0.03)
    b = hw.batch(probs, dtype="f32c", method="mstvd")
    u = torch.from_numpy(b.pack(lines)).cuda()
    t = np.zeros(len(probs))
    t[5] = 1.0 if mix == "uniform" else 0.008
    singles = [hw.mstvd(p, int(p.ncells[0]), dtype="f32c") for p in probs]
    us = [torch.from_numpy(v.copy()).cuda() for v in lines]
    ts = [float(x) for x in t]
    for n, tout in enumerate(touts):
        b.integrate(u, t, tout, dts)
        got = b.unpack(u)
        for i in range(len(probs)):
            ts[i] = singles[i].integrate(us[i], ts[i], tout, dts[i])
            assert t[i] == ts[i], i
            assert np.isfinite(got[i]).all()
            assert np.array_equal(got[i], us[i].cpu().numpy()), (i, tout)
        if n == 0:
            b.tune(u, dts, probe_steps=2)
    assert list(b.steps_done) == [s.nsteps for s in singles]
