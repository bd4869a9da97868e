"""The MIXED kernel's difference-form algebra (hr-weno_gb300/csrc/hrw_mixed.cuh,
stage1d_mixed.cu), checked on the CPU through a numpy model of its FP32 path
(tests/mixed_model.py) against the oracle evaluated in binary128 (the REAL128 build of the
reference's formulas, src/hrweno_kinds.F90:13-14).

On cells where the kernel's rounding-error bound admits the FP32 path, dt L agrees with the
exact right-hand side to within that bound, and the bound is within the per-stage budget of
2^-53 max|u|; every variant the kernel covers (k = 2, 3; Burgers, linear advection; the first
stage and a stage with a float-pair increment; the full weights and the linear-weight pass that
warps take where the weights' deviations cannot matter) is checked.
"""
import numpy as np
import pytest

from mixed_model import mixed_dtl, split


def large_line(n, k, fn):
    from hrweno import Problem, workloads
    prob, u0, dt = workloads.large_burgers(n, k=k, numerics="strict")
    if fn == "linear":
        prob = Problem(kind="fv1d", ncells=(n, 1), k=k, flux="lax_friedrichs", fn=("linear", "linear"),
                       coef_a=(0.7, 0.0), coef_b=(0.0, 0.0), alpha=(1.0, 1.0), bc=("copy", "copy"),
                       xmin=(-5.0, 0.0), xmax=(5.0, 1.0), numerics="strict")
        dt = 0.4 * (10.0 / n)
    return prob, u0, dt


@pytest.mark.parametrize("nl", [True, False], ids=["weights", "linear_pass"])
@pytest.mark.parametrize("stage", ["first", "increment"])
@pytest.mark.parametrize("fn", ["burgers", "linear"])
@pytest.mark.parametrize("k", [3, 2])
def test_fp32_path_within_its_bound(orc, k, fn, stage, nl):
    n = 1 << 19
    prob, u0, dt = large_line(n, k, fn)
    g = 0.7 if fn == "linear" else 0.0
    dx = 10.0 / n
    dv = None
    v = u0
    if stage == "increment":
        # the stage input u + d1 with d1 a float-pair increment whose sum with u is exact in FP64
        d1 = (orc.rhs(prob, u0, prec=128) * dt).astype(np.float32)
        v = u0 + d1.astype(np.float64)
        dh, dl = split(v - u0)
        exact = dh.astype(np.float64) + dl.astype(np.float64) == v - u0
        v = np.where(exact, v, u0)
        dh, dl = split(v - u0)
        dv = (dh, dl)
    ref = orc.rhs(prob, v, prec=128) * dt
    cells, dtl, bound = mixed_dtl(u0, k, 1e-6, prob.alpha[0], dt, dx, fn=fn, g=g, dv=dv, nl=nl)
    err = np.abs(dtl - ref[cells])
    lim = 2.0 ** (np.floor(np.log2(np.max(np.abs(u0)))) - 53)
    soft = bound <= lim
    assert soft.mean() > 0.4  # much of a resolved line takes the FP32 path (more as n grows)
    # the bound holds wherever the FP32 path is taken
    assert np.all(err[soft] <= bound[soft]), float(np.max(err[soft] - bound[soft]))
    assert float(err[soft].max()) <= lim
    # and the FP32 path is far more accurate than the bound needs on this resolved line
    assert float(err[soft].max()) <= lim / 4


def test_split_is_the_fp64_value_to_47_bits():
    """The kernel's split_t: h is d truncated to 24 bits (exact in FP32), l the rest rounded to
    FP32, so that h + l is d to 2^-47 |d| (2^-74 <= |d| < 2^127)."""
    rng = np.random.default_rng(3)
    d = rng.standard_normal(100000) * np.exp2(rng.uniform(-70, 60, 100000))
    d = d[(np.abs(d) >= 2.0 ** -74) & (np.abs(d) < 2.0 ** 127)]
    h, lo = split(d)
    recon = h.astype(np.float64) + lo.astype(np.float64)
    assert np.all(np.abs(recon - d) <= 2.0 ** -47 * np.abs(d))
    assert np.all(np.abs(h.astype(np.float64)) <= np.abs(d))  # truncation toward zero
    assert np.all(np.abs(d - h.astype(np.float64)) < 2.0 ** -23 * np.abs(d))


def pack_model(h, lo):
    """numpy restatement of the kernel's mx::pack (float pair -> double by integer operations)"""
    h = np.asarray(h, np.float32)
    lo = np.asarray(lo, np.float32)
    hb = h.view(np.uint32).astype(np.int64)
    eb = (hb >> 23) & 0xFF
    se = np.clip(52 - (eb - 127) + 127, 1, 254)
    scale = ((se << 23).astype(np.uint32)).view(np.float32)
    k = np.rint((lo * scale).astype(np.float64)).astype(np.int64)
    k = np.where(eb >= 57, k, 0)
    k = np.where(hb & 0x80000000, -k, k)
    k = np.where(((hb & 0x7FFFFF) == 0) & (k < 0), 2 * k, k)
    return (h.astype(np.float64).view(np.int64) + k).view(np.float64)


def test_pack_is_the_pair_to_2e_52():
    """The last MIXED stage adds a float-pair increment to u with one FP64 addition, after
    packing the pair into the double nearest it (within 2^-52 of its value): random normalised
    pairs, powers of two with negative low words (the step into the lower binade), both signs."""
    rng = np.random.default_rng(11)
    n = 200000
    h = (rng.standard_normal(n) * np.exp2(rng.uniform(-60, 60, n))).astype(np.float32)
    h[: n // 4] = np.exp2(rng.integers(-60, 60, n // 4)).astype(np.float32) * rng.choice([-1, 1], n // 4)
    ulp = np.spacing(np.abs(h)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, n) * ulp).astype(np.float32)
    # keep the pairs normalised (fl32(h + l) == h)
    keep = (h + lo) == h
    h, lo = h[keep], lo[keep]
    exact = h.astype(np.longdouble) + lo.astype(np.longdouble)
    got = pack_model(h, lo).astype(np.longdouble)
    err = np.abs(got - exact) / np.abs(exact)
    assert float(err.max()) <= 2.0 ** -52, float(err.max())
