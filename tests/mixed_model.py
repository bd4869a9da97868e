"""A numpy model of the MIXED kernel's FP32 path (hr-weno_gb300/csrc/stage1d_mixed.cu,
hrw_mixed.cuh), for the CPU tests of its difference-form algebra.

It follows the kernel's formulas cell by cell, vectorised over the line: FP64 neighbour
differences split into float pairs, FP32 second differences, the interface sums X and Y, the
weight deviations from factored indicator differences, the float-pair S and the FP32 T and
quadratic terms, dt L = -c (4 dF) as a pair, and the kernel's rounding-error bound.  Products
and sums are rounded to float32 after each operation (fused multiply-adds are evaluated in
float64 and rounded once, which matches a true fused multiply-add except in rare double-rounding
cases); the model therefore tracks the kernel to a few float32 ulps of each term, which is what
the algebra checks need.  Only interior cells (four cells from either end and beyond) are
modelled, as only those take the FP32 path.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def r(x):
    """round to float32"""
    return np.asarray(x, dtype=np.float64).astype(f32)


def fma(a, b, c):
    return r(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def split(d):
    """FP64 d -> (h, l) as the kernel's split_t: h = d truncated to 24 significant bits,
    l = fl32(d - h); |d| < 2^-126 gives (0, 0) and |d| < 2^-74 gives l = 0"""
    d = np.asarray(d, np.float64)
    bits = d.view(np.uint64) & ~np.uint64(0x1FFFFFFF)
    ht = bits.view(np.float64)
    h = ht.astype(f32)
    lo = (d - ht).astype(f32)
    E = ((d.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    lo = np.where(E >= 949, lo, f32(0))
    h = np.where(E >= 897, h, f32(0))
    return h, lo


def rec3(d, D, tA, eps):
    """kernel's mx::rec3 on arrays: d = (dmm, dm, d0, d1), D = (A2, A1, A0), tA likewise"""
    dmm, dm, d0, d1 = d
    A2, A1, A0 = D
    B0 = fma(-2.0, d0, A0)
    B1 = r(dm + d0)
    B2 = fma(2.0, dm, A2)
    e0 = fma(r(0.25 * B0), B0, tA[2])
    e1 = fma(r(0.25 * B1), B1, tA[1])
    e2 = fma(r(0.25 * B2), B2, tA[0])
    a10, a21 = r(A1 - A0), r(A2 - A1)
    b10 = r(a10 * fma(13.0 / 12.0, r(A1 + A0), r(-0.25 * r(fma(3.0, d0, dm) - A0))))
    b21 = r(a21 * fma(13.0 / 12.0, r(A2 + A1), r(0.25 * fma(3.0, dm, r(A2 + d0)))))
    b20 = r(b21 + b10)
    s0, s1, s2 = r(e0 * e0), r(e1 * e1), r(e2 * e2)
    q10, q20, q21 = r(b10 * r(e1 + e0)), r(b20 * r(e2 + e0)), r(b21 * r(e2 + e1))
    P0, P1, P2 = r(s1 * s2), r(s0 * s2), r(s0 * s1)
    rD = r(1.0 / fma(3.0, P0, fma(6.0, P1, P2)).astype(np.float64))
    rDt = r(1.0 / fma(3.0, P2, fma(6.0, P1, P0)).astype(np.float64))
    u20, u10, u21 = r(q20 * s1), r(q10 * s2), r(q21 * s0)
    N0 = fma(6.0, u10, u20)
    N2 = -fma(6.0, u21, r(3.0 * u20))
    M0 = fma(6.0, u10, r(3.0 * u20))
    M2 = -fma(6.0, u21, u20)
    rrn = r(fma(r(3.0 * N0), a10, r(r(2.0 * N2) * a21)) * r(rD * f32(1.0 / 60.0)))
    rln = r(fma(r(-2.0 * M0), a10, r(r(-3.0 * M2) * a21)) * r(rDt * f32(1.0 / 60.0)))
    dev = r(r(fma(3.0, np.abs(N0), np.abs(N2)) * rD + fma(3.0, np.abs(M2), np.abs(M0)) * rDt) * 0.2)
    rlin = r(fma(24.0, d0, fma(-3.0, d1, fma(11.0, dm, r(-2.0 * dmm)))) * f32(1.0 / 60.0))
    llin = r(fma(2.0, d1, fma(-11.0, d0, fma(-24.0, dm, r(3.0 * dmm)))) * f32(1.0 / 60.0))
    return r(rlin + rrn), r(llin + rln), rrn, rln, dev


def rec2(d, D, eps):
    dm, d0 = d
    A = D[0]
    e0, e1 = fma(d0, d0, eps), fma(dm, dm, eps)
    s0, s1 = r(e0 * e0), r(e1 * e1)
    q10 = r(r(-A * r(dm + d0)) * r(e0 + e1))
    rD = r(1.0 / fma(2.0, s1, s0).astype(np.float64))
    rDt = r(1.0 / fma(2.0, s0, s1).astype(np.float64))
    rrn = r(r(r(q10 * A) * rD) * f32(1.0 / 3.0))
    rln = r(r(r(-q10 * A) * rDt) * f32(1.0 / 3.0))
    dev = r(r(np.abs(q10) * r(rD + rDt)) * f32(4.0 / 3.0))
    rr = r(fma(1.0 / 3.0, d0, r(f32(1.0 / 6.0) * dm)) + rrn)
    rl = r(-fma(1.0 / 6.0, d0, r(f32(1.0 / 3.0) * dm)) + rln)
    return rr, rl, rrn, rln, dev


def lin(k, d):
    """the kernel's mx::lin: linear-weight parts of rr and rl"""
    if k == 3:
        dmm, dm, d0, d1 = d
        rr = r(fma(24.0, d0, fma(-3.0, d1, fma(11.0, dm, r(-2.0 * dmm)))) * f32(1.0 / 60.0))
        rl = r(fma(2.0, d1, fma(-11.0, d0, fma(-24.0, dm, r(3.0 * dmm)))) * f32(1.0 / 60.0))
    else:
        dm, d0 = d
        rr = fma(1.0 / 3.0, d0, r(f32(1.0 / 6.0) * dm))
        rl = -fma(1.0 / 6.0, d0, r(f32(1.0 / 3.0) * dm))
    return rr, rl


def mixed_dtl(u, k, eps, alpha, dt, dx, fn="burgers", g=0.0, dv=None, nl=True):
    """dt L(v) of the FP32 path for the interior cells j = 4 .. n-5 of v = u (+ dv, a float-pair
    increment given as (h, l) arrays), and the kernel's bound on its rounding error, as
    (cells, dtL (float64 value of the pair), bound).  The bound is per cell here; the kernel
    takes the largest over each lane's window, which is no smaller.  nl = False: the
    linear-weight pass (weights dropped); its bound includes the dropped parts and is inf where
    the kernel would not take that pass (indicator differences above eps / 100)."""
    u = np.asarray(u, np.float64)
    n = u.size
    d64 = u[1:] - u[:-1]              # d_q = u_{q+1} - u_q, q = 0 .. n-2
    dh, dl = split(d64)
    if dv is not None:                # d(v) = d(u) + (dv_{q+1} - dv_q) in pairs
        vh, vl = dv
        bh, bl = r(vh[1:] - vh[:-1]), r(vl[1:] - vl[:-1])
        s = r(dh + bh)
        bb = r(s - dh)
        e = r(r(dh - r(s - bb)) + r(bh - bb))
        lo = r(e + r(dl + bl))
        h2 = r(s + lo)
        dl = r(lo - r(h2 - s))
        dh = h2
    D = r(r(dh[1:] - dh[:-1]) + r(dl[1:] - dl[:-1]))  # D_q = Dd_q, q = 0 .. n-3
    df = r(dh + dl)                   # d to FP32 precision (the kernel's d[])
    epsf = f32(eps)
    cells = np.arange(4, n - 4)
    # reconstructions of cells j-1, j, j+1 for every interior j: index arrays on cell c
    def rec(c):
        if not nl:
            dd = (df[c - 2], df[c - 1], df[c], df[c + 1]) if k == 3 else (df[c - 1], df[c])
            rr, rl = lin(k, dd)
            z = np.zeros_like(rr)
            return rr, rl, z, z, z
        if k == 3:
            dd = (df[c - 2], df[c - 1], df[c], df[c + 1])
            DD = (D[c - 2], D[c - 1], D[c])
            tA = tuple(fma(r(f32(13.0 / 12.0) * x), x, epsf) for x in DD)
            return rec3(dd, DD, tA, epsf)
        return rec2((df[c - 1], df[c]), (D[c - 1],), epsf)
    Rm, R0, Rp = rec(cells - 1), rec(cells), rec(cells + 1)

    def XY(i):
        if k == 3:
            X = r(fma(6.0, r(D[i - 1] + D[i]), -r(D[i - 2] + D[i + 1])) * f32(1.0 / 30.0))
            Y = r(-fma(-3.0, r(D[i] - D[i - 1]), r(D[i + 1] - D[i - 2])) * f32(1.0 / 30.0))
        else:
            X = r(r(D[i - 1] + D[i]) * f32(1.0 / 6.0))
            Y = r(r(D[i] - D[i - 1]) * f32(1.0 / 6.0))
        return X, Y
    Xj, Yj = XY(cells)
    Xm, Ym = XY(cells - 1)
    j = cells
    aR, bR = R0[0], r(df[j] + Rp[1])
    aL, bL = r(Rm[0] - df[j - 1]), R0[1]
    Sn = r(r(R0[2] + Rp[3]) - r(Rm[2] + R0[3]))
    Tn = r(r(R0[2] - Rp[3]) - r(Rm[2] - R0[3]))
    sh = r(dh[j] + dh[j - 1])
    bb = r(sh - dh[j])
    se = r(r(dh[j] - r(sh - bb)) + r(dh[j - 1] - bb))
    sl = r(r(r(se + r(dl[j] + dl[j - 1])) - r(Xj - Xm)) + Sn)
    T = r(r(Yj - Ym) + Tn)
    if fn == "burgers":
        Vh, Vl = split(u[j])
        if dv is not None:
            Vl = r(Vl + r(dv[0][j] + dv[1][j]))
    else:
        Vh = np.full(j.size, f32(g))
        Vl = np.full(j.size, f32(g - float(f32(g))))
    p = r(r(2.0 * Vh) * sh)
    pl = fma(r(2.0 * Vh), sh, -p)
    pl = fma(r(2.0 * Vh), sl, pl)
    pl = fma(r(2.0 * Vl), sh, pl)
    q = r(r(2.0 * f32(alpha)) * T)
    if fn == "burgers":
        q = r(q + r(fma(aR, aR, r(bR * bR)) - fma(aL, aL, r(bL * bL))))
    c = dt / (4.0 * dx)
    ch = f32(c)
    cl = f32(c - float(ch))
    Fh = r(p + r(pl + q))
    Fl = r(r(pl + q) - r(Fh - p))
    th = r(ch * Fh)
    tl = fma(ch, Fh, -th)
    tl = fma(ch, Fl, fma(cl, Fh, tl))
    dtl = -(th.astype(np.float64) + tl.astype(np.float64))
    # the kernel's bound (per cell, over the cell's window)
    lo, hi = j - 3, j + 3
    Md = np.maximum.reduce([np.abs(df[lo + t]) for t in range(6)])
    Mdd = np.maximum.reduce([np.abs(D[np.clip(lo + t, 0, D.size - 1)]) for t in range(5)])
    dev = np.maximum.reduce([Rm[4], R0[4], Rp[4]])
    inv_eps = f32(1.0 / eps)
    if not nl:  # the linear-weight pass's bound, from the window maxima alone
        Md64, Mdd64 = Md.astype(np.float64), Mdd.astype(np.float64)
        Vb = (np.abs(u[j]) + (np.abs(dv[0][j]) if dv is not None else 0.0)) * 1.001
        if fn != "burgers":
            Vb = np.full(j.size, abs(float(f32(g))))
        Db = 4.0 * Mdd64 * (Md64 + 2.5 * Mdd64)
        eSkip = 6.0 * Db * Mdd64 * float(inv_eps)
        eL = 2.0 ** -21 * Mdd64 + 2.0 ** -46 * Md64 + eSkip
        a_f = float(f32(alpha))
        e4 = 2.0 * Vb * eL + 2.0 * a_f * eL + 2.0 ** -92 * (Vb + a_f)
        if fn == "burgers":
            e4 = e4 + Md64 * (2.0 ** -18 * Md64 + 8.0 * eSkip)
        bound = float(f32(dt / (4.0 * dx))) * e4
        return cells, dtl, np.where(Db * float(inv_eps) <= 0.01, bound, np.inf)
    eNL = r(2.0 ** -18 * Mdd.astype(np.float64) * dev + 2.0 ** -12 * Mdd.astype(np.float64) ** 2
            * (Md.astype(np.float64) + Mdd) * inv_eps)
    eST = 2.0 ** -21 * Mdd + 2.0 ** -46 * Md + eNL
    Vb = np.abs(Vh.astype(np.float64)) * 1.001
    e4 = 2.0 * Vb * eST + 2.0 * float(f32(alpha)) * eST + 2.0 ** -92 * (Vb + float(f32(alpha)))
    if fn == "burgers":
        errmax = np.maximum(np.abs(aR), np.abs(bR)) + np.maximum(np.abs(aL), np.abs(bL))
        e4 = e4 + 2.0 ** -21 * Md * 2.0 * errmax
    return cells, dtl, float(ch) * e4
