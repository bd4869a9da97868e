"""TEST INFRASTRUCTURE ONLY - ctypes wrapper of the CPU oracle (oracle/hrweno_oracle.cpp).

Only tests/, __graft_entry__.smoke() and the cpu-baseline leg of bench.py import this module;
the product library never does.  The oracle restates HugoMVale/HR-WENO's Fortran in the
reference's operation order (see the header of hrweno_oracle.cpp) and is pinned by the
reference's own known-answer tests (tests/test_oracle_kat.py).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "hrweno_oracle.cpp"
LIB = HERE / "_build" / "libhrweno_oracle.so"
# Two builds of the same source:
#  parity   -O2, no fused multiply-add: the reference's operation order, the parity checker
#  baseline -O3 with the compiler's default contraction (as a gfortran -O3 build of the
#           reference would be): the fastest build of the restatement, used only to time the
#           CPU baseline; its results agree with the parity build to rounding
BUILDS = {
    "parity": (LIB, ["-O2", "-ffp-contract=off"]),
    "baseline": (HERE / "_build" / "libhrweno_oracle_o3.so", ["-O3"]),
}
COMMON = ["-fopenmp", "-fPIC", "-shared", "-std=c++17"]

_lib = None
_variant = "parity"


def build(force: bool = False, variant: str = "parity") -> Path:
    """Compile one build of the oracle with g++."""
    out, flags = BUILDS[variant]
    out.parent.mkdir(exist_ok=True)
    hdr = HERE.parent / "include" / "hrweno_gpu.h"
    if force or not out.exists() or out.stat().st_mtime < max(SRC.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["g++", *flags, *COMMON, "-o", str(out), str(SRC)], check=True)
    return out


def select_build(variant: str) -> None:
    """Use the 'parity' (default) or the 'baseline' build for the calls that follow."""
    global _lib, _variant
    if variant not in BUILDS:
        raise ValueError(variant)
    if variant != _variant:
        _variant = variant
        _lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(str(build(variant=_variant)))
        dp = C.POINTER(C.c_double)
        L.orc_last_error.restype = C.c_char_p
        L.orc_weno_reconstruct.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, dp, dp, dp, dp]
        L.orc_weno_calc_cnu.argtypes = [C.c_int, C.c_int, dp, dp]
        L.orc_numflux.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_numflux.restype = C.c_double
        L.orc_rhs.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_double, dp, dp]
        L.orc_ode_create.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.orc_ode_create.restype = C.c_void_p
        L.orc_ode_integrate.argtypes = [C.c_void_p, dp, dp, C.c_double, C.c_double, C.c_int]
        L.orc_ode_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_longlong)]
        L.orc_ode_destroy.argtypes = [C.c_void_p]
        L.orc_tl_misfit.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp, dp, C.c_double,
                                    C.c_longlong, dp, dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """Threads of the oracle's 1D cell loops (1: serial, as the reference); returns the count."""
    return lib().orc_set_threads(int(n))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleError(RuntimeError):
    pass


def reconstruct(v, k: int = 3, eps: float = 1e-6, xedges=None, prec: int = 64):
    """weno(nc, k, eps, xedges)%reconstruct(v, vl, vr) -> (vl, vr)."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    vl, vr = np.empty_like(v), np.empty_like(v)
    xe = None if xedges is None else np.ascontiguousarray(xedges, dtype=np.float64)
    rc = lib().orc_weno_reconstruct(prec, v.size, k, eps, None if xe is None else _p(xe),
                                    _p(v), _p(vl), _p(vr))
    if rc:
        raise OracleError(lib().orc_last_error().decode())
    return vl, vr


def calc_cnu(nc: int, k: int, xedges) -> np.ndarray:
    """cnu(0:k-1, -1:k-1, 1:nc) as an array [nc, k+1, k]."""
    xe = np.ascontiguousarray(xedges, dtype=np.float64)
    out = np.empty(k * (k + 1) * nc)
    lib().orc_weno_calc_cnu(nc, k, _p(xe), _p(out))
    return out.reshape(nc, k + 1, k)


FLUX_TEST_UXT = 100


def numflux(kind: int, fn: int, vm: float, vp: float, x: float, t: float, alpha: float = 0.0,
            a: float = 1.0, b: float = 0.0) -> float:
    """lax_friedrichs (kind 0) or godunov (kind 1) with flux fn."""
    return lib().orc_numflux(kind, fn, a, b, vm, vp, x, t, alpha)


def rhs(problem, v, t: float = 0.0, prec: int = 64) -> np.ndarray:
    """vdot = L(v) of a hrweno Problem."""
    cp = problem.to_c()
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.empty_like(v)
    lib().orc_rhs(prec, C.addressof(cp), v.size, t, _p(v), _p(out))
    return out


def tl_misfit(problem, u0, du0, target, dt: float, nsteps: int, order: int = 3):
    """(J, dJ): J = 0.5 ||u(T) - target||^2 after nsteps steps from u0 and its derivative in
    the direction du0, by the tangent-linear (dual number) model of the oracle."""
    cp = problem.to_c()
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    du0 = np.ascontiguousarray(du0, dtype=np.float64)
    target = np.ascontiguousarray(target, dtype=np.float64)
    J, dJ = C.c_double(), C.c_double()
    lib().orc_tl_misfit(C.addressof(cp), u0.size, order, _p(u0), _p(du0), _p(target), dt,
                        nsteps, C.byref(J), C.byref(dJ))
    return J.value, dJ.value


class ODE:
    """rktvd (method 0) / mstvd (method 1) of the oracle at precision prec (32, 64, 128)."""

    def __init__(self, problem, neq: int, method: int = 0, order: int = 3, prec: int = 64):
        self._cp = problem.to_c()
        self._h = lib().orc_ode_create(prec, C.addressof(self._cp), neq, method, order)
        if not self._h:
            raise OracleError(lib().orc_last_error().decode())
        self.neq = neq

    def integrate(self, u: np.ndarray, t: float, tout: float, dt: float, itask: int = 1) -> float:
        assert u.dtype == np.float64 and u.flags.c_contiguous and u.size == self.neq
        tt = C.c_double(t)
        lib().orc_ode_integrate(self._h, _p(u), C.byref(tt), tout, dt, itask)
        return tt.value

    def info(self):
        fe, st, ns = C.c_int(), C.c_int(), C.c_longlong()
        lib().orc_ode_info(self._h, C.byref(fe), C.byref(st), C.byref(ns))
        return fe.value, st.value, ns.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_ode_destroy(self._h)
            self._h = None
