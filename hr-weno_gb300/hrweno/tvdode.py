"""rktvd / mstvd types (src/hrweno_tvdode.f90): TVD Runge-Kutta and multistep integrators.

The reference's `integrate(u, t, tout, dt)` updates u and t in place; Python floats are
immutable, so integrate() updates u in place and returns the new t.
"""
from __future__ import annotations

import ctypes as C

from . import _abi as A
from ._arrays import describe
from .problems import Problem

# "f64": the FP64 method; "f32": a REAL32 build of the reference (float32 arrays, FP32 time);
# "f32c": compensated FP32 bulk precision (user arrays stay float64)
_DT = {"f64": A.HRW_F64, "f32": A.HRW_F32, "f32c": A.HRW_F32C}


class _tvdode:
    dtype = "f64"

    def __init__(self, h, problem: Problem, neq: int, dtype: str):
        self._h = h
        self.problem = problem
        self.neq = neq
        self.dtype = dtype

    def integrate(self, u, t: float, tout: float, dt: float, itask: int = 1) -> float:
        """For dtype "f32" u is float32 and t, tout, dt are rounded to FP32 (the returned t is
        the FP32 time, exactly)."""
        real32 = self.dtype == "f32"
        mem, p, d = describe(u, self.neq, True, f64_only=not real32)
        if real32 and d != A.HRW_F32:
            raise TypeError("a REAL32 (dtype 'f32') integrator takes float32 arrays")
        tt = C.c_double(t)
        A.check(A.lib().hrw_integrate(self._h, mem, p, C.byref(tt), float(tout), float(dt),
                                      int(itask)))
        return tt.value

    def set_stream(self, stream) -> None:
        """Run on a CUDA stream (an int handle, e.g. torch.cuda.Stream().cuda_stream)."""
        A.check(A.lib().hrw_ode_set_stream(self._h, C.c_void_p(int(stream) if stream else 0)))

    def set_graphs(self, enable: bool) -> None:
        """Replay captured CUDA graphs for long integrations (default) or launch each stage."""
        A.check(A.lib().hrw_ode_set_graphs(self._h, int(bool(enable))))

    def set_cluster(self, enable: bool) -> None:
        """Run every step of an integrate call of a short uniform 1D line (6 to 4096 cells) in one
        thread-block cluster launch (default), or launch stage by stage.  Same results."""
        A.check(A.lib().hrw_ode_set_cluster(self._h, int(bool(enable))))

    def _info(self):
        fe, st, ns = C.c_int(), C.c_int(), C.c_int64()
        A.check(A.lib().hrw_ode_info(self._h, C.byref(fe), C.byref(st), C.byref(ns)))
        return fe.value, st.value, ns.value

    @property
    def fevals(self) -> int:
        return self._info()[0]

    @property
    def istate(self) -> int:
        return self._info()[1]

    @property
    def nsteps(self) -> int:
        return self._info()[2]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and A._lib is not None:
            A._lib.hrw_ode_destroy(h)
            self._h = None


class rktvd(_tvdode):  # noqa: N801
    """rktvd(fu, neq, order) with fu given as a Problem (src/hrweno_tvdode.f90:69-95)."""

    def __init__(self, problem: Problem, neq: int, order: int = 3, dtype: str = "f64"):
        h = C.c_void_p()
        self._cp = problem.to_c()
        A.check(A.lib().hrw_rktvd_create(C.byref(self._cp), int(neq), int(order), _DT[dtype],
                                         C.byref(h)))
        super().__init__(h, problem, int(neq), dtype)
        self.order = int(order)


class mstvd(_tvdode):  # noqa: N801
    """mstvd(fu, neq) with fu given as a Problem (src/hrweno_tvdode.f90:180-201)."""

    def __init__(self, problem: Problem, neq: int, dtype: str = "f64"):
        h = C.c_void_p()
        self._cp = problem.to_c()
        A.check(A.lib().hrw_mstvd_create(C.byref(self._cp), int(neq), _DT[dtype], C.byref(h)))
        super().__init__(h, problem, int(neq), dtype)
        self.order = 3
