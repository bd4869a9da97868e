"""Problem descriptors: the right-hand side L(u) that the reference passes as a procedure.

The reference's integrators call a user subroutine `fu(t, u, udot)` through a procedure
pointer (src/hrweno_tvdode.f90:16,50-57).  The GPU stage kernels cannot call back into host
code, so the right-hand side is described by data instead; the fields mirror the examples'
choices (example/example1_burgers_1d_fv.f90:72-122, example/example2_pbe_2d_fv.f90:73-155).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

_FLUX = {"lax_friedrichs": A.HRW_FLUX_LAX_FRIEDRICHS, "godunov": A.HRW_FLUX_GODUNOV}
# flux functions f(u, x): "burgers" u^2/2, "linear" (a + b x) u, "burgers_linear" u^2/2 + (a + b x) u
_FN = {"burgers": A.HRW_FN_BURGERS, "linear": A.HRW_FN_LINEAR, "burgers_linear": A.HRW_FN_BURGERS_LINEAR}
_BC = {"copy": A.HRW_BC_COPY, "zero": A.HRW_BC_ZERO, "zero_inflow": A.HRW_BC_ZERO_INFLOW}
_NUM = {"fast": A.HRW_NUMERICS_FAST, "strict": A.HRW_NUMERICS_STRICT,
        "mixed": A.HRW_NUMERICS_MIXED}


@dataclass
class Problem:
    """Description of L(u).  kind: 'fv1d', 'fv2d' or 'linear_ode'."""

    kind: str = "fv1d"
    ncells: tuple = (1, 1)
    k: int = 3
    eps: float = 1e-6
    flux: str = "lax_friedrichs"
    fn: tuple = ("burgers", "burgers")
    coef_a: tuple = (1.0, 1.0)
    coef_b: tuple = (0.0, 0.0)
    alpha: tuple = (1.0, 1.0)
    bc: tuple = ("copy", "copy")
    xmin: tuple = (0.0, 0.0)
    xmax: tuple = (1.0, 1.0)
    width: tuple = (None, None)
    rates: object = None
    numerics: str = "fast"
    xedges: tuple = (None, None)
    _keep: list = field(default_factory=list, repr=False, compare=False)  # arrays to_c() points at

    @property
    def neq(self) -> int:
        if self.kind == "fv2d":
            return int(self.ncells[0]) * int(self.ncells[1])
        if self.kind == "linear_ode":
            return len(self.rates)
        return int(self.ncells[0])

    def to_c(self) -> A.HrwProblem:
        p = A.HrwProblem()
        p.kind = {"fv1d": A.HRW_PROBLEM_FV1D, "fv2d": A.HRW_PROBLEM_FV2D,
                  "linear_ode": A.HRW_PROBLEM_LINEAR_ODE}[self.kind]
        nc = list(self.ncells) + [1] * (2 - len(self.ncells))
        if self.kind == "linear_ode":
            nc = [len(self.rates), 1]
        p.ncells[0], p.ncells[1] = int(nc[0]), int(nc[1])
        p.k = int(self.k)
        p.eps = float(self.eps)
        p.flux = _FLUX[self.flux]
        p.numerics = _NUM[self.numerics]
        self._keep = []
        for d in range(2):
            p.fn[d] = _FN[self.fn[d]]
            p.coef_a[d] = float(self.coef_a[d])
            p.coef_b[d] = float(self.coef_b[d])
            p.alpha[d] = float(self.alpha[d])
            p.bc[d] = _BC[self.bc[d]]
            p.xmin[d] = float(self.xmin[d])
            p.xmax[d] = float(self.xmax[d])
            w = self.width[d]
            if w is not None:
                w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1)
                if w.size != p.ncells[d]:  # the library reads ncells widths
                    raise A.HrwError(A.HRW_EINVAL, "Invalid input 'width': size(width) /= ncells.")
                self._keep.append(w)
                p.width[d] = w.ctypes.data_as(C.POINTER(C.c_double))
            xe = self.xedges[d] if self.xedges is not None else None
            if xe is not None:
                xe = np.ascontiguousarray(xe, dtype=np.float64).reshape(-1)
                if xe.size != p.ncells[d] + 1:  # the library reads ncells + 1 edges
                    raise A.HrwError(A.HRW_EINVAL,
                                     "Invalid input 'xedges': size(xedges) /= ncells + 1.")
                self._keep.append(xe)
                p.xedges[d] = xe.ctypes.data_as(C.POINTER(C.c_double))
        if self.rates is not None:
            r = np.ascontiguousarray(self.rates, dtype=np.float64)
            self._keep.append(r)
            p.rates = r.ctypes.data_as(C.POINTER(C.c_double))
        return p


def burgers_1d(nc: int, xmin: float = -5.0, xmax: float = 5.0, k: int = 3, eps: float = 1e-6,
               flux: str = "lax_friedrichs", alpha: float = 1.0, bc: str = "copy", width=None,
               numerics: str = "fast") -> Problem:
    """1D inviscid Burgers FV, f(u) = u^2/2 (example/example1_burgers_1d_fv.f90)."""
    return Problem(kind="fv1d", ncells=(nc, 1), k=k, eps=eps, flux=flux,
                   fn=("burgers", "burgers"), alpha=(alpha, alpha), bc=(bc, bc),
                   xmin=(xmin, 0.0), xmax=(xmax, 1.0), width=(width, None), numerics=numerics)


def pbe_2d(nc1: int, nc2: int, g1=(1.0, 0.5), g2=(0.5, 0.0), k: int = 3, eps: float = 1e-6,
           flux: str = "godunov", bc: str = "zero_inflow", xmin=(0.0, 0.0), xmax=(1.0, 1.0),
           numerics: str = "fast") -> Problem:
    """2D population balance FV, d(g1 n)/dx1 + d(g2 n)/dx2 (example/example2_pbe_2d_fv.f90);
    g_d = a + b x evaluated at the interface, given as (a, b)."""
    return Problem(kind="fv2d", ncells=(nc1, nc2), k=k, eps=eps, flux=flux,
                   fn=("linear", "linear"), coef_a=(g1[0], g2[0]), coef_b=(g1[1], g2[1]),
                   alpha=(abs(g1[0]) + abs(g1[1]), abs(g2[0]) + abs(g2[1])), bc=(bc, bc),
                   xmin=tuple(xmin), xmax=tuple(xmax), numerics=numerics)


def linear_ode(rates, numerics: str = "fast") -> Problem:
    """u_i' = a_i u_i, the integrator test problem (test/test_tvdode.f90:107-118)."""
    r = np.ascontiguousarray(rates, dtype=np.float64)
    return Problem(kind="linear_ode", ncells=(len(r), 1), rates=r, numerics=numerics)
