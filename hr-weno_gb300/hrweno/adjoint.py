"""adjoint: gradient of J = 0.5 ||u(T) - target||^2 with respect to u0 (hrw_adjoint_* C ABI).

No counterpart in the reference.  The forward map is nsteps rktvd(order 3) steps
(src/hrweno_tvdode.f90:161-169) of an FV1D problem with the global Lax-Friedrichs flux at fixed
alpha; the reverse sweep is the hand-written discrete adjoint of the fused stage kernels, with
forward recompute from checkpoints.  The pass that records a segment also records each cell's
WENO-map derivatives (the WENO tape) when memory allows, so the reverse pass reads them instead
of recomputing them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._arrays import describe, same_space
from .problems import Problem


def _setup(L):
    if getattr(L, "_adj_ready", False):
        return
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    dp = C.POINTER(C.c_double)
    L.hrw_adjoint_create.argtypes = [C.POINTER(A.HrwProblem), i, i, C.POINTER(vp)]
    L.hrw_adjoint_gradient.argtypes = [vp, i, vp, vp, d, C.c_int64, dp, vp]
    L.hrw_adjoint_forward.argtypes = [vp, i, vp, vp, d, C.c_int64, dp, vp]
    L.hrw_adjoint_vjp.argtypes = [vp, i, vp, vp, d, C.c_int64, vp]
    L.hrw_adjoint_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.hrw_adjoint_tape_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.hrw_adjoint_set_stream.argtypes = [vp, vp]
    L.hrw_adjoint_destroy.argtypes = [vp]
    for n in ("hrw_adjoint_create", "hrw_adjoint_gradient", "hrw_adjoint_forward", "hrw_adjoint_vjp",
              "hrw_adjoint_info", "hrw_adjoint_tape_info", "hrw_adjoint_set_stream",
              "hrw_adjoint_destroy"):
        getattr(L, n).restype = C.c_int
    L._adj_ready = True


class adjoint:  # noqa: N801
    """adjoint(problem, nseg=1, checkpoint_every=45): nseg packed problems of ncells each, on a
    uniform line or the problem's non-uniform one (xedges, the same edges in every segment);
    checkpoint_every=0 picks the segment length from the free device memory (the whole
    trajectory with the WENO tape when it fits, else sqrt(nsteps) segments)."""

    def __init__(self, problem: Problem, nseg: int = 1, checkpoint_every: int = 45):
        L = A.lib()
        _setup(L)
        self._cp = problem.to_c()
        h = C.c_void_p()
        A.check(L.hrw_adjoint_create(C.byref(self._cp), int(nseg), int(checkpoint_every),
                                     C.byref(h)))
        self._h = h
        self.nseg = int(nseg)
        self.size = int(problem.ncells[0]) * self.nseg

    def gradient(self, u0, target, dt: float, nsteps: int, grad=None):
        """(J, grad): J[nseg] (numpy) and dJ/du0 (same kind of array as u0)."""
        m0, p0, _ = describe(u0, self.size, False)
        m1, p1, _ = describe(target, self.size, False)
        if grad is None:
            grad = u0.new_empty(u0.shape) if hasattr(u0, "new_empty") else np.empty_like(u0)
        m2, p2, _ = describe(grad, self.size, True)
        same_space(m0, m1, m2)
        J = np.empty(self.nseg)
        A.check(A.lib().hrw_adjoint_gradient(self._h, m0, p0, p1, float(dt), int(nsteps),
                                             J.ctypes.data_as(C.POINTER(C.c_double)), p2))
        return J, grad

    def forward(self, u0, target, dt: float, nsteps: int, uT=None):
        """(J, uT) of the forward solve alone (J is None when target is None)."""
        m0, p0, _ = describe(u0, self.size, False)
        mems = [m0]
        p1 = None
        if target is not None:
            m1, p1, _ = describe(target, self.size, False)
            mems.append(m1)
        pT = None
        if uT is not None:
            mT, pT, _ = describe(uT, self.size, True)
            mems.append(mT)
        same_space(*mems)
        J = np.empty(self.nseg)
        A.check(A.lib().hrw_adjoint_forward(self._h, m0, p0, p1, float(dt), int(nsteps),
                                            J.ctypes.data_as(C.POINTER(C.c_double)), pT))
        return (J if target is not None else None), uT

    def vjp(self, u0, lambda_T, dt: float, nsteps: int, grad=None):
        """d <lambda_T, u(T)> / du0."""
        m0, p0, _ = describe(u0, self.size, False)
        m1, p1, _ = describe(lambda_T, self.size, False)
        if grad is None:
            grad = u0.new_empty(u0.shape) if hasattr(u0, "new_empty") else np.empty_like(u0)
        m2, p2, _ = describe(grad, self.size, True)
        same_space(m0, m1, m2)
        A.check(A.lib().hrw_adjoint_vjp(self._h, m0, p0, p1, float(dt), int(nsteps), p2))
        return grad

    @property
    def forward_steps(self) -> int:
        """Forward steps (initial pass + recompute) of the last gradient call."""
        n = C.c_int64()
        A.check(A.lib().hrw_adjoint_info(self._h, C.byref(n), None))
        return n.value

    @property
    def checkpoint_every(self) -> int:
        """Checkpoint interval used by the last gradient call."""
        n = C.c_int64()
        A.check(A.lib().hrw_adjoint_info(self._h, None, C.byref(n)))
        return n.value

    @property
    def tape_bytes(self) -> tuple[int, int]:
        """(state bytes, WENO-tape bytes) the last gradient call kept on the device; a WENO
        tape of 0 bytes means the reverse pass recomputed the WENO maps from the states."""
        s, w = C.c_int64(), C.c_int64()
        A.check(A.lib().hrw_adjoint_tape_info(self._h, C.byref(s), C.byref(w)))
        return s.value, w.value

    def set_stream(self, stream) -> None:
        A.check(A.lib().hrw_adjoint_set_stream(self._h, C.c_void_p(int(stream) if stream else 0)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and A._lib is not None:
            A._lib.hrw_adjoint_destroy(h)
            self._h = None
