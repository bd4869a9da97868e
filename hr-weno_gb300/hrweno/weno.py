"""weno type (src/hrweno_weno.f90:23-50): construct once per grid line, then reconstruct."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._arrays import describe, same_space


class weno:  # noqa: N801 - the reference's type name
    """weno(ncells, k=3, eps=1e-6, xedges=None), as weno_init (src/hrweno_weno.f90:54-127).

    Invalid input raises HrwError with the reference's message where the reference would
    `error stop`."""

    def __init__(self, ncells: int, k: int = 3, eps: float = 1e-6, xedges=None,
                 numerics: str = "fast"):
        L = A.lib()
        h = C.c_void_p()
        xe = None
        if xedges is not None:
            xe = np.ascontiguousarray(xedges, dtype=np.float64)
            if xe.size != ncells + 1:
                raise A.HrwError(A.HRW_EINVAL,
                                 "Invalid input 'xedges': size(xedges) /= ncells + 1.")
        A.check(L.hrw_weno_create(int(ncells), int(k), float(eps),
                                  xe.ctypes.data_as(C.POINTER(C.c_double)) if xe is not None else None,
                                  C.byref(h)))
        self._h = h
        # k <= 0 and eps <= 0 select the defaults, as in hrw_weno_create
        self.ncells = int(ncells)
        self.k = int(k) if int(k) > 0 else 3
        self.eps = float(eps) if float(eps) > 0.0 else 1e-6
        self.uniform_grid = xedges is None
        if numerics != "fast":
            A.check(L.hrw_weno_set_numerics(h, A.HRW_NUMERICS_STRICT))

    def reconstruct(self, v, vl, vr) -> None:
        """vl(i) = v^+_{i-1/2}, vr(i) = v^-_{i+1/2} (src/hrweno_weno.f90:129-219)."""
        m0, p0, d0 = describe(v, self.ncells, False, f64_only=False)
        m1, p1, d1 = describe(vl, self.ncells, True, f64_only=False)
        m2, p2, d2 = describe(vr, self.ncells, True, f64_only=False)
        same_space(m0, m1, m2)
        if not d0 == d1 == d2:
            raise ValueError("v, vl and vr must share one element type")
        A.check(A.lib().hrw_weno_reconstruct(self._h, d0, m0, p0, p1, p2))

    @property
    def cnu(self) -> np.ndarray:
        """Non-uniform coefficients cnu(0:k-1, -1:k-1, 1:nc) as an array [nc, k+1, k]."""
        out = np.empty(self.k * (self.k + 1) * self.ncells)
        A.check(A.lib().hrw_weno_cnu(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.ncells, self.k + 1, self.k)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and A._lib is not None:
            A._lib.hrw_weno_destroy(h)
            self._h = None
