"""ctypes view of the C ABI declared in include/hrweno_gpu.h.

The shared library is built in-tree by hr-weno_gb300/build.py.  Loading fails loudly when it
is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libhrweno_gb300.so"

# status codes
HRW_OK, HRW_EINVAL, HRW_ECUDA, HRW_ESTATE, HRW_ETIMEOUT, HRW_ENOMEM = range(6)
HRW_F64, HRW_F32, HRW_F32C = 0, 1, 2
HRW_MEM_HOST, HRW_MEM_DEVICE = 0, 1
HRW_PROBLEM_FV1D, HRW_PROBLEM_FV2D, HRW_PROBLEM_LINEAR_ODE = 1, 2, 3
HRW_FLUX_LAX_FRIEDRICHS, HRW_FLUX_GODUNOV = 0, 1
HRW_FN_BURGERS, HRW_FN_LINEAR, HRW_FN_BURGERS_LINEAR = 0, 1, 2
HRW_BC_COPY, HRW_BC_ZERO, HRW_BC_ZERO_INFLOW = 0, 1, 2
HRW_NUMERICS_FAST, HRW_NUMERICS_STRICT, HRW_NUMERICS_MIXED = 0, 1, 2


class HrwProblem(C.Structure):
    """struct hrw_problem (field order and types as in the header)."""

    _fields_ = [
        ("kind", C.c_int32),
        ("ncells", C.c_int32 * 2),
        ("k", C.c_int32),
        ("eps", C.c_double),
        ("flux", C.c_int32),
        ("fn", C.c_int32 * 2),
        ("coef_a", C.c_double * 2),
        ("coef_b", C.c_double * 2),
        ("alpha", C.c_double * 2),
        ("bc", C.c_int32 * 2),
        ("xmin", C.c_double * 2),
        ("xmax", C.c_double * 2),
        ("width", C.POINTER(C.c_double) * 2),
        ("rates", C.POINTER(C.c_double)),
        ("numerics", C.c_int32),
        ("xedges", C.POINTER(C.c_double) * 2),
    ]


class HrwError(RuntimeError):
    """A C-ABI call returned a non-zero status; .code is the status, message the library's."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Load the library once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python hr-weno_gb300/build.py` "
                "(the GPU path has no fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.hrw_last_error.restype = C.c_char_p
        L.hrw_problem_init.argtypes = [C.POINTER(HrwProblem)]
        L.hrw_problem_init.restype = None
        L.hrw_weno_create.argtypes = [i, i, d, C.POINTER(C.c_double), C.POINTER(vp)]
        L.hrw_weno_set_numerics.argtypes = [vp, i]
        L.hrw_weno_reconstruct.argtypes = [vp, i, i, vp, vp, vp]
        L.hrw_weno_cnu.argtypes = [vp, C.POINTER(C.c_double)]
        L.hrw_weno_destroy.argtypes = [vp]
        L.hrw_rktvd_create.argtypes = [C.POINTER(HrwProblem), i, i, i, C.POINTER(vp)]
        L.hrw_mstvd_create.argtypes = [C.POINTER(HrwProblem), i, i, C.POINTER(vp)]
        L.hrw_integrate.argtypes = [vp, i, vp, C.POINTER(C.c_double), d, d, i]
        L.hrw_ode_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)]
        L.hrw_ode_set_stream.argtypes = [vp, vp]
        L.hrw_ode_set_graphs.argtypes = [vp, i]
        L.hrw_ode_set_cluster.argtypes = [vp, i]
        L.hrw_ode_destroy.argtypes = [vp]
        L.hrw_rhs.argtypes = [C.POINTER(HrwProblem), i, d, vp, vp, vp]
        for name in ("hrw_weno_create", "hrw_weno_set_numerics", "hrw_weno_reconstruct",
                     "hrw_weno_cnu", "hrw_weno_destroy", "hrw_rktvd_create", "hrw_mstvd_create",
                     "hrw_integrate", "hrw_ode_info", "hrw_ode_set_stream", "hrw_ode_destroy",
                     "hrw_ode_set_graphs", "hrw_ode_set_cluster",
                     "hrw_rhs"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != HRW_OK:
        raise HrwError(rc, lib().hrw_last_error().decode())
