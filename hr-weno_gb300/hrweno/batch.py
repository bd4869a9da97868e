"""batch: many independent rktvd solves of 1D problems advanced together (hrw_batch_* C ABI).

Each problem is one reference solve, `rktvd(fu_i, neq_i, order)` integrated with its own t and
dt (src/hrweno_tvdode.f90:69-178); the batch advances all of them with one persistent launch
per size class.  States are packed: problem i occupies u[offsets[i] : offsets[i] + ncells_i].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._arrays import describe
from .problems import Problem

_DT = {"f64": A.HRW_F64, "f32c": A.HRW_F32C}


def _setup(L):
    if getattr(L, "_batch_ready", False):
        return
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    dp = C.POINTER(C.c_double)
    L.hrw_batch_create.argtypes = [C.POINTER(A.HrwProblem), i, i, i, C.POINTER(vp)]
    L.hrw_batch_create_mstvd.argtypes = [C.POINTER(A.HrwProblem), i, i, C.POINTER(vp)]
    L.hrw_batch_layout.argtypes = [vp, C.POINTER(C.c_int64)]
    L.hrw_batch_integrate.argtypes = [vp, i, vp, dp, d, dp, i]
    L.hrw_batch_tune.argtypes = [vp, i, vp, dp, i, C.c_char_p]
    L.hrw_batch_advance.argtypes = [vp, i, vp, dp, dp, C.c_int64]
    L.hrw_batch_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int64)]
    L.hrw_batch_set_stream.argtypes = [vp, vp]
    L.hrw_batch_destroy.argtypes = [vp]
    for n in ("hrw_batch_create", "hrw_batch_create_mstvd", "hrw_batch_layout", "hrw_batch_integrate", "hrw_batch_tune",
              "hrw_batch_advance",
              "hrw_batch_info", "hrw_batch_set_stream", "hrw_batch_destroy"):
        getattr(L, n).restype = C.c_int
    L._batch_ready = True


class batch:  # noqa: N801
    """batch(problems, order=3, dtype="f64", method="rktvd"): problems are FV1D Problem
    descriptors on uniform grids or non-uniform ones (xedges); dtype "f64" or "f32c" (the
    compensated FP32 form, states still packed as float64).

    method="mstvd" makes every problem an mstvd(fu_i, neq_i) solve (src/hrweno_tvdode.f90:180-271):
    each keeps its multistep history between calls, and its first call runs the RK3 start."""

    def __init__(self, problems: list[Problem], order: int = 3, dtype: str = "f64",
                 method: str = "rktvd"):
        L = A.lib()
        _setup(L)
        arr = (A.HrwProblem * len(problems))()
        self._keep = []
        for k, p in enumerate(problems):
            arr[k] = p.to_c()
            self._keep.append(p)
        h = C.c_void_p()
        if method == "mstvd":
            A.check(L.hrw_batch_create_mstvd(arr, len(problems), _DT[dtype], C.byref(h)))
            order = 3
        elif method == "rktvd":
            A.check(L.hrw_batch_create(arr, len(problems), int(order), _DT[dtype], C.byref(h)))
        else:
            raise ValueError("method must be 'rktvd' or 'mstvd'")
        self._h = h
        self.method = method
        self.nprob = len(problems)
        self.order = int(order)
        off = np.empty(self.nprob + 1, dtype=np.int64)
        A.check(L.hrw_batch_layout(h, off.ctypes.data_as(C.POINTER(C.c_int64))))
        self.offsets = off
        self.ncells = np.array([p.ncells[0] for p in problems], dtype=np.int64)

    @property
    def size(self) -> int:
        """Length of the packed state."""
        return int(self.offsets[-1])

    def _check_times(self, t, dt) -> None:
        """t (updated in place: a float64 numpy array) and dt hold one value per problem."""
        if t is not None and not (isinstance(t, np.ndarray) and t.dtype == np.float64
                                  and t.ndim == 1 and t.size == self.nprob and t.flags.c_contiguous
                                  and t.flags.writeable):
            raise ValueError(f"t must be a writable contiguous float64 numpy array of {self.nprob} times")
        if np.size(dt) != self.nprob:
            raise ValueError(f"dt must hold {self.nprob} step sizes, one per problem")

    def pack(self, lines) -> np.ndarray:
        u = np.zeros(self.size)
        for k, v in enumerate(lines):
            u[self.offsets[k]: self.offsets[k] + self.ncells[k]] = v
        return u

    def unpack(self, u) -> list:
        u = u.cpu().numpy() if hasattr(u, "cpu") else np.asarray(u)
        return [u[self.offsets[k]: self.offsets[k] + self.ncells[k]] for k in range(self.nprob)]

    def integrate(self, u, t: np.ndarray, tout: float, dt: np.ndarray, itask: int = 1) -> None:
        """integrate(u_i, t[i], tout, dt[i], itask) for every problem; u and t in place."""
        mem, p, _ = describe(u, self.size, True)
        self._check_times(t, dt)
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        A.check(A.lib().hrw_batch_integrate(self._h, mem, p, t.ctypes.data_as(dp), float(tout),
                                            dt.ctypes.data_as(dp), int(itask)))

    def advance(self, u, t: np.ndarray, dt: np.ndarray, nsteps: int) -> None:
        """Exactly nsteps steps of every problem (nsteps integrate calls with itask=2)."""
        mem, p, _ = describe(u, self.size, True)
        self._check_times(t, dt)
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        A.check(A.lib().hrw_batch_advance(self._h, mem, p, t.ctypes.data_as(dp),
                                          dt.ctypes.data_as(dp), int(nsteps)))

    def tune(self, u, dt: np.ndarray, probe_steps: int = 5, cache_path: str | None = None):
        """Autotune the (group, cells-per-thread) shape of each size class; returns shapes."""
        mem, p, _ = describe(u, self.size, False)
        self._check_times(None, dt)
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        A.check(A.lib().hrw_batch_tune(self._h, mem, p, dt.ctypes.data_as(C.POINTER(C.c_double)),
                                       int(probe_steps),
                                       cache_path.encode() if cache_path else None))
        return self.shapes

    @property
    def shapes(self):
        s = (C.c_int * 6)()
        A.check(A.lib().hrw_batch_info(self._h, s, None))
        return [(s[2 * c], s[2 * c + 1]) for c in range(3)]

    @property
    def steps_done(self) -> np.ndarray:
        out = np.empty(self.nprob, dtype=np.int64)
        A.check(A.lib().hrw_batch_info(self._h, None, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def set_stream(self, stream) -> None:
        A.check(A.lib().hrw_batch_set_stream(self._h, C.c_void_p(int(stream) if stream else 0)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and A._lib is not None:
            A._lib.hrw_batch_destroy(h)
            self._h = None
