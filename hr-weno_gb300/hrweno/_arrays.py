"""Array plumbing: numpy arrays are host memory, CUDA torch tensors are device memory."""
from __future__ import annotations

import numpy as np

from . import _abi as A


def describe(x, n: int, writable: bool, f64_only: bool = True):
    """Return (mem, pointer, dtype) of a contiguous 1D-viewable array of n elements.

    The integrators, batches and the adjoint read and write their arrays as n doubles, so
    they take float64 only (f64_only): a float32 array would be accessed past its end.
    reconstruct passes the element type on to the library, which checks it."""
    if isinstance(x, np.ndarray):
        if f64_only and x.dtype != np.float64:
            raise TypeError("arrays must be float64")
        if x.dtype not in (np.float64, np.float32):
            raise TypeError("arrays must be float64 or float32")
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        if writable and not x.flags.writeable:
            raise ValueError("output array is read-only")
        if x.size != n:
            raise ValueError(f"array has {x.size} elements, expected {n}")
        dt = A.HRW_F64 if x.dtype == np.float64 else A.HRW_F32
        return A.HRW_MEM_HOST, x.ctypes.data, dt
    try:
        import torch
    except ImportError as e:  # pragma: no cover
        raise TypeError("unsupported array type") from e
    if isinstance(x, torch.Tensor):
        if f64_only and x.dtype != torch.float64:
            raise TypeError("tensors must be float64")
        if x.dtype not in (torch.float64, torch.float32):
            raise TypeError("tensors must be float64 or float32")
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        if x.numel() != n:
            raise ValueError(f"tensor has {x.numel()} elements, expected {n}")
        dt = A.HRW_F64 if x.dtype == torch.float64 else A.HRW_F32
        mem = A.HRW_MEM_DEVICE if x.is_cuda else A.HRW_MEM_HOST
        return mem, x.data_ptr(), dt
    raise TypeError(f"unsupported array type {type(x)!r}")


def same_space(*mems) -> int:
    """The one memory space of a call's arrays (a call copies host arrays in and out, and uses
    device arrays in place, as a whole)."""
    if len(set(mems)) != 1:
        raise ValueError("the arrays of one call must all be host arrays or all CUDA tensors")
    return mems[0]
