"""Array plumbing: numpy arrays are host memory, CUDA torch tensors are device memory."""
from __future__ import annotations

import numpy as np

from . import _abi as A


def describe(x, n: int, writable: bool):
    """Return (mem, pointer, dtype) of a contiguous 1D-viewable array of n elements."""
    if isinstance(x, np.ndarray):
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
