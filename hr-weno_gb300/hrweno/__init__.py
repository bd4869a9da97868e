"""GB300 implementation of HR-WENO's hot path, with the reference's Python-facing names.

    from hrweno import weno, rktvd, mstvd, Problem

mirrors the Fortran modules hrweno_weno (weno, %reconstruct) and hrweno_tvdode (rktvd, mstvd,
%integrate) of HugoMVale/HR-WENO.  Arrays are numpy arrays (host) or CUDA torch tensors
(device); all compute runs in the CUDA library built from hr-weno_gb300/csrc.
"""
from ._abi import (HRW_BC_COPY, HRW_BC_ZERO, HRW_BC_ZERO_INFLOW, HRW_EINVAL, HRW_ENOMEM,  # noqa: F401
                   HRW_ECUDA, HRW_ESTATE, HRW_ETIMEOUT, HRW_F32, HRW_F32C, HRW_F64,
                   HRW_FLUX_GODUNOV, HRW_FLUX_LAX_FRIEDRICHS, HRW_FN_BURGERS, HRW_FN_BURGERS_LINEAR,
                   HRW_FN_LINEAR, HRW_MEM_DEVICE, HRW_MEM_HOST, HRW_NUMERICS_FAST,
                   HRW_NUMERICS_MIXED, HRW_NUMERICS_STRICT, HRW_OK, HRW_PROBLEM_FV1D, HRW_PROBLEM_FV2D,
                   HRW_PROBLEM_LINEAR_ODE, HrwError, lib)
from .adjoint import adjoint  # noqa: F401
from .batch import batch  # noqa: F401
from .problems import Problem, burgers_1d, linear_ode, pbe_2d  # noqa: F401
from .tvdode import mstvd, rktvd  # noqa: F401
from .weno import weno  # noqa: F401


def weno_solve(*args, **kwargs):
    """Differentiable u(T) = weno_solve(u0, problem, dt, nsteps) for PyTorch (torch_op)."""
    from .torch_op import weno_solve as _ws
    return _ws(*args, **kwargs)
