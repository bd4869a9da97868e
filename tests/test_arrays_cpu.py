"""Host-side array checks of the Python mirror (CPU only): every array a call hands to the
library is float64 where the library reads doubles, contiguous, of the right length, and all
arrays of one call live in one memory space.  These checks run before any library call."""
import numpy as np
import pytest


def test_describe_requires_float64_by_default(hw):
    import torch
    from hrweno._arrays import describe
    with pytest.raises(TypeError, match="float64"):
        describe(np.zeros(8, dtype=np.float32), 8, True)
    with pytest.raises(TypeError, match="float64"):
        describe(torch.zeros(8, dtype=torch.float32), 8, True)
    # reconstruct passes the element type on to the library, which checks it
    assert describe(np.zeros(8, dtype=np.float32), 8, True, f64_only=False)[2] == hw.HRW_F32
    assert describe(np.zeros(8), 8, True)[2] == hw.HRW_F64


def test_describe_shape_layout_and_access(hw):
    import torch
    from hrweno._arrays import describe
    with pytest.raises(ValueError, match="C-contiguous"):
        describe(np.zeros(16)[::2], 8, False)
    with pytest.raises(ValueError, match="expected 8"):
        describe(np.zeros(9), 8, False)
    ro = np.zeros(8)
    ro.flags.writeable = False
    assert describe(ro, 8, False)[1] == ro.ctypes.data
    with pytest.raises(ValueError, match="read-only"):
        describe(ro, 8, True)
    with pytest.raises(ValueError, match="contiguous"):
        describe(torch.zeros(16, dtype=torch.float64)[::2], 8, False)
    with pytest.raises(TypeError, match="unsupported"):
        describe([0.0] * 8, 8, False)
    from hrweno import _abi as A
    t = torch.zeros(8, dtype=torch.float64)  # a CPU tensor is host memory
    assert describe(t, 8, False) == (A.HRW_MEM_HOST, t.data_ptr(), A.HRW_F64)


def test_same_space():
    from hrweno import _abi as A
    from hrweno._arrays import same_space
    assert same_space(A.HRW_MEM_DEVICE, A.HRW_MEM_DEVICE) == A.HRW_MEM_DEVICE
    with pytest.raises(ValueError, match="all be host arrays or all CUDA tensors"):
        same_space(A.HRW_MEM_DEVICE, A.HRW_MEM_HOST, A.HRW_MEM_DEVICE)


def test_integrate_rejects_float32_before_the_library(hw):
    """A float32 state of neq elements would be read as neq doubles: integrate refuses it."""
    ode = object.__new__(hw.rktvd)
    ode._h, ode.neq = None, 8
    with pytest.raises(TypeError, match="float64"):
        ode.integrate(np.zeros(8, dtype=np.float32), 0.0, 1.0, 0.1)
    ode.dtype = "f32"  # a REAL32 integrator takes float32 only
    with pytest.raises(TypeError, match="float32"):
        ode.integrate(np.zeros(8), 0.0, 1.0, 0.1)
    b = object.__new__(hw.batch)
    b._h, b.offsets, b.nprob = None, np.array([0, 8]), 1
    with pytest.raises(TypeError, match="float64"):
        b.advance(np.zeros(8, dtype=np.float32), np.zeros(1), np.ones(1), 1)
    a = object.__new__(hw.adjoint)
    a._h, a.size, a.nseg = None, 8, 1
    with pytest.raises(TypeError, match="float64"):
        a.forward(np.zeros(8, dtype=np.float32), None, 0.1, 1)


def test_batch_times_are_checked(hw):
    """t is updated in place and dt read per problem: both must hold one value per problem."""
    b = object.__new__(hw.batch)
    b._h, b.offsets, b.nprob = None, np.array([0, 64, 128]), 2
    u = np.zeros(128)
    for t, dt in (([0.0, 0.0], np.ones(2)),            # t not an array
                  (np.zeros(3), np.ones(2)),           # t too long
                  (np.zeros(2, dtype=np.float32), np.ones(2)),
                  (np.zeros(4)[::2], np.ones(2)),      # t not contiguous
                  (np.zeros(2), np.ones(1))):          # dt too short
        with pytest.raises(ValueError):
            b.advance(u, t, dt, 1)
        with pytest.raises(ValueError):
            b.integrate(u, t, 1.0, dt)
    with pytest.raises(ValueError, match="dt must hold 2"):
        b.tune(u, np.ones(3))


def test_problem_grid_arrays_are_checked(hw):
    """The library reads ncells widths and ncells + 1 edges from the descriptor's host arrays."""
    from hrweno import HrwError
    hw.burgers_1d(10, width=np.full(10, 0.1)).to_c()
    with pytest.raises(HrwError, match="size\\(width\\) /= ncells"):
        hw.burgers_1d(10, width=np.full(9, 0.1)).to_c()
    hw.Problem(ncells=(10, 1), xedges=(np.linspace(0, 1, 11), None)).to_c()
    with pytest.raises(HrwError, match="size\\(xedges\\) /= ncells \\+ 1"):
        hw.Problem(ncells=(10, 1), xedges=(np.linspace(0, 1, 10), None)).to_c()
