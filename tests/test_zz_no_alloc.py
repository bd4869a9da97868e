"""hrw_rktvd3_steps_noalloc: RK3 steps whose stage arrays live in a fixed buffer inside the
library, for callers that cannot allocate device memory (a framework whose caching allocator
owns the device, or a step loop that must avoid cudaMalloc's implicit synchronisation).

The entry point is called through the C ABI and checked against the handle-based path
(hrw_rktvd_create + hrw_integrate on device memory) on two calls in a row: it launches the
same kernels in the same order, so the results must agree bit for bit (tolerance 0).  The
file sorts last so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from hrweno import _abi as A
    L = A.lib()
    L.hrw_rktvd3_steps_noalloc.argtypes = [C.POINTER(A.HrwProblem), C.c_void_p, C.c_double,
                                           C.c_int, C.c_void_p]
    L.hrw_rktvd3_steps_noalloc.restype = C.c_int
    return A, L


@pytest.mark.parametrize("numerics", ["strict", "fast"])
@pytest.mark.parametrize("nc,k", [(500, 3), (4099, 2), (1 << 20, 3)])
def test_noalloc_matches_handle_path(hw, numerics, nc, k):
    import torch
    from hrweno import workloads
    A, L = _lib()
    prob, u0, dt = workloads.large_burgers(nc, k=k, numerics=numerics)
    cp = prob.to_c()

    ref = torch.from_numpy(u0.copy()).cuda()
    ode = hw.rktvd(prob, nc, 3)
    got = torch.from_numpy(u0.copy()).cuda()
    t = 0.0
    for nsteps in (3, 4):  # two calls in a row; the second reuses the buffer's old contents
        t = ode.integrate(ref, t, t + (nsteps - 0.5) * dt, dt)
        A.check(L.hrw_rktvd3_steps_noalloc(C.byref(cp), got.data_ptr(), dt, nsteps, None))
        torch.cuda.synchronize()
        assert torch.equal(got, ref), (numerics, nc, k, nsteps)


def test_noalloc_rejects_oversize_and_nonuniform(hw):
    import torch
    from hrweno import workloads
    A, L = _lib()
    n = (1 << 20) + 1
    prob, _, dt = workloads.large_burgers(n, k=3, u0=np.ones(n))
    u = torch.ones(n, dtype=torch.float64, device="cuda")
    rc = L.hrw_rktvd3_steps_noalloc(C.byref(prob.to_c()), u.data_ptr(), dt, 1, None)
    assert rc == A.HRW_EINVAL
    assert "HRW_NOALLOC_MAX_CELLS" in L.hrw_last_error().decode()
    prob, _, dt = workloads.large_burgers(64, k=3, u0=np.ones(64))
    prob.width = (np.full(64, 10.0 / 64), None)
    rc = L.hrw_rktvd3_steps_noalloc(C.byref(prob.to_c()), u.data_ptr(), dt, 1, None)
    assert rc == A.HRW_EINVAL and "uniform" in L.hrw_last_error().decode()
    assert torch.equal(u, torch.ones_like(u))  # nothing ran
