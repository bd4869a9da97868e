"""The 2D stage kernels' bounded wait for their TMA tile copies, driven to expiry.

A block that gives up waiting flags its handle, waits (with the default bound) for its copies to
land and leaves; the host then reports HRW_ETIMEOUT and puts the handle in the error state, as
the reference's integrate refuses to continue once istate < 1 (src/hrweno_tvdode.f90:22-28,
126,228,286-297).  The test sets the first wait's poll limit to 0 (no poll at all), so the
timeout path runs while every copy still arrives: nothing is left in flight.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N1 = N2 = 64  # rows of 64 doubles / floats: 16-byte row pitch, so every 2D kernel takes the TMA loader


def diag():
    from hrweno import _abi as A
    L = A.lib()
    L.hrw_diag_set_tile_wait_limit.argtypes = [C.c_int]
    L.hrw_diag_set_tile_wait_limit.restype = C.c_int
    return L


@pytest.fixture
def short_wait(hw):
    L = diag()
    assert L.hrw_diag_set_tile_wait_limit(0) == 0
    try:
        yield
    finally:
        assert L.hrw_diag_set_tile_wait_limit(-1) == 0


def pulse():
    x = (np.arange(N1) + 0.5) / N1
    y = (np.arange(N2) + 0.5) / N2
    X, Y = np.meshgrid(x, y)  # row j = x2 index: u((j-1)*nc1 + i)
    return np.exp(-((X - 0.3) ** 2 + (Y - 0.3) ** 2) / 0.01).reshape(-1)


@pytest.mark.parametrize("dtype", ["f64", "f32c", "f32"])
@pytest.mark.parametrize("method", ["rktvd", "mstvd"])
def test_integrate_times_out_and_refuses(hw, orc, short_wait, dtype, method):
    import torch
    from hrweno import _abi as A
    prob = hw.pbe_2d(N1, N2)
    dt = 0.3 / (1.5 * N1 + 0.5 * N2)
    ode = hw.rktvd(prob, N1 * N2, 3, dtype=dtype) if method == "rktvd" else hw.mstvd(prob, N1 * N2, dtype=dtype)
    u0 = pulse().astype(np.float32) if dtype == "f32" else pulse()
    ug = torch.from_numpy(u0).cuda()
    with pytest.raises(hw.HrwError) as e:
        ode.integrate(ug, 0.0, 2.5 * dt, dt)
    assert e.value.code == A.HRW_ETIMEOUT
    assert "bounded wait" in str(e.value)
    assert ode.istate == -1
    with pytest.raises(hw.HrwError) as e2:  # (src/hrweno_tvdode.f90:126): no further steps
        ode.integrate(ug, 0.0, 2.5 * dt, dt)
    assert e2.value.code == A.HRW_ESTATE


@pytest.mark.parametrize("dtype", ["f64", "f32c", "f32"])
def test_rhs_times_out(hw, short_wait, dtype):
    import torch
    from hrweno import _abi as A
    prob = hw.pbe_2d(N1, N2)
    v = torch.from_numpy(pulse().astype(np.float32) if dtype == "f32" else pulse()).cuda()
    out = torch.empty_like(v)
    cp = prob.to_c()
    code = {"f64": A.HRW_F64, "f32c": A.HRW_F32C, "f32": A.HRW_F32}[dtype]
    rc = A.lib().hrw_rhs(C.byref(cp), code, 0.0, v.data_ptr(), out.data_ptr(), None)
    assert rc == A.HRW_ETIMEOUT
    assert "bounded wait" in A.lib().hrw_last_error().decode()


def test_fresh_handle_after_restore(hw, orc):
    """With the default limit restored, a new handle runs and matches the oracle bit for bit
    (STRICT), and a handle that timed out does not affect it."""
    import torch
    L = diag()
    prob = hw.pbe_2d(N1, N2, numerics="strict")
    dt = 0.3 / (1.5 * N1 + 0.5 * N2)
    assert L.hrw_diag_set_tile_wait_limit(0) == 0
    try:
        bad = hw.rktvd(prob, N1 * N2, 3)
        with pytest.raises(hw.HrwError):
            bad.integrate(torch.from_numpy(pulse()).cuda(), 0.0, 2.5 * dt, dt)
    finally:
        assert L.hrw_diag_set_tile_wait_limit(-1) == 0
    ug = torch.from_numpy(pulse()).cuda()
    tg = hw.rktvd(prob, N1 * N2, 3).integrate(ug, 0.0, 2.5 * dt, dt)
    uo = pulse()
    to = orc.ODE(prob, N1 * N2, 0, 3).integrate(uo, 0.0, 2.5 * dt, dt)
    assert tg == to
    assert np.array_equal(ug.cpu().numpy(), uo)
    assert bad.istate == -1
