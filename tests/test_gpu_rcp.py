"""The FAST path's reciprocal (an rcp.approx.f64 seed and one cubic Newton-Raphson step,
rcp_fast in hr-weno_gb300/csrc/hrw_device.cuh) against IEEE division on the device.

Bound: at most 1 ulp from the correctly rounded 1/x over x in [2^-1000, 2^1000], the range
the FAST weights keep their denominators in."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulp_distance(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def test_rcp_fast_within_one_ulp(hw):
    import torch
    from hrweno import _abi as A
    L = A.lib()
    L.hrw_diag_rcp.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.hrw_diag_rcp.restype = C.c_int
    rng = np.random.default_rng(7)
    n = 1 << 22
    e = rng.uniform(-1000.0, 1000.0, n)
    x = np.exp2(e) * rng.uniform(1.0, 2.0, n) / 2.0
    # the range ends, powers of two and their neighbours, and mantissas near 1 and 2
    edge = [2.0 ** -1000, 2.0 ** 1000, 1.0, np.nextafter(1.0, 2.0), np.nextafter(2.0, 1.0), 3.0, 1.5,
            2.0 ** -999 * 1.9999999999999998, 2.0 ** 999 * 1.0000000000000002]
    x = np.concatenate([np.array(edge), x])
    x = x[(x >= 2.0 ** -1000) & (x <= 2.0 ** 1000)]
    xd = torch.from_numpy(x).cuda()
    fast = torch.empty_like(xd)
    exact = torch.empty_like(xd)
    assert L.hrw_diag_rcp(xd.data_ptr(), fast.data_ptr(), exact.data_ptr(), xd.numel()) == 0
    f, q = fast.cpu().numpy(), exact.cpu().numpy()
    assert np.array_equal(q, 1.0 / x)  # the device's IEEE division is the correctly rounded 1/x
    d = ulp_distance(f, q)
    assert int(d.max()) <= 1, (int(d.max()), x[np.argmax(d)])
    # report how often the fast reciprocal is not the correctly rounded one
    print(f"rcp_fast: {np.count_nonzero(d)} of {d.size} results 1 ulp off, max {int(d.max())} ulp")
