"""integrate on host arrays: pageable arrays are copied in and out; page-locked lines of at least
2 x 152 x 1024 cells (rktvd order 3, FP64) overlap the copies with the first and last stages
by chunks.  Every path gives the bits of the device-array path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("numerics", ["fast", "strict"])
@pytest.mark.parametrize("n", [5000, 1 << 16, 1 << 19, (1 << 19) + 777])
@pytest.mark.parametrize("itask", [1, 2])
def test_host_arrays_match_device(hw, numerics, n, itask):
    import torch
    from hrweno import workloads
    prob, u0, dt = workloads.large_burgers(n, k=3, numerics=numerics)
    results = {}
    for kind in ("device", "pageable", "pinned"):
        if kind == "device":
            u = torch.from_numpy(u0.copy()).cuda()
        elif kind == "pageable":
            u = u0.copy()
        else:
            u = torch.from_numpy(u0.copy()).pin_memory()
        ode = hw.rktvd(prob, n, 3)
        t = 0.0
        for _ in range(5 if itask == 2 else 1):
            t = ode.integrate(u, t, t + (7.5 if itask == 1 else 0.5) * dt, dt, itask=itask)
        results[kind] = (t, u.cpu().numpy() if hasattr(u, "cpu") else u)
    for kind in ("pageable", "pinned"):
        assert results[kind][0] == results["device"][0]
        assert np.array_equal(results[kind][1], results["device"][1]), kind


def test_pinned_host_mstvd_and_f32c(hw):
    """mstvd and the compensated form on a page-locked host array (these copy in and out)."""
    import torch
    from hrweno import workloads
    n = 4096
    prob, u0, dt = workloads.large_burgers(n, k=3)
    for make in (lambda: hw.mstvd(prob, n), lambda: hw.rktvd(prob, n, 3, dtype="f32c")):
        a = torch.from_numpy(u0.copy()).cuda()
        b = torch.from_numpy(u0.copy()).pin_memory()
        ta = make().integrate(a, 0.0, 9.5 * dt, dt)
        tb = make().integrate(b, 0.0, 9.5 * dt, dt)
        assert ta == tb and np.array_equal(a.cpu().numpy(), b.numpy())
