"""The reference's example driver on the GPU path: its output files match the same driver run
with the oracle (STRICT numerics: every value bit-identical, so every formatted digit too)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_example1_files_match_oracle(hw, orc, tmp_path):
    from hrweno import examples
    from hrweno.output import u_header, u_record, write_grid
    from hrweno.workloads import centres
    t, u = examples.example1(tmp_path / "gpu", numerics="strict")
    nc = 500
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="godunov", alpha=1.0, bc="copy",
                         numerics="strict")
    x = centres(nc, -5.0, 5.0)
    o = orc.ODE(prob, nc, 0, 3)
    uo = np.exp(-x ** 2)
    to = 0.0
    lines = [u_header(nc)]
    for ii in range(101):
        to = o.integrate(uo, to, 12.0 * ii / 100, 1e-2)
        lines.append(u_record(to, uo))
    (tmp_path / "ref").mkdir()
    write_grid(tmp_path / "ref" / "x.txt", x, np.full(nc, 10.0 / nc))
    assert (tmp_path / "gpu" / "x.txt").read_text() == (tmp_path / "ref" / "x.txt").read_text()
    assert (tmp_path / "gpu" / "u.txt").read_text() == "\n".join(lines) + "\n"
    assert t == to and np.array_equal(u, uo)


def test_example2_runs(hw, tmp_path):
    from hrweno import examples
    t, u = examples.example2(tmp_path / "ex2")
    rows = (tmp_path / "ex2" / "u.txt").read_text().splitlines()
    assert len(rows) == 102 and abs(t - 5.0) < 6e-3
    assert all(len(r.split()) == 1 + 250 * 250 for r in rows)
    for d in (1, 2):
        assert len((tmp_path / "ex2" / f"x{d}.txt").read_text().splitlines()) == 251
    # the pulse moves with unit velocity along both axes; closed boundaries keep the mass
    # (zero boundary fluxes) until it reaches x = 10, after t = 7
    assert np.all(np.isfinite(u)) and u.max() < 1.1 and u.min() > -0.1
    dx = 10.0 / 250
    assert abs(u.sum() * dx * dx - 4.0) < 1e-9


def test_snapshot_writer_reports_a_failed_write(tmp_path):
    """A record the worker thread cannot write (here: its file was closed under it) is raised
    in the caller's next snapshot() or close(), instead of leaving snapshot() waiting forever
    for a slot."""
    import torch
    from hrweno.output import SnapshotWriter
    x = np.linspace(0.0, 1.0, 16)
    out = SnapshotWriter(tmp_path, [(x, np.full(16, 1.0 / 16))], depth=2)
    out._fh.close()
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="snapshot writer failed"):
        for k in range(8):
            out.snapshot(0.1 * k, u)
    out._work.put(None)  # stop the worker; close() would raise the same error again
    out._thread.join()
