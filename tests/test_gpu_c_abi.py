"""The C ABI called from C (tests/c/abi_example.c, compiled here with the system C compiler
against include/hrweno_gpu.h and the library): reconstruct and an rktvd(3) integration on host
arrays, bit-identical to the oracle in STRICT numerics, and an invalid input that returns a
status with the reference's message instead of aborting."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def run_example(tmp_path, numerics):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from hrweno import _abi
    lib = Path(_abi.LIB_PATH)
    exe = tmp_path / "abi_example"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(ROOT / "tests" / "c" / "abi_example.c"),
                    "-o", str(exe), "-L", str(lib.parent), "-l" + lib.stem[3:],
                    "-Wl,-rpath," + str(lib.parent), "-lm"], check=True)
    out = subprocess.run([str(exe), str(numerics)], check=True, capture_output=True, text=True).stdout
    lines = out.splitlines()
    head = lines[0].split()
    err = lines[1]
    blocks, cur = {}, None
    for ln in lines[2:]:
        if ln in ("vl", "vr", "u"):
            cur = ln
            blocks[cur] = []
        else:
            blocks[cur].append(float(ln))
    return head, err, {k: np.array(v) for k, v in blocks.items()}


@pytest.mark.parametrize("numerics", [1, 0])  # STRICT, FAST
def test_c_caller_matches_oracle(hw, orc, tmp_path, numerics):
    head, err, res = run_example(tmp_path, numerics)
    nc = 500
    x = -5.0 + 10.0 / nc * (np.arange(nc) + 0.5)
    v = np.where(np.abs(x) < 1.0, 1.0, 0.0)
    vl, vr = orc.reconstruct(v, 3, 1e-6)
    prob = hw.burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy",
                         numerics="strict" if numerics == 1 else "fast")
    u = np.exp(-x * x)
    o = orc.ODE(prob, nc, 0, 3)
    t = o.integrate(u, 0.0, 1.0, 1e-2)
    fevals, istate, nsteps = o.info()
    assert float(head[1]) == t and int(head[3]) == nsteps and int(head[5]) == fevals
    assert int(head[7]) == istate
    assert err.startswith("invalid_k 1 Invalid input 'k'. Valid range: 1 <= k <= 3.")
    if numerics == 1:
        assert np.array_equal(res["vl"], vl) and np.array_equal(res["vr"], vr)
        assert np.array_equal(res["u"], u)
    else:
        assert np.max(np.abs(res["vl"] - vl)) <= 1e-13 * np.max(np.abs(vl))
        assert np.max(np.abs(res["u"] - u)) <= 1e-12 * np.max(np.abs(u))
