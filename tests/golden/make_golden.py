"""Write tests/golden/*.json.

kat_reference.json holds the reference's own constants and known answers, written out from
its source text (src/hrweno_weno.f90:11-21 tables; test/*.f90 parameters):
    python tests/golden/make_golden.py
oracle_config1.json holds oracle outputs of the 500-cell Burgers case at a few output times,
a regression pin for the GPU tests (regenerate with --oracle after a deliberate change).
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]


def kat():
    c = {
        "1": [[1.0], [1.0]],
        "2": [[3 / 2, -1 / 2], [1 / 2, 1 / 2], [-1 / 2, 3 / 2]],
        "3": [[11 / 6, -7 / 6, 1 / 3], [1 / 3, 5 / 6, -1 / 6], [-1 / 6, 5 / 6, 1 / 3],
              [1 / 3, -7 / 6, 11 / 6]],
    }
    d = {"1": [1.0], "2": [2 / 3, 1 / 3], "3": [0.3, 0.6, 0.1]}
    return {"c_tables": c, "d_tables": d,
            "source": "src/hrweno_weno.f90:11-21 (c(j,r) listed as [r+1][j])"}


def config1(times=(1.2, 3.0, 6.0, 12.0)):
    sys.path[:0] = [str(ROOT), str(ROOT / "hr-weno_gb300")]
    from oracle import oracle
    from hrweno.problems import burgers_1d
    nc = 500
    x = -5.0 + (10.0 / nc) * (np.arange(nc) + 0.5)
    prob = burgers_1d(nc, -5.0, 5.0, k=3, eps=1e-6, flux="lax_friedrichs", alpha=1.0, bc="copy")
    ode = oracle.ODE(prob, nc, method=0, order=3)
    u = np.exp(-x ** 2)
    # u0 is stored itself: libm exp() may differ in the last bit between machines
    out = {"nc": nc, "dt": 1e-2, "u0_desc": "exp(-x^2) at centres of [-5,5]",
           "u0": u.tolist(), "snapshots": []}
    t = 0.0
    for tout in times:
        t = ode.integrate(u, t, tout, 1e-2)
        out["snapshots"].append({"tout": tout, "t": t, "u": u.tolist()})
    return out


if __name__ == "__main__":
    (HERE / "kat_reference.json").write_text(json.dumps(kat(), indent=1))
    if "--oracle" in sys.argv:
        (HERE / "oracle_config1.json").write_text(json.dumps(config1()))
