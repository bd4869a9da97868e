"""The C-ABI library loads and exports every entry point the header declares; validation
mirrors the reference's constructors.  No compute call runs here (CPU only)."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(hrw_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_header(hw):
    import ctypes
    L = ctypes.CDLL(str(ROOT / "hr-weno_gb300" / "hrweno" / "_lib" / "libhrweno_gb300.so"))
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(L, s), s


def test_weno_validation_messages(hw):
    from hrweno import HrwError, weno
    with pytest.raises(HrwError, match=r"Invalid input 'ncells'. Valid range: ncells > 0."):
        weno(0)
    with pytest.raises(HrwError, match=r"Invalid input 'k'. Valid range: 1 <= k <= 3."):
        weno(10, k=4)
    with pytest.raises(HrwError, match=r"Invalid input 'eps'. Valid range: eps > epsilon."):
        weno(10, eps=1e-17)
    with pytest.raises(HrwError, match=r"size\(xedges\) /= ncells \+ 1"):
        weno(10, xedges=np.linspace(0, 1, 10))


def test_ode_validation_messages(hw):
    from hrweno import HrwError, burgers_1d, rktvd, mstvd
    p = burgers_1d(10)
    with pytest.raises(HrwError, match=r"Invalid input 'neq'. Valid range: neq >= 1."):
        rktvd(p, 0, 3)
    with pytest.raises(HrwError, match=r"Invalid input 'order' in 'rktvd'. Valid range: 1 <= k <= 3."):
        rktvd(p, 10, 4)
    with pytest.raises(HrwError, match=r"neq /= product of ncells"):
        mstvd(p, 11)
    bad = burgers_1d(10, k=5)
    with pytest.raises(HrwError, match=r"Invalid input 'k'"):
        rktvd(bad, 10, 3)
