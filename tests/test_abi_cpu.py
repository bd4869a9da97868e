"""The C-ABI library loads and exports every entry point the header declares; validation
mirrors the reference's constructors.  No compute call runs here (CPU only)."""
import ctypes as C
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


def _header_problem_fields():
    """(name, count) of struct hrw_problem in include/hrweno_gpu.h, in order."""
    import re
    text = (ROOT / "include" / "hrweno_gpu.h").read_text()
    body = text[text.index("typedef struct hrw_problem {"):text.index("} hrw_problem;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for m in re.finditer(r"([A-Za-z_][\w ]*?[\s*]+)(\w+)(?:\[(\d+)\])?;", body.split("{", 1)[1]):
        fields.append((m.group(2), int(m.group(3) or 1)))
    return fields


def test_problem_layouts_agree():
    """struct hrw_problem, its ctypes mirror and the Fortran bind(c) type of the binding module
    (hr-weno_gb300/fortran/hrweno_gpu.F90) list the same fields in the same order (a missing
    field shifts every later one)."""
    import re
    import ctypes as C
    from hrweno import _abi
    hdr = _header_problem_fields()
    cty = [(name, getattr(t, "_length_", 1)) for name, t in _abi.HrwProblem._fields_]
    assert hdr == cty, (hdr, cty)
    text = (ROOT / "hr-weno_gb300" / "fortran" / "hrweno_gpu.F90").read_text()
    block = text[text.index("type, bind(c) :: hrw_problem"):]
    block = block[:block.index("end type")]
    fort = []
    for line in block.splitlines()[1:]:
        decl = line.split("::", 1)[1] if "::" in line else ""
        for item in re.finditer(r"(\w+)(?:\((\d+)\))?", decl):
            fort.append((item.group(1), int(item.group(2) or 1)))
    assert fort == hdr, (fort, hdr)


def test_problem_offsets_match_c_compiler(tmp_path):
    """Offsets and size of struct hrw_problem as the C compiler lays it out, against ctypes."""
    import shutil
    import subprocess
    from hrweno import _abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = [n for n, _ in _abi.HrwProblem._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "hrweno_gpu.h"\nint main(void) {\n'
                   + "".join(f'  printf("%zu\\n", offsetof(hrw_problem, {n}));\n' for n in names)
                   + '  printf("%zu\\n", sizeof(hrw_problem));\n  return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = [getattr(_abi.HrwProblem, n).offset for n in names] + [C.sizeof(_abi.HrwProblem)]
    assert got == want, (got, want)


def test_f32c_rejects_burgers_linear(hw):
    from hrweno import HrwError
    prob = hw.Problem(kind="fv1d", ncells=(100, 1), fn=("burgers_linear", "burgers_linear"),
                      coef_a=(0.5, 0.0), xmin=(-1.0, 0.0), xmax=(1.0, 1.0))
    with pytest.raises(HrwError, match=r"HRW_F32C supports BURGERS and LINEAR"):
        hw.rktvd(prob, 100, 3, dtype="f32c")


def test_batch_edges_are_checked(hw):
    """A batch's non-uniform lines (FP64 or compensated FP32) need increasing edges; the check
    names the problem and runs before any CUDA call."""
    from hrweno import HrwError
    nx = 16
    xe = np.linspace(0.0, 1.0, nx + 1) ** 2
    xe[5] = xe[4]
    probs = [hw.Problem(kind="fv1d", ncells=(nx, 1), k=3), hw.Problem(kind="fv1d", ncells=(nx, 1), k=3, xedges=(xe, None))]
    for dtype in ("f64", "f32c"):
        with pytest.raises(HrwError, match="edges must increase.*problem 1"):
            hw.batch(probs, dtype=dtype)


def test_real32_validation_before_any_cuda_call(hw):
    """A REAL32 handle (dtype "f32") applies the reference's checks to the FP32 values a REAL32
    build holds: eps > epsilon(1.0_real32) (src/hrweno_weno.f90:92) and a grid that stays valid
    once rounded to FP32.  Validation runs before any CUDA call, so this needs no GPU."""
    from hrweno import HrwError
    ok = hw.burgers_1d(100, eps=1e-6)
    tiny_eps = hw.burgers_1d(100, eps=1e-8)  # valid in REAL64
    with pytest.raises(HrwError, match=r"Invalid input 'eps'. Valid range: eps > epsilon."):
        hw.rktvd(tiny_eps, 100, 3, dtype="f32")
    with pytest.raises(HrwError, match=r"Invalid input 'eps'. Valid range: eps > epsilon."):
        hw.mstvd(tiny_eps, 100, dtype="f32")
    # edges 1e-9 apart around 1 are distinct doubles but one FP32 value
    xe = 1.0 + 1e-9 * np.arange(11)
    collapsed = hw.Problem(kind="fv1d", ncells=(10, 1), xedges=(xe, None))
    with pytest.raises(HrwError, match=r"edges must increase in REAL32"):
        hw.rktvd(collapsed, 10, 3, dtype="f32")
    narrow = hw.Problem(kind="fv1d", ncells=(10, 1), xmin=(1.0, 0.0), xmax=(1.0 + 1e-9, 1.0))
    with pytest.raises(HrwError, match=r"xmax > xmin must hold in REAL32"):
        hw.rktvd(narrow, 10, 3, dtype="f32")
    thin = hw.burgers_1d(10, width=np.full(10, 1e-50))
    with pytest.raises(HrwError, match=r"widths must be > 0 in REAL32"):
        hw.rktvd(thin, 10, 3, dtype="f32")
    assert ok.eps == 1e-6


def test_last_error_is_per_thread(hw):
    """hrw_last_error() holds the message of the last failing call on the calling thread: an
    error on one thread neither shows on nor overwrites another's (validation fails before
    any CUDA call, so this runs without a GPU)."""
    import threading
    from hrweno import _abi as A
    L = A.lib()
    h = C.c_void_p()
    assert L.hrw_weno_create(0, 3, 1e-6, None, C.byref(h)) == A.HRW_EINVAL
    mine = L.hrw_last_error().decode()
    seen = {}

    def other():
        seen["before"] = L.hrw_last_error().decode()
        hh = C.c_void_p()
        seen["rc"] = L.hrw_weno_create(10, 4, 1e-6, None, C.byref(hh))
        seen["after"] = L.hrw_last_error().decode()

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen == {"before": "", "rc": A.HRW_EINVAL,
                    "after": "Invalid input 'k'. Valid range: 1 <= k <= 3."}
    assert L.hrw_last_error().decode() == mine == "Invalid input 'ncells'. Valid range: ncells > 0."


def test_rhs_rejects_null_arrays(hw):
    """hrw_rhs takes device arrays; a null one returns HRW_EINVAL before any CUDA call."""
    from hrweno import _abi as A
    cp = hw.burgers_1d(16).to_c()
    rc = A.lib().hrw_rhs(C.byref(cp), A.HRW_F64, 0.0, None, None, None)
    assert rc == A.HRW_EINVAL and A.lib().hrw_last_error().decode() == "Invalid input: null pointer."


def test_adjoint_and_batch_validation_messages(hw):
    """The adjoint and batch constructors validate before any CUDA call."""
    from hrweno import HrwError
    p = hw.burgers_1d(16, xmin=1.0, xmax=1.0)
    with pytest.raises(HrwError, match=r"Valid range: xmax > xmin"):
        hw.adjoint(p)
    with pytest.raises(HrwError, match=r"Valid range: xmax > xmin. \(problem 1\)"):
        hw.batch([hw.burgers_1d(16), p])
    with pytest.raises(HrwError, match=r"global Lax-Friedrichs"):
        hw.adjoint(hw.burgers_1d(16, flux="godunov"))
    with pytest.raises(HrwError, match=r"with nseg > 1, ncells must be a multiple of 8"):
        hw.adjoint(hw.burgers_1d(12), nseg=2)
    with pytest.raises(HrwError, match=r"batches take non-uniform lines as xedges"):
        hw.batch([hw.burgers_1d(10, width=np.full(10, 0.1))])


def test_headers_compile_strictly_and_example_links(hw, tmp_path):
    """The public headers are plain C99/C11 and C++17 under -pedantic -Wall -Wextra -Werror, and
    the C caller (tests/c/abi_example.c) links against the library.  A C++ program calls
    hrw_problem_init, which touches no CUDA state, so this runs without a GPU."""
    import shutil
    import subprocess
    from hrweno import _abi
    cc, cxx = shutil.which("gcc") or shutil.which("cc"), shutil.which("g++") or shutil.which("c++")
    if cc is None or cxx is None:
        pytest.skip("no C/C++ compiler")
    lib = Path(_abi.LIB_PATH)
    link = ["-L", str(lib.parent), "-l" + lib.stem[3:], "-Wl,-rpath," + str(lib.parent)]
    strict = ["-pedantic", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include")]
    for std in ("c99", "c11"):
        subprocess.run([cc, "-std=" + std, *strict, str(ROOT / "tests" / "c" / "abi_example.c"),
                        "-o", str(tmp_path / ("abi_" + std)), *link, "-lm"], check=True)
    src = tmp_path / "headers.cpp"
    src.write_text('#include "hrweno_gpu.h"\n#include "hrweno_diag.h"\n'
                   "int main() {\n  hrw_problem p;\n  hrw_problem_init(&p);\n"
                   "  return p.kind == HRW_PROBLEM_FV1D && p.k == 3 && p.xedges[0] == nullptr ? 0 : 1;\n}\n")
    exe = tmp_path / "headers"
    subprocess.run([cxx, "-std=c++17", *strict, str(src), "-o", str(exe), *link], check=True)
    assert subprocess.run([str(exe)]).returncode == 0


def test_rhs_rejects_grids_beyond_the_int_range(hw):
    """A 2D grid of more than 2^31 - 1 cells is refused with a message (its cell count is formed
    in 64 bits, before any CUDA call), not wrapped around to a negative int."""
    from hrweno import _abi as A
    cp = hw.pbe_2d(50000, 50000).to_c()
    rc = A.lib().hrw_rhs(C.byref(cp), A.HRW_F64, 0.0, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == A.HRW_EINVAL
    assert A.lib().hrw_last_error().decode() == "Invalid input 'ncells': more than 2^31 - 1 cells."


def test_constants_agree_with_the_header():
    """Every enum constant of include/hrweno_gpu.h has the same value in the Python package."""
    import hrweno
    txt = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "hrweno_gpu.h").read_text(), flags=re.S)
    consts = {n: int(v) for n, v in re.findall(r"\b(HRW_[A-Z0-9_]+)\s*=\s*(\d+)", txt)}
    assert len(consts) >= 20
    for name, value in consts.items():
        assert getattr(hrweno, name) == value, name


def test_fortran_binding_names_exist():
    """Every C entry point the Fortran module binds (bind(c, name=...)) is declared in the
    header and exported by the library; the module keeps the reference's type names."""
    import re
    text = (ROOT / "hr-weno_gb300" / "fortran" / "hrweno_gpu.F90").read_text()
    hdr = (ROOT / "include" / "hrweno_gpu.h").read_text()
    names = re.findall(r'bind\(c,\s*name="(\w+)"\)', text)
    assert len(names) >= 10
    for n in names:
        assert re.search(rf"\b{n}\s*\(", hdr), n
    for t in ("weno", "rktvd", "mstvd"):
        assert re.search(rf"^\s*type(, extends\(\w+\))? :: {t}\s*$", text, flags=re.M), t
        assert re.search(rf"^\s*interface {t}\s*$", text, flags=re.M), t
    for m in ("reconstruct", "integrate"):
        assert re.search(rf"procedure :: {m} =>", text), m
