"""The examples' output formats (example/example1_burgers_1d_fv.f90:153-177), on the CPU."""
import numpy as np

from hrweno.output import fortran_a, fortran_es, u_header, u_record, write_grid


def test_fortran_es_descriptors():
    assert fortran_es(1.0, 16, 5, 3) == "    1.00000E+000"
    assert fortran_es(-2.5e-300, 16, 5, 3) == "   -2.50000E-300"
    assert fortran_es(0.0, 16, 5, 3) == "    0.00000E+000"
    assert fortran_es(12.009999999999788, 16, 5, 3) == "    1.20100E+001"
    assert fortran_es(-4.99, 15, 5) == "   -4.99000E+00"
    assert fortran_es(1.5e-120, 15, 5) == "    1.50000-120"
    assert fortran_a("t", 16) == " " * 15 + "t"


def test_grid_and_records(tmp_path):
    x = np.array([-4.99, 4.99])
    write_grid(tmp_path / "x.txt", x, np.array([0.02, 0.02]))
    lines = (tmp_path / "x.txt").read_text().splitlines()
    assert lines[0] == "    i            x(i)           dx(i)"
    assert lines[1] == "    1    -4.99000E+00     2.00000E-02"
    # each record ends with the blank of the list-directed write that closes it
    assert u_header(2) == " " * 15 + "t" + " " + " " * 12 + "u(1)" + " " + " " * 12 + "u(2) "
    assert u_record(0.5, [1.0, -0.25]) == "    5.00000E-001     1.00000E+000    -2.50000E-001 "
