"""The reader of the reference's text snapshot format '(7(1PE12.5,1X))' (wb_read_dat), on
files written here: no GPU is involved.  The writers (2D output_file of
2d/benchmark_2d_dg.f90:468-495, 1D output_file of benchmark_1d.f90:69-100) round-trip
through it in tests/test_gpu_io.py."""
import os

import numpy as np
import pytest


def f1pe12_5(v):
    """Fortran 1PE12.5 as the reference's compilers print it (E dropped for |exp| >= 100)."""
    s = "%.5E" % v
    mant, ex = s.split("E")
    e = int(ex)
    if abs(e) >= 100:
        s = mant + ("-" if e < 0 else "+") + "%03d" % abs(e)
    return "%12s" % s


def write_records(path, rows):
    with open(path, "w") as f:
        for r in rows:
            for k in range(0, len(r), 7):  # 7 values per line, the descriptor's repeat count
                f.write(" ".join(f1pe12_5(v) for v in r[k:k + 7]) + "\n")


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "initwo_sample.dat")


def test_reads_the_references_own_snapshot(wb):
    """Records of the reference's initwo.dat (its output_file, 150 x 150 cells): the reader
    gives what np.loadtxt -- the reader of the reference's post-processing -- gives."""
    got = wb.read_dat(GOLDEN, 6)
    np.testing.assert_array_equal(got, np.loadtxt(GOLDEN))
    assert got.shape[0] >= 150 and np.any(got < 0)


def test_format_reproduces_the_references_bytes():
    """The 1PE12.5 formatter (the model of the writers' format in these tests) re-creates
    every sampled record of the reference's snapshot byte for byte: right-justified
    12-column fields, one blank between them and none at the end of the record."""
    for ln in open(GOLDEN).read().splitlines():
        assert ln == " ".join(f1pe12_5(float(t)) for t in ln.split()), ln


def test_reads_what_the_format_writes(wb, tmp_path):
    rng = np.random.default_rng(1)
    rows = rng.standard_normal((40, 6)) * 10.0 ** rng.integers(-12, 12, (40, 6))
    rows[3, 2] = 0.0
    rows[5, 4] = -1.5e-120   # three-digit exponents: 1.50000-120
    rows[7, 1] = 2.25e+150
    p = tmp_path / "snap.dat"
    write_records(p, rows)
    assert "-1.50000-120" in open(p).read()
    got = wb.read_dat(str(p), 6)
    assert got.shape == rows.shape
    # 1PE12.5 keeps six significant digits
    np.testing.assert_allclose(got, rows, rtol=5e-6, atol=0)


def test_records_longer_than_seven_values_continue_on_the_next_line(wb, tmp_path):
    rows = np.arange(1, 3 * 9 + 1, dtype=float).reshape(3, 9) * 1.5
    p = tmp_path / "wide.dat"
    write_records(p, rows)
    assert len(open(p).read().splitlines()) == 6
    np.testing.assert_array_equal(wb.read_dat(str(p), 9), rows)


def test_nan_and_blank_lines(wb, tmp_path):
    p = tmp_path / "nan.dat"
    p.write_text("\n" + f1pe12_5(1.0) + "          NaN\n\n" + f1pe12_5(-2.0) + " " + f1pe12_5(3.0) + "\n")
    got = wb.read_dat(str(p), 2)
    assert got.shape == (2, 2) and np.isnan(got[0, 1])
    np.testing.assert_array_equal(got[1], [-2.0, 3.0])


@pytest.mark.parametrize("text,ncols", [
    (" 1.00000E+00  2.00000E+00 \n", 3),                 # a record cut short
    (" 1.00000E+00  2.00000E+00  3.00000E+00 \n", 2),    # two records on one line
    (" 1.00000E+00  abc \n", 2),                         # not a number
    (" 1.00000E+00  2.0000E+0x \n", 2),
])
def test_rejects_malformed_files(wb, tmp_path, text, ncols):
    p = tmp_path / "bad.dat"
    p.write_text(text)
    with pytest.raises(wb.WbError) as ei:
        wb.read_dat(str(p), ncols)
    assert ei.value.status == wb.WB_ERR_ARG


def test_capacity_and_missing_file(wb, tmp_path):
    import ctypes
    L = wb.lib()
    p = tmp_path / "three.dat"
    write_records(p, np.ones((3, 2)))
    out = np.zeros((2, 2))
    n = ctypes.c_int64()
    rc = L.wb_read_dat(str(p).encode(), 2, out.ctypes.data_as(ctypes.c_void_p), 2, ctypes.byref(n))
    assert rc == wb.WB_ERR_ARG and n.value == 2
    rc = L.wb_read_dat(str(tmp_path / "none.dat").encode(), 2, out.ctypes.data_as(ctypes.c_void_p),
                       2, ctypes.byref(n))
    assert rc == wb.WB_ERR_ARG
