"""Fortran-formatted outputs of swm_tests (no GPU needed for the writers)."""
import numpy as np

from imodel_gb300 import output


def test_fortran_e_format():
    assert output.fortran_e(1.0, 20, 10) == "    0.1000000000E+01"
    assert output.fortran_e(-0.00123456789012, 20, 10) == "   -0.1234567890E-02"
    assert output.fortran_e(0.0, 20, 10) == "    0.0000000000E+00"
    assert output.fortran_e(9.99999999999, 20, 10) == "    0.1000000000E+02"
    assert output.fortran_e(1.5e-150, 20, 10) == "    0.1500000000-149"
    assert len(output.fortran_e(123.456, 28, 16)) == 28


def test_errors_line_layout(tmp_path, grid_at):
    g = grid_at(2)
    p = output.write_errors(str(tmp_path), g, 2, 960, 450.0, 432000.0, 1e-3, 2e-4, 3e-3, 4e-4,
                            1e-15, 1e-9, -2e-8, 3e-10)
    lines = open(p).read().splitlines()
    assert lines[0].startswith("       Mesh  TCase    nTime")
    line = lines[1]
    assert len(line) == 12 + 4 + 10 + 11 * 20 + 120
    assert int(line[:12]) == g.nv and int(line[12:16]) == 2 and int(line[16:26]) == 960
    vals = [float(line[26 + 20 * i: 46 + 20 * i]) for i in range(11)]
    np.testing.assert_allclose(vals[:3], [450.0, 5.0, 1e-3], rtol=1e-10)
    assert line.rstrip().endswith("swm_tc2_dt450_HTC_trsk10_areageo icos_eqs_nopt_2")


def test_field_dump_roundtrip(tmp_path, grid_at):
    g = grid_at(3)
    vals = np.arange(g.nv, dtype=np.float64)
    p = output.field_dump(str(tmp_path / "h.dat"), g, vals, nlat=36, nlon=72)
    a = np.fromfile(p, dtype=np.float32).reshape(-1, 3)
    assert a.shape == (36 * 72, 3)
    assert a[:, 0].min() > -180 and a[:, 1].max() < 90
    assert set(np.unique(a[:, 2])).issubset(set(vals.astype(np.float32)))
