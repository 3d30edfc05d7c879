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


def _read_whitespace_table(path):
    """The reference's readers (pyscripts/imodel_data.py:50-52,
    imodel_data_evol.py:47-53) load these files with pandas.read_csv(
    delim_whitespace=True): the first line names the columns, every other
    line holds one whitespace-separated value per column.  Restated here
    (pandas is not a dependency)."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    head = lines[0].split()
    rows = [ln.split() for ln in lines[1:]]
    for r in rows:
        assert len(r) == len(head), (path, len(r), len(head))
    return {name: [r[i] for r in rows] for i, name in enumerate(head)}


def test_outputs_parse_with_the_reference_readers_columns(tmp_path, grid_at):
    """Every column the reference's plotting options select
    (tests/golden/pyscripts_columns.json, from pyscripts/options_*.csv)
    exists in the written files and its values parse."""
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                       "pyscripts_columns.json")))
    g = grid_at(2)
    for k, ntime in ((1, 960), (2, 1920)):
        output.write_errors(str(tmp_path), g, 2, ntime, 450.0, ntime * 450.0, 1e-3 * k, 2e-4,
                            3e-3, 4e-4, 1e-15, 1e-9, -2e-8, 3e-10)
    t = _read_whitespace_table(os.path.join(str(tmp_path), "swm_errors.txt"))
    for name in gold["options_swm_conv.csv"] + gold["options_template.csv"]:
        assert name in t, name
    assert [int(v) for v in t["Mesh"]] == [g.nv, g.nv]
    assert [int(v) for v in t["nTime"]] == [960, 1920]
    np.testing.assert_allclose([float(v) for v in t["MaxError_h"]], [1e-3, 2e-3], rtol=1e-9)
    np.testing.assert_allclose([float(v) for v in t["TimeDays"]], [5.0, 10.0], rtol=1e-9)
    assert t["Methods"][0] == output.swmname(2, 450.0) and t["Grid"][0] == g.name

    e = {"errormaxrel_h": 1.5e-3, "error2_h": 2.5e-4, "errormaxrel_u": 3.5e-3, "error2_u": 4.5e-4}
    p = str(tmp_path / "evol.txt")
    f = output.open_with_header(p, output._EVOL_ERR_HEAD)
    for k in (0, 96, 192):
        f.write(output.evolution_error_line(g, 2, k, 192, 450.0, 0.1, k * 450.0, e, 1e-15,
                                            1e-9, 2e-9, 3e-9, 4e-9, 1e-7, 2e-7, 0.0) + "\n")
    f.close()
    t = _read_whitespace_table(p)
    for name in gold["options_template_evol.csv"]:
        assert name in t, name
    np.testing.assert_allclose([float(v) for v in t["TimeDays"]], [0.0, 0.5, 1.0], atol=1e-12)
    np.testing.assert_allclose([float(v) for v in t["error2_h"]], [2.5e-4] * 3, rtol=1e-9)

    p = str(tmp_path / "me.txt")
    f = output.open_with_header(p, output._EVOL_HEAD)
    f.write(output.mass_energy_line(g, 2, 96, 192, 450.0, 0.1, 43200.0, 1e-15, 1e-9, 2e-9,
                                    3e-9, 4e-9, 1e-7) + "\n")
    f.close()
    t = _read_whitespace_table(p)
    assert float(t["time(dys)"][0]) == 0.5 and float(t["Tenergy"][0]) == 3e-9
