"""The reference driver's file formats (driver_files.py) against the
reference's own example files (tests/golden/io, copied by
tests/golden/make_fixtures.py): control_file.dat, initial_config.dat and
the first records of an output.VTF trajectory.  No GPU needed."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
IO = os.path.join(ROOT, "tests", "golden", "io")


@pytest.fixture(scope="module")
def df():
    spec = importlib.util.spec_from_file_location(
        "rsd_driver_files", os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "driver_files.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_list_directed_values(df):
    assert df.read_values("3*0.0 1.d0, .TRUE. t F ! note", "rrrrlll") == [0.0, 0.0, 0.0, 1.0, True, True, False]
    assert df.read_values("false 7", "li") == [False, 7]
    with pytest.raises(df.FormatError):
        df.read_values("1.0", "rr")
    with pytest.raises(df.FormatError):
        df.read_values("maybe", "l")


def test_control_file_of_the_example(df):
    c = df.read_control(os.path.join(IO, "control_file.dat"))
    assert len(c) == len(df.CONTROL) and "kBT" not in c
    assert c["correction_method"] == 0 and c["FTS_method"] is False and c["useGMRESmethod"] is True
    assert c["IsCaseLattice"] == 0 and c["timestep"] == 5000 and c["NUM_THREADS"] == 6
    assert c["radii_test"] == 1.0 and c["radii_true"] == 1e-4 and c["g_gravity"] == 9.8
    assert c["u_bg"] == [0.0] * 3 and c["omega_bg"] == [0.0] * 3 and c["EI_bg"] == [0.0] * 6
    assert c["mu_f"] == 1e-3 and c["pho_f"] == 1000.0 and c["LINERR"] == 1e-4
    assert c["T0"] == 0.0 and c["END_TIME"] == 10.0 and c["BASE_DT"] == 5e-3 and c["K_WRITE"] == 2
    assert c["Permittivity"] == 7.2e-10 and c["Surfaceenergy"] == 4.7e-3 and c["BROWN"] is False


def test_control_file_reads_kbt_when_brownian(df, tmp_path):
    src = open(os.path.join(IO, "control_file.dat")).read()
    assert ".false.                  ! BROWN" in src
    p = tmp_path / "control_file.dat"
    p.write_text(src.replace(".false.                  ! BROWN", ".true.                   ! BROWN"))
    c = df.read_control(str(p))
    assert c["BROWN"] is True and c["kBT"] == 1e-17


def test_initial_config_of_the_example(df):
    d = df.read_initial_config(os.path.join(IO, "initial_config.dat"))
    assert (d["NX"], d["NY"], d["NZ"], d["Np"]) == (2, 2, 2, 100)
    assert (d["K_rb"], d["Nswimer"], d["rb_counts"], d["F_rb"], d["Nfilament"]) == (1, 100, [100], 0, 0)
    assert d["LB"] == [4.64] * 3 and d["hot_start"] is False and d["U_pos"] is None
    assert len(d["conf"]) == 100 and d["conf"][1] == [2.01, 0.0, 0.0] and d["radii"][:2] == [1.0, 1.0]


def test_vtf_records_of_the_example_reformat_exactly(df):
    path = os.path.join(IO, "output_head.VTF")
    lines = [line.rstrip("\n") for line in open(path) if line.strip()]
    rows = df.read_vtf(path)
    assert len(rows) == len(lines) == 40
    for line, r in zip(lines, rows):
        assert df.vtf_record(r[0], r[1:4], r[4], r[5:8]) == line


@pytest.mark.parametrize("hot", [False, True])
def test_initial_config_round_trip(df, tmp_path, hot):
    conf = [[0.1, -2.0, 3.25], [1e-7, 4.5, 0.0]]
    radii = [1.0, 0.6]
    U = [0.5, -0.25, 1e-9, 0.0, 2.0, -3.0] if hot else None
    p = str(tmp_path / "initial_config.dat")
    df.write_initial_config(p, conf, radii, [9.5, 9.5, 9.5], T=0.75, U_pos=U)
    d = df.read_initial_config(p)
    assert d["Np"] == 2 and d["hot_start"] is hot and d["LB"] == [9.5] * 3
    assert d["conf"] == conf and d["radii"] == radii and d["T"] == [0.75, 0.75] and d["U_pos"] == U


def test_fortran_es_and_e_formats(df):
    assert df.fortran_es(1.0) == "   1.000000000000000E+00"
    assert df.fortran_es(-2.5e-7) == "  -2.500000000000000E-07"
    assert df.fortran_es(3e150) == "   3.000000000000000+150"
    assert df.fortran_e(0.0) == "  0.000000000000000E+000"
    assert df.fortran_e(-2.01) == " -0.201000000000000E+001"
    assert df.fortran_e(5e-5) == "  0.500000000000000E-004"
    rec = df.yeta_record(0.5, [1, 2, 3, 4, 5], 25.79, 0.0, 1.0, 0.0)
    assert len(rec) == 10 * 24 and rec.startswith("   5.000000000000000E-01")
