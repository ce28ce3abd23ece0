"""Model parameters by record name (HPSim.get_db_model / set_db_model /
get_db_epics, hpsim_module.cpp:52-360; hpsim_gb300/dbloader.py): values read
as the database renders them as text, changes written to the database (its
triggers recompute the model columns) and handed to the beamline's elements.
A database with the reference's table layout and triggers of the same kind is
built here; where the reference tree is present its transport-line database
is changed in a copy.  Host only: no GPU."""
import math
import os
import shutil
import sqlite3

import pytest

from hpsim_gb300 import HPSim, dbloader, lattices as L

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DB = os.environ.get("HPS_REFERENCE_DB", os.path.join(HERE, "..", "..", "reference", "db"))

SCHEMA = """
create table linac (view_index INTEGER, name TEXT, model_type TEXT, model_index INTEGER);
create table epics_channel (id INTEGER, lcs_name TEXT, value REAL);
create table buncher (id INTEGER, name TEXT, view_index INTEGER, on_off INTEGER, phase_model REAL,
  phase_offset_cal REAL, voltage_model REAL, frequency_model REAL, aperture_model REAL, phase_channel INTEGER,
  model_index INTEGER);
create table drift (id INTEGER, name TEXT, view_index INTEGER, length_model REAL, aperture_model REAL,
  model_index INTEGER);
create table spch_comp (id INTEGER, name TEXT, view_index INTEGER, fraction_model REAL, model_index INTEGER);
create table caperture (id INTEGER, name TEXT, view_index INTEGER, aperture_model REAL, in_out_model INTEGER,
  model_index INTEGER);
create table raperture (id INTEGER, name TEXT, view_index INTEGER, aperture_xl_model REAL,
  aperture_xr_model REAL, aperture_yt_model REAL, aperture_yb_model REAL, in_out_model INTEGER,
  model_index INTEGER);
create table quad (id INTEGER, name TEXT, view_index INTEGER, gradient_model REAL, length_model REAL,
  aperture_model REAL, monitor INTEGER, model_index INTEGER);
create table rf_module (id INTEGER, name TEXT, cell_length_betalambda_design REAL, amplitude_scale_cal REAL,
  phase_offset_cal REAL);
create table rf_gap (id INTEGER, name TEXT, view_index INTEGER, module_id INTEGER, cell_id INTEGER,
  tank_id INTEGER, length_model REAL, frequency_model REAL, amplitude_model REAL, amplitude_design REAL,
  ref_phase_model REAL, beam_phase_shift_model REAL, energy_out_model REAL, beta_center_model REAL,
  dg_model REAL, t_model REAL, tp_model REAL, sp_model REAL, model_index INTEGER);
create table transit_time_factor (module_id INTEGER, tank_id INTEGER, beta_g REAL, beta_min REAL, ta0 REAL,
  ta1 REAL, ta2 REAL, ta3 REAL, ta4 REAL, ta5 REAL, sa1 REAL, sa2 REAL, sa3 REAL, sa4 REAL, sa5 REAL);
-- the model columns follow the calibration columns, as in the reference's databases
create trigger buncher_phase after update of phase_offset_cal on buncher begin
  update buncher set phase_model =
    radians(phase_offset_cal + (select value from epics_channel where epics_channel.id = buncher.phase_channel))
  where rowid = new.rowid; end;
create trigger module_amplitude after update of amplitude_scale_cal on rf_module begin
  update rf_gap set amplitude_model = amplitude_design * new.amplitude_scale_cal where module_id = new.id; end;
create trigger module_phase after update of phase_offset_cal on rf_module begin
  update rf_gap set beam_phase_shift_model = radians(new.phase_offset_cal) where module_id = new.id; end;
"""


def make_db(path):
    c = sqlite3.connect(path)
    c.executescript(SCHEMA)
    lin = [("B1", "buncher"), ("D1", "drift"), ("SC1", "spch_comp"), ("CA1", "caperture"), ("RA1", "raperture"),
           ("Q1", "quad"), ("G1", "dtl_gap"), ("Q2", "quad"), ("G2", "dtl_gap"), ("Q3", "quad")]
    for vi, (name, mt) in enumerate(lin):
        c.execute("insert into linac values (?, ?, ?, NULL)", (vi, name, mt))
    c.execute("insert into epics_channel values (7, 'TEST:PH1', 10.0)")
    c.execute("insert into buncher values (1, 'B1', 0, 1, 0.1, 0.0, 0.15, 201.25, 0.02, 7, NULL)")
    c.execute("insert into drift values (1, 'D1', 1, 0.1, 0.0, NULL)")
    c.execute("insert into spch_comp values (1, 'SC1', 2, 0.5, NULL)")
    c.execute("insert into caperture values (1, 'CA1', 3, 0.01, 1, NULL)")
    c.execute("insert into raperture values (1, 'RA1', 4, 0.01, 0.012, 0.013, 0.014, 1, NULL)")
    for vi, name in ((5, "Q1"), (7, "Q2"), (9, "Q3")):
        c.execute("insert into quad values (?, ?, ?, 40.0, 0.04, 0.0, 0, NULL)", (vi, name, vi))
    c.execute("insert into rf_module values (3, 'MOD1', 1.0, 1.0, 0.0)")
    for vi, name, cell in ((6, "G1", 1), (8, "G2", 2)):
        c.execute("insert into rf_gap values (?, ?, ?, 3, ?, 1, 0.06, 201.25, 2.5, 2.5, -0.45, 0.0, 0.8, 0.04, "
                  "0.0, 0.85, 0.0, 0.1, NULL)", (vi, name, vi, cell))
        c.execute("insert into transit_time_factor values (3, ?, 0.04, 0.01, 0.85, 0.4, -1.2, 0.5, 0, 0, 0.1, "
                  "-0.1, 0.3, 0, 0)", (cell,))
    c.commit()
    c.close()


@pytest.fixture()
def lattice(tmp_path):
    from hpsim_gb300 import build
    build.build()
    path = str(tmp_path / "lat.db")
    make_db(path)
    dbc = HPSim.DBConnection(path)
    return dbc, HPSim.BeamLine(dbc)


def param(bl, name, key):
    t, _, p = bl.element(bl.index(name))
    return p[L.param_index(t, key)]


def test_values_by_record_name(lattice):
    dbc, _ = lattice
    assert HPSim.get_db_model("SC1", "fraction_model", dbc) == "0.5"
    assert HPSim.get_db_model("B1", "voltage_model", dbc) == "0.15"
    assert HPSim.get_db_model("RA1", "in_out_model", dbc) == "1"
    assert HPSim.get_db_model("G2", "amplitude_model", dbc) == "2.5"
    assert HPSim.get_db_model("nope", "fraction_model", dbc) is None
    assert HPSim.get_db_model("SC1", "no_such_field", dbc) is None
    assert HPSim.get_db_epics("TEST:PH1", dbc) == "10.0"
    assert HPSim.get_db_epics("TEST:NONE", dbc) is None


def test_set_model_reaches_database_and_elements(lattice):
    dbc, bl = lattice
    HPSim.set_db_model("SC1", "fraction_model", "0.25", dbc, bl)
    assert HPSim.get_db_model("SC1", "fraction_model", dbc) == "0.25"
    assert param(bl, "SC1", "fraction") == 0.25
    # the trigger recomputes the phase from the offset and the channel value
    HPSim.set_db_model("B1", "phase_offset_cal", "-5", dbc, bl)
    assert param(bl, "B1", "phase") == pytest.approx(math.radians(5.0), rel=1e-15)
    assert float(HPSim.get_db_model("B1", "phase_model", dbc)) == param(bl, "B1", "phase")
    HPSim.set_db_model("CA1", "aperture_model", "0.02", dbc, bl)
    HPSim.set_db_model("CA1", "in_out_model", "0", dbc, bl)
    assert param(bl, "CA1", "aperture") == 0.02 and param(bl, "CA1", "in") == 0.0
    for f, k, v in (("aperture_xl_model", "xl", 0.021), ("aperture_yb_model", "yb", 0.024)):
        HPSim.set_db_model("RA1", f, str(v), dbc, bl)
        assert param(bl, "RA1", k) == v
    # a module change reaches every gap of the module
    HPSim.set_db_model("MOD1", "amplitude_scale_cal", "1.1", dbc, bl)
    HPSim.set_db_model("MOD1", "phase_offset_cal", "3", dbc, bl)
    for g in ("G1", "G2"):
        assert param(bl, g, "amplitude") == pytest.approx(2.75, rel=1e-15)
        assert param(bl, g, "phase_ref") == -0.45
        assert param(bl, g, "phase_shift") == pytest.approx(math.radians(3.0), rel=1e-15)
    # a field of a table set_db_model does not serve changes nothing
    q = param(bl, "Q1", "gradient")
    assert dbloader.set_db_model("Q1", "gradient_model", "12", dbc, bl) is False
    assert param(bl, "Q1", "gradient") == q


def test_indices_kept_on_the_connection(lattice):
    """The beamline indices the connection keeps (a read-only file keeps
    none) find the elements when the file's model_index column is empty."""
    dbc, bl = lattice
    with dbc._conn:
        dbc._conn.execute("update spch_comp set model_index = NULL")
    HPSim.set_db_model("SC1", "fraction_model", "0.75", dbc, bl)
    assert param(bl, "SC1", "fraction") == 0.75


def test_bad_calls(lattice, capsys):
    dbc, bl = lattice
    HPSim.set_db_model("nope", "fraction_model", "1", dbc, bl)
    assert "can't make the change for nope:fraction_model" in capsys.readouterr().err
    with pytest.raises(ValueError):
        HPSim.set_db_model("SC1", "fraction_model", "half", dbc, bl)
    with pytest.raises(TypeError):
        HPSim.set_db_model("SC1", "fraction_model", "1", bl, dbc)
    with pytest.raises(NotImplementedError):
        HPSim.set_db_epics("TEST:PH1", "3", dbc, bl)


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DB, "tbtd.db")), reason="reference databases absent")
def test_reference_transport_database(tmp_path):
    """A copy of the reference's tbtd.db: a buncher's phase offset, through
    the database's own trigger, and a compensation fraction reach the
    beamline built from it."""
    from hpsim_gb300 import build
    build.build()
    path = str(tmp_path / "tbtd.db")
    shutil.copy(os.path.join(REF_DB, "tbtd.db"), path)
    dbc = HPSim.DBConnection(path)
    bl = HPSim.BeamLine(dbc)
    c = sqlite3.connect(path)
    bname, chan = c.execute("select name, phase_channel from buncher order by view_index limit 1").fetchone()
    sname = c.execute("select name from spch_comp order by view_index limit 1").fetchone()[0]
    c.close()
    HPSim.set_db_model(bname, "phase_offset_cal", "12.5", dbc, bl)
    ph = float(HPSim.get_db_model(bname, "phase_model", dbc))
    (cv,) = sqlite3.connect(path).execute("select value from epics_channel where id = ?", (chan,)).fetchone()
    assert ph == pytest.approx(math.radians(12.5 + cv), rel=1e-12)
    assert param(bl, bname, "phase") == ph
    HPSim.set_db_model(sname, "fraction_model", "0.3", dbc, bl)
    assert param(bl, sname, "fraction") == 0.3


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DB, "..", "pylib", "hpsim.py")), reason="reference absent")
def test_module_names_the_reference_python_layer_uses():
    """Every HPSim.<name> that the reference's pylib/hpsim.py uses exists in
    this module (set_db_epics among them, raising)."""
    import re
    src = open(os.path.join(REF_DB, "..", "pylib", "hpsim.py")).read()
    names = set(re.findall(r"\bHPSim\.([A-Za-z_]\w*)", src)) - {"so"}  # "HPSim.so" is the library's file name
    assert names and all(hasattr(HPSim, n) for n in names), sorted(n for n in names if not hasattr(HPSim, n))


def test_math_functions_for_triggers_without_sqlite_builtins():
    """A SQLite without its math functions gets them from Python's math
    module (a domain error gives NULL, as SQLite's own do)."""
    mem = sqlite3.connect(":memory:")

    class NoMath:  # a connection whose SQLite lacks the functions
        def execute(self, sql, *a):
            if sql.startswith("select pi()"):
                raise sqlite3.OperationalError("no such function: pi")
            return mem.execute(sql, *a)

        def create_function(self, *a, **k):
            return mem.create_function(*a, **k)

    dbloader._math_functions(NoMath())
    pi, p, c, a, r, bad = mem.execute("select pi(), power(2, 3), cos(0), acos(0.5), radians(180), acos(2)").fetchone()
    assert (pi, p, c, r, bad) == (math.pi, 8.0, 1.0, math.pi, None) and a == pytest.approx(math.pi / 3, rel=1e-15)
