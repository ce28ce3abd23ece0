"""Lattice databases -> element records (hpsim_gb300/dbloader.py against
GenerateBeamLine, src/beamline/src/init.cpp:20-429): a database with the
reference's tables built here, an attached second database, model_index
bookkeeping, read-only files, and -- where the reference tree is present --
the reference's own databases and the fixtures made from them."""
import os
import sqlite3

import numpy as np
import pytest

from hpsim_gb300 import HPSim, dbloader, lattices as L

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree's lattice databases, beside this repository (or named by
# HPS_REFERENCE_DB); the tests that read them are skipped where it is absent
REF_DB = os.environ.get("HPS_REFERENCE_DB", os.path.join(HERE, "..", "..", "reference", "db"))

TABLES = {
    "linac": "view_index INTEGER, name TEXT, model_type TEXT, model_index INTEGER",
    "quad": "view_index INTEGER, gradient_model REAL, length_model REAL, aperture_model REAL, monitor INTEGER, "
            "model_index INTEGER",
    "drift": "view_index INTEGER, length_model REAL, aperture_model REAL, model_index INTEGER",
    "rf_module": "id INTEGER, cell_length_betalambda_design REAL",
    "rf_gap": "view_index INTEGER, module_id INTEGER, cell_id INTEGER, tank_id INTEGER, length_model REAL, "
              "frequency_model REAL, amplitude_model REAL, ref_phase_model REAL, beam_phase_shift_model REAL, "
              "energy_out_model REAL, beta_center_model REAL, dg_model REAL, t_model REAL, tp_model REAL, "
              "sp_model REAL, model_index INTEGER",
    "transit_time_factor": "module_id INTEGER, tank_id INTEGER, beta_g REAL, beta_min REAL, ta0 REAL, ta1 REAL, "
                           "ta2 REAL, ta3 REAL, ta4 REAL, ta5 REAL, sa1 REAL, sa2 REAL, sa3 REAL, sa4 REAL, "
                           "sa5 REAL",
    "rotation": "view_index INTEGER, angle_model REAL, model_index INTEGER",
    "caperture": "view_index INTEGER, aperture_model REAL, in_out_model INTEGER, model_index INTEGER",
    "raperture": "view_index INTEGER, aperture_xl_model REAL, aperture_xr_model REAL, aperture_yt_model REAL, "
                 "aperture_yb_model REAL, in_out_model INTEGER, model_index INTEGER",
    "diagnostics": "view_index INTEGER, monitor INTEGER, model_index INTEGER",
    "buncher": "view_index INTEGER, voltage_model REAL, frequency_model REAL, phase_model REAL, "
               "aperture_model REAL, on_off INTEGER, model_index INTEGER",
    "dipole": "view_index INTEGER, rho_model REAL, angle_model REAL, edge_angle1_model REAL, "
              "edge_angle2_model REAL, half_gap_model REAL, k1_model REAL, k2_model REAL, "
              "field_index_model REAL, kenergy_model REAL, model_index INTEGER",
    "spch_comp": "view_index INTEGER, fraction_model REAL, model_index INTEGER",
    "steerer": "view_index INTEGER, bl_h_model REAL, bl_v_model REAL, model_index INTEGER",
    "epics_channel": "lcs_name TEXT",
}


def make_db(path, rows, tag):
    """rows: [(model_type, name, {table column: value}, extra inserts)]"""
    c = sqlite3.connect(path)
    for t, cols in TABLES.items():
        c.execute(f"create table {t} ({cols})")
    for vi, (mtype, name, vals, extra) in enumerate(rows):
        c.execute("insert into linac values (?, ?, ?, NULL)", (vi, name, mtype))
        tbl = dbloader.KINDS[mtype]
        vals = dict(vals, view_index=vi)
        c.execute(f"insert into {tbl} ({', '.join(vals)}) values ({', '.join('?' * len(vals))})", list(vals.values()))
        for t, v in extra:
            c.execute(f"insert into {t} ({', '.join(v)}) values ({', '.join('?' * len(v))})", list(v.values()))
    c.execute("insert into epics_channel values (?)", (f"{tag}:PV1",))
    c.commit()
    c.close()


RNG = np.random.default_rng(7)


def r():
    return float(RNG.normal())


def first_db_rows():
    fit = {"module_id": 1, "tank_id": 3, "beta_g": 0.04, "beta_min": 0.035,
           **{f"ta{k}": r() for k in range(6)}, **{f"sa{k}": r() for k in range(1, 6)}}
    fit_ccl = dict(fit, tank_id=5, beta_g=0.43)
    gap = {"module_id": 1, "cell_id": 3, "tank_id": 9, "length_model": 0.05, "frequency_model": 201.25,
           "amplitude_model": 1.7, "ref_phase_model": -0.41, "beam_phase_shift_model": 3.6,
           "energy_out_model": 0.81, "beta_center_model": 0.0407, "dg_model": 0.0026, "t_model": 0.7,
           "tp_model": 0.07, "sp_model": 0.05}
    ccl = dict(gap, cell_id=99, tank_id=5, frequency_model=805.0)
    return [
        ("quad", "Q1", {"gradient_model": r(), "length_model": 0.03, "aperture_model": 0.0075, "monitor": 1}, []),
        ("drift", "D1", {"length_model": 0.2, "aperture_model": 0.01}, []),
        ("dtl_gap", "G1", gap, [("rf_module", {"id": 1, "cell_length_betalambda_design": 1.0}),
                                ("transit_time_factor", fit), ("transit_time_factor", fit_ccl)]),
        ("ccl_gap", "C1", ccl, []),
        ("rotation", "R1", {"angle_model": 0.3}, []),
        ("caperture", "A1", {"aperture_model": 0.02, "in_out_model": 1}, []),
        ("raperture", "A2", {"aperture_xl_model": 0.01, "aperture_xr_model": 0.02, "aperture_yt_model": 0.03,
                             "aperture_yb_model": 0.04, "in_out_model": 0}, []),
        ("diagnostics", "M1", {"monitor": 1}, []),
        ("buncher", "B1", {"voltage_model": 0.15, "frequency_model": 201.25, "phase_model": -1.57,
                           "aperture_model": 0.01, "on_off": 1}, []),
        ("dipole", "BM1", {"rho_model": 0.57, "angle_model": 1.41, "edge_angle1_model": 0.45,
                           "edge_angle2_model": 0.44, "half_gap_model": 0.038, "k1_model": 0.45, "k2_model": 2.8,
                           "field_index_model": 0.1, "kenergy_model": 0.75}, []),
        ("spch_comp", "S1", {"fraction_model": 0.6}, []),
        ("steerer", "ST1", {"bl_h_model": 1e-4, "bl_v_model": -2e-4}, []),
    ]


def check_record(e, mtype, vals, fits):
    code, name, p = e
    P = lambda k: p[L.param_index(code, k)]  # noqa: E731
    if mtype == "quad":
        assert code == L.QUAD and P("gradient") == vals["gradient_model"] and P("length") == 0.03
        assert P("aperture") == 0.0075 and P("monitor") == 1.0
    elif mtype == "drift":
        assert code == L.DRIFT and P("length") == 0.2 and P("aperture") == 0.01
    elif mtype in ("dtl_gap", "ccl_gap"):
        assert code == (L.RFGAP_DTL if mtype == "dtl_gap" else L.RFGAP_CCL)
        fit = fits[mtype]
        assert P("fit_beta_center") == fit["beta_g"] and P("fit_beta_min") == fit["beta_min"]
        assert [P(f"fit_t{k}") for k in range(6)] == [fit[f"ta{k}"] for k in range(6)]
        assert [P(f"fit_s{k}") for k in range(1, 6)] == [fit[f"sa{k}"] for k in range(1, 6)]
        for k, col in (("frequency", "frequency_model"), ("amplitude", "amplitude_model"),
                       ("phase_ref", "ref_phase_model"), ("phase_shift", "beam_phase_shift_model"),
                       ("energy_out", "energy_out_model"), ("beta_center", "beta_center_model"),
                       ("dg", "dg_model"), ("t", "t_model"), ("tp", "tp_model"), ("sp", "sp_model"),
                       ("length", "length_model")):
            assert P(k) == vals[col], k
        assert P("cell_length_over_beta_lambda") == 1.0
    elif mtype == "rotation":
        assert code == L.ROTATION and P("angle") == 0.3
    elif mtype == "caperture":
        assert code == L.APERTURE_C and P("aperture") == 0.02 and P("in") == 1.0
    elif mtype == "raperture":
        assert code == L.APERTURE_R and (P("xl"), P("xr"), P("yt"), P("yb")) == (0.01, 0.02, 0.03, 0.04)
        assert P("in") == 0.0  # out unless the database says in, as the reference's constructor
    elif mtype == "diagnostics":
        assert code == L.DIAGNOSTICS and P("monitor") == 1.0
    elif mtype == "buncher":
        assert code == L.BUNCHER and (P("voltage"), P("frequency"), P("phase"), P("on")) == (0.15, 201.25, -1.57, 1.0)
    elif mtype == "dipole":
        assert code == L.DIPOLE and (P("radius"), P("angle"), P("field_index"), P("kinetic_energy")) == \
            (0.57, 1.41, 0.1, 0.75)
    elif mtype == "spch_comp":
        assert code == L.SPCHCOMP and P("fraction") == 0.6
    elif mtype == "steerer":
        assert code == L.STEERER and (P("blh"), P("blv")) == (1e-4, -2e-4)


def test_every_element_kind_and_an_attached_database(tmp_path):
    rows = first_db_rows()
    a, b = str(tmp_path / "a.db"), str(tmp_path / "b.db")
    make_db(a, rows, "A")
    rows_b = [("drift", "DB1", {"length_model": 0.5, "aperture_model": 0.0}, []),
              ("quad", "QB1", {"gradient_model": -3.0, "length_model": 0.03, "aperture_model": 0.0,
                               "monitor": 0}, [])]
    make_db(b, rows_b, "B")
    dbc = HPSim.DBConnection(a)
    dbc.attach_db(b, "db1")
    els = dbloader.generate_beamline(dbc)
    assert [e[1] for e in els] == [r[1] for r in rows] + ["DB1", "QB1"]
    fits = {"dtl_gap": rows[2][3][1][1], "ccl_gap": rows[2][3][2][1]}
    for e, (mtype, _, vals, _) in zip(els, rows):
        check_record(e, mtype, vals, fits)
    assert els[-1][2][L.param_index(L.QUAD, "gradient")] == -3.0
    # model_index: the element's position in the beamline, in its own table
    c = sqlite3.connect(a)
    assert c.execute("select model_index from quad where view_index = 0").fetchone()[0] == 0
    assert c.execute("select model_index from steerer").fetchone()[0] == len(rows) - 1
    c.close()
    c = sqlite3.connect(b)
    assert c.execute("select model_index from quad").fetchone()[0] == len(rows) + 1
    c.close()
    assert dbc.get_epics_channels() == ["A:PV1", "B:PV1"]
    dbc.clear_model_index()
    c = sqlite3.connect(a)
    assert c.execute("select count(*) from quad where model_index is not null").fetchone()[0] == 0
    c.close()


def test_read_only_database_keeps_indices_on_the_connection(tmp_path):
    a = str(tmp_path / "ro.db")
    make_db(a, first_db_rows(), "A")
    dbc = HPSim.DBConnection(a)
    dbc._conn.close()
    dbc._conn = sqlite3.connect(f"file:{a}?mode=ro", uri=True)  # as for a read-only file
    els = dbloader.generate_beamline(dbc)
    assert len(els) == len(first_db_rows())
    assert dbc.model_index[("main", "quad", 0)] == 0
    assert dbc.model_index[("main", "steerer", len(els) - 1)] == len(els) - 1
    c = sqlite3.connect(a)
    assert c.execute("select count(*) from quad where model_index is not null").fetchone()[0] == 0
    c.close()


def test_missing_database_raises(tmp_path):
    with pytest.raises(ValueError):
        HPSim.DBConnection(str(tmp_path / "nope.db"))


@pytest.mark.skipif(not os.path.isdir(REF_DB), reason="the reference's lattice databases are not present")
@pytest.mark.parametrize("name", ["dtl", "tbtd"])
def test_fixtures_are_the_reference_databases(name):
    """The committed fixtures equal a fresh load of the reference's own
    database, and each record equals the database's model columns."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_db_lattices as M
    els = M.load(REF_DB, name)
    z = np.load(os.path.join(HERE, "golden", f"db_{name}.npz"))
    assert list(z["types"]) == [e[0] for e in els]
    assert list(z["names"]) == [e[1] for e in els]
    assert np.array_equal(z["params"], np.stack([e[2] for e in els]))
    c = sqlite3.connect(f"file:{REF_DB}/{name}.db?mode=ro", uri=True)
    rows = c.execute("select name, model_type from linac").fetchall()
    assert [n for n, t in rows if t in dbloader.KINDS] == [e[1] for e in els]
    if name == "dtl":
        g = c.execute("select amplitude_model, ref_phase_model, energy_out_model from rf_gap "
                      "order by view_index limit 1").fetchone()
        first_gap = next(e for e in els if e[0] == L.RFGAP_DTL)
        p = first_gap[2]
        assert (p[L.param_index(L.RFGAP_DTL, "amplitude")], p[L.param_index(L.RFGAP_DTL, "phase_ref")],
                p[L.param_index(L.RFGAP_DTL, "energy_out")]) == tuple(float(v) for v in g)
