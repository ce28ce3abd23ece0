"""Lattice databases -> beamline elements (GenerateBeamLine,
src/beamline/src/init.cpp:20-429; DBConnection, src/util/src/sql_utility.cpp:
211-367).

The reference reads one table per element kind from every database of a
connection (``main`` and the attached ones, in order), walking each
database's ``linac`` table, and records each element's position in the
beamline in the ``model_index`` column of its table.  This module does the
same over Python's ``sqlite3``: it reads the ``*_model`` columns only (the
values the reference's model uses; the SQL math extension the reference
loads serves the EPICS-facing columns and is not needed for them) and
returns element records for ``hps_beamline_add``.  ``model_index`` is
written back when the database file is writable, as the reference does; for
a read-only file the indices are kept on the connection object instead
(``DBConnection.model_index``).

Element records follow include/hps_layout.h through ``lattices.element``;
apertures and bunchers are in/on only when the database says so, as the
reference's constructors default to out/off.
"""
from __future__ import annotations

import os
import sqlite3

from . import lattices as L

# linac.model_type -> (table, element kind)
KINDS = {
    "quad": "quad", "drift": "drift", "dtl_gap": "rf_gap", "ccl_gap": "rf_gap",
    "rotation": "rotation", "caperture": "caperture", "raperture": "raperture",
    "diagnostics": "diagnostics", "buncher": "buncher", "dipole": "dipole",
    "spch_comp": "spch_comp", "steerer": "steerer",
}


def open_connection(db_addr):
    """DBConnection(db_addr): the connection and its database list
    [("main", path)]."""
    if not os.path.exists(db_addr):
        raise ValueError(f"DBConnection: no database at {db_addr}")
    conn = sqlite3.connect(db_addr)
    return conn, [("main", db_addr)]


def attach(dbc, db_addr, db_name=None):
    """DBConnection::AttachDB: ``attach '<addr>' as <name>``."""
    if not os.path.exists(db_addr):
        raise ValueError(f"attach_db: no database at {db_addr}")
    name = db_name or f"db{len(dbc.dbs)}"
    dbc._conn.execute(f"attach ? as {_ident(name)}", (db_addr,))
    dbc.dbs.append((name, db_addr))


def _ident(name):
    if not name.replace("_", "").isalnum():
        raise ValueError(f"bad database alias: {name!r}")
    return name


def _one(conn, sql, args=()):
    row = conn.execute(sql, args).fetchone()
    if row is None:
        raise ValueError(f"lattice database: no row for {sql} {args}")
    return row


def _f(v):
    """std::atof of the reference's text value (NULL and '' give 0)."""
    if v is None:
        return 0.0
    try:
        return float(v)
    except (TypeError, ValueError):
        return 0.0


def _on(v):
    """std::atoi(v) > 0."""
    try:
        return int(float(v)) > 0
    except (TypeError, ValueError):
        return False


def _element(conn, db, kind, name, vi):
    q = lambda cols, tbl: _one(conn, f"select {cols} from {db}.{tbl} where view_index = ?", (vi,))  # noqa: E731
    if kind == "quad":
        g, ln, ap, mon = q("gradient_model, length_model, aperture_model, monitor", "quad")
        return L.element(L.QUAD, name, gradient=_f(g), length=_f(ln), aperture=_f(ap),
                         monitor=1.0 if _on(mon) else 0.0)
    if kind == "drift":
        ln, ap = q("length_model, aperture_model", "drift")
        return L.element(L.DRIFT, name, length=_f(ln), aperture=_f(ap))
    if kind in ("dtl_gap", "ccl_gap"):
        # DTL fits join on the cell id, CCL fits on the tank id (init.cpp:118-130)
        key = "cell_id" if kind == "dtl_gap" else "tank_id"
        fit = _one(conn, f"select t1.beta_g, t1.beta_min, t1.ta0, t1.ta1, t1.ta2, t1.ta3, t1.ta4, t1.ta5, "
                         f"t1.sa1, t1.sa2, t1.sa3, t1.sa4, t1.sa5 from {db}.transit_time_factor t1 join "
                         f"{db}.rf_gap t2 on t1.module_id = t2.module_id and t1.tank_id = t2.{key} "
                         f"where t2.view_index = ?", (vi,))
        (ln, fr, amp, ph, shift, wout, bc, dg, t, tp, sp) = q(
            "length_model, frequency_model, amplitude_model, ref_phase_model, beam_phase_shift_model, "
            "energy_out_model, beta_center_model, dg_model, t_model, tp_model, sp_model", "rf_gap")
        clbl = _one(conn, f"select cell_length_betalambda_design from {db}.rf_module where id = "
                          f"(select module_id from {db}.rf_gap where view_index = ?)", (vi,))[0]
        names = ["fit_beta_center", "fit_beta_min", "fit_t0", "fit_t1", "fit_t2", "fit_t3", "fit_t4",
                 "fit_t5", "fit_s1", "fit_s2", "fit_s3", "fit_s4", "fit_s5"]
        kw = {k: _f(v) for k, v in zip(names, fit)}
        kw.update(length=_f(ln), frequency=_f(fr), cell_length_over_beta_lambda=_f(clbl), amplitude=_f(amp),
                  phase_ref=_f(ph), phase_shift=_f(shift), energy_out=_f(wout), beta_center=_f(bc),
                  dg=_f(dg), t=_f(t), tp=_f(tp), sp=_f(sp))
        return L.element(L.RFGAP_DTL if kind == "dtl_gap" else L.RFGAP_CCL, name, **kw)
    if kind == "rotation":
        (a,) = q("angle_model", "rotation")
        return L.element(L.ROTATION, name, angle=_f(a))
    if kind == "caperture":
        ap, io = q("aperture_model, in_out_model", "caperture")
        return L.element(L.APERTURE_C, name, aperture=_f(ap), **{"in": 1.0 if _on(io) else 0.0})
    if kind == "raperture":
        xl, xr, yt, yb, io = q("aperture_xl_model, aperture_xr_model, aperture_yt_model, aperture_yb_model, "
                               "in_out_model", "raperture")
        return L.element(L.APERTURE_R, name, xl=_f(xl), xr=_f(xr), yt=_f(yt), yb=_f(yb),
                         **{"in": 1.0 if _on(io) else 0.0})
    if kind == "diagnostics":
        (mon,) = q("monitor", "diagnostics")
        return L.element(L.DIAGNOSTICS, name, monitor=1.0 if _on(mon) else 0.0)
    if kind == "buncher":
        v, fr, ph, ap, on = q("voltage_model, frequency_model, phase_model, aperture_model, on_off", "buncher")
        return L.element(L.BUNCHER, name, voltage=_f(v), frequency=_f(fr), phase=_f(ph), aperture=_f(ap),
                         on=1.0 if _on(on) else 0.0)
    if kind == "dipole":
        r, a, e1, e2, hg, k1, k2, fi, ke = q(
            "rho_model, angle_model, edge_angle1_model, edge_angle2_model, half_gap_model, k1_model, "
            "k2_model, field_index_model, kenergy_model", "dipole")
        return L.element(L.DIPOLE, name, radius=_f(r), angle=_f(a), edge_in=_f(e1), edge_out=_f(e2),
                         half_gap=_f(hg), k1=_f(k1), k2=_f(k2), field_index=_f(fi), kinetic_energy=_f(ke))
    if kind == "spch_comp":
        (fr,) = q("fraction_model", "spch_comp")
        return L.element(L.SPCHCOMP, name, fraction=_f(fr))
    if kind == "steerer":
        h, v = q("bl_h_model, bl_v_model", "steerer")
        return L.element(L.STEERER, name, blh=_f(h), blv=_f(v))
    return None  # model types the reference does not build are skipped, as there


def generate_beamline(dbc):
    """GenerateBeamLine: the element records of every database of the
    connection, in database order and each database's ``linac`` order."""
    conn = dbc._conn
    out = []
    index = {}
    writes = []
    for db, _ in dbc.dbs:
        rows = conn.execute(f"select name, view_index, model_type from {_ident(db)}.linac").fetchall()
        for name, vi, mtype in rows:
            e = _element(conn, _ident(db), mtype, name, vi)
            if e is None:
                continue
            index[(db, KINDS[mtype], vi)] = len(out)
            writes.append((db, KINDS[mtype], len(out), vi))
            out.append(e)
    dbc.model_index = index
    try:
        with conn:
            for db, tbl, mi, vi in writes:
                conn.execute(f"update {db}.{tbl} set model_index = ? where view_index = ?", (mi, vi))
    except sqlite3.OperationalError:
        pass  # read-only database: the indices stay on the connection object
    return out


def clear_model_index(dbc):
    """DBConnection::ClearModelIndex: model_index = NULL in every table that
    has the column (sql_utility.cpp:332-351)."""
    conn = dbc._conn
    dbc.model_index = {}
    try:
        with conn:
            for db, _ in dbc.dbs:
                for (tbl,) in conn.execute(f"select name from {_ident(db)}.sqlite_master where type = 'table'"):
                    cols = [r[1] for r in conn.execute(f"pragma {db}.table_info({tbl})")]
                    if "model_index" in cols:
                        conn.execute(f"update {db}.{tbl} set model_index = NULL")
    except sqlite3.OperationalError:
        pass


def epics_channels(dbc):
    """DBConnection::GetEPICSChannels: lcs_name of every epics_channel row."""
    out = []
    for db, _ in dbc.dbs:
        out += [r[0] for r in dbc._conn.execute(f"select lcs_name from {_ident(db)}.epics_channel")]
    return out
