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


def _math_functions(conn):
    """The databases' triggers call pi(), power(), cos(), acos() and their
    kin; SQLite builds without its math functions get them from Python's
    math module."""
    try:
        conn.execute("select pi(), power(2, 2), cos(0), acos(1), radians(0)").fetchone()
        return
    except sqlite3.OperationalError:
        pass
    import math

    def safe(f):
        def g(*a):
            try:
                return None if any(x is None for x in a) else f(*(float(x) for x in a))
            except (ValueError, OverflowError):
                return None  # NULL, as SQLite's own functions give for a domain error
        return g
    fns = {"pi": (0, lambda: math.pi), "power": (2, math.pow), "pow": (2, math.pow), "sqrt": (1, math.sqrt),
           "cos": (1, math.cos), "sin": (1, math.sin), "tan": (1, math.tan), "acos": (1, math.acos),
           "asin": (1, math.asin), "atan": (1, math.atan), "atan2": (2, math.atan2), "exp": (1, math.exp),
           "ln": (1, math.log), "log10": (1, math.log10), "radians": (1, math.radians),
           "degrees": (1, math.degrees)}
    for name, (n, f) in fns.items():
        conn.create_function(name, n, safe(f), deterministic=True)


def open_connection(db_addr):
    """DBConnection(db_addr): the connection and its database list
    [("main", path)]."""
    if not os.path.exists(db_addr):
        raise ValueError(f"DBConnection: no database at {db_addr}")
    conn = sqlite3.connect(db_addr)
    _math_functions(conn)
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


# ---- model and channel values by record name (hpsim_module.cpp:86-360) ----

def _tables(conn, db):
    return [r[0] for r in conn.execute(f"select name from {_ident(db)}.sqlite_master where type = 'table'")]


def _columns(conn, db, tbl):
    """The table's column names; none for a table whose name is not a plain
    identifier (no element table has such a name)."""
    if not tbl.replace("_", "").isalnum():
        return []
    return [r[1] for r in conn.execute(f"pragma {_ident(db)}.table_info({tbl})")]


def _text(conn, sql, args):
    """GetDataFromDB: the first row's first column as SQLite renders it as
    text; '' for no row, NULL, or a table without the queried columns."""
    try:
        row = conn.execute(sql, args).fetchone()
    except sqlite3.OperationalError:
        return ""
    return "" if row is None or row[0] is None else str(row[0])


def get_db_model(record_name, field_name, dbc):
    """GetDbModel (hpsim_module.cpp:307-360): the value of ``field_name`` of
    the record called ``record_name``, from the first table (every database
    of the connection in order, ``epics_channel`` excluded) that has the
    column and a non-NULL value there, as text; None when none has."""
    conn = dbc._conn
    for db, _ in dbc.dbs:
        for tbl in _tables(conn, db):
            if tbl == "epics_channel" or field_name not in _columns(conn, db, tbl):
                continue
            v = _text(conn, f"select cast({field_name} as text) from {db}.{tbl} where name = ?", (record_name,))
            if v != "":
                return v
    return None


def get_db_epics(pv_name, dbc):
    """GetDbEPICS (hpsim_module.cpp:269-305): the ``value`` of the
    ``epics_channel`` row whose ``lcs_name`` is ``pv_name`` (first database
    that has one), as text; None when no database has a value for it."""
    conn = dbc._conn
    for db, _ in dbc.dbs:
        v = _text(conn, f"select cast(value as text) from {_ident(db)}.epics_channel where lcs_name = ?",
                  (pv_name,))
        if v != "":
            return v
    return None


def _sql_number(value):
    """The reference pastes ``value`` into the UPDATE statement as an SQL
    literal: an integer literal stays an integer, anything else numeric is a
    real; here it is bound as a parameter of that type."""
    s = str(value).strip()
    try:
        return int(s) if s.lstrip("+-").isdigit() else float(s)
    except ValueError:
        raise ValueError(f"set_db_model: {value!r} is not a number") from None


# tables set_db_model changes, and for each the fields whose new model value
# it also hands to the beamline's element: (field changed, model column read
# back after the database's triggers ran, element parameter)
_MODEL_PUSH = {
    "spch_comp": {"fraction_model": ("fraction_model", "fraction")},
    "buncher": {"phase_offset_cal": ("phase_model", "phase")},
    "raperture": {f: (f, p) for f, p in (("aperture_xl_model", "xl"), ("aperture_xr_model", "xr"),
                                         ("aperture_yt_model", "yt"), ("aperture_yb_model", "yb"),
                                         ("in_out_model", "in"))},
    "caperture": {"aperture_model": ("aperture_model", "aperture"), "in_out_model": ("in_out_model", "in")},
    "rf_module": {},
}
# rf_module fields and the rf_gap columns -> element parameters they reach
_RF_PUSH = {
    "phase_offset_cal": (("beam_phase_shift_model", "phase_shift"),),
    "amplitude_scale_cal": (("amplitude_model", "amplitude"), ("ref_phase_model", "phase_ref")),
    "amplitude_tilt_cal": (("amplitude_model", "amplitude"), ("ref_phase_model", "phase_ref")),
    "voltage_cal": (("amplitude_model", "amplitude"), ("ref_phase_model", "phase_ref")),
}


def _model_index(dbc, db, tbl, where, args):
    """The beamline index of a record: the connection's own record of it
    (kept for every database, writable or not), else the table's
    model_index column."""
    conn = dbc._conn
    row = conn.execute(f"select view_index, model_index from {db}.{tbl} where {where}", args).fetchone()
    if row is None:
        return None
    mi = dbc.model_index.get((db, tbl, row[0]))
    if mi is None and row[1] is not None:
        mi = int(row[1])
    return mi


def _push(beamline, index, key, text):
    if index is None or beamline is None:
        return
    v = _f(text)
    if key == "in":
        v = 1.0 if _on(text) else 0.0
    beamline.set_param(int(index), key, v)


def set_db_model(record_name, field_name, value, dbc, beamline):
    """SetDbModel (hpsim_module.cpp:86-267): set ``field_name`` of the record
    ``record_name`` in the first of the tables buncher, rf_module, spch_comp,
    raperture and caperture (every database of the connection in order) that
    has the column and the record, let the database's triggers recompute the
    model columns, and hand the new model values to the beamline's elements:
    a space-charge compensation's fraction, a buncher's phase (after
    ``phase_offset_cal``), an aperture's sizes and in/out flag, and for an RF
    module every gap of the module (``phase_offset_cal``: the beam phase
    shift; ``amplitude_scale_cal``, ``amplitude_tilt_cal``, ``voltage_cal``:
    amplitude and reference phase).  Returns True when a table took the
    change, False (with a message on stderr, as the reference prints) when
    none had the record and field."""
    import sys
    conn = dbc._conn
    num = _sql_number(value)
    for db, _ in dbc.dbs:
        for tbl in _tables(conn, db):
            if tbl not in _MODEL_PUSH or field_name not in _columns(conn, db, tbl):
                continue
            if conn.execute(f"select 1 from {db}.{tbl} where name = ? limit 1", (record_name,)).fetchone() is None:
                continue
            try:
                with conn:
                    conn.execute(f"update {db}.{tbl} set {field_name} = ? where name = ?", (num, record_name))
            except sqlite3.Error as e:
                raise RuntimeError(f"set_db_model: {record_name}:{field_name}: {e}") from None
            if tbl == "rf_module":
                cols = _RF_PUSH.get(field_name, ())
                if cols:
                    gaps = conn.execute(
                        f"select view_index, model_index, {', '.join(c for c, _ in cols)} from {db}.rf_gap "
                        f"where module_id = (select id from {db}.rf_module where name = ?)", (record_name,)).fetchall()
                    for vi, mi_col, *vals in gaps:
                        mi = dbc.model_index.get((db, "rf_gap", vi), mi_col)
                        for (_, key), v in zip(cols, vals):
                            _push(beamline, mi, key, v)
            elif field_name in _MODEL_PUSH[tbl]:
                col, key = _MODEL_PUSH[tbl][field_name]
                text = _text(conn, f"select cast({col} as text) from {db}.{tbl} where name = ?", (record_name,))
                _push(beamline, _model_index(dbc, db, tbl, "name = ?", (record_name,)), key, text)
            return True
    print(f"Error in set_db_model: can't make the change for {record_name}:{field_name}", file=sys.stderr)
    return False
