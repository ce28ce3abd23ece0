"""Python 3 mirror of the reference's ``HPSim`` extension module.

Same classes, method names, positional/keyword arguments and defaults as the
CPython 2 extension (src/pywrapper/src/wrap_beam.cpp, wrap_beamline.cpp,
wrap_spacecharge.cpp, wrap_simulator.cpp, hpsim_module.cpp), implemented over
the C ABI of include/hpsim_gb300.h.  Where the reference prints to stderr and
returns None on bad input, these raise ``ValueError``; CUDA failures raise
``HPSimError``.  Additions (marked below) cover what the reference could only
do through its lattice database.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lattices as _lat
from ._capi import call, dptr, lib, uptr, HPSimError  # noqa: F401

_COORD = {"x": 0, "xp": 1, "y": 2, "yp": 3, "phi": 4, "w": 5}
_ST = {n: i for i, n in enumerate(
    "x_avg x_avg_good xp_avg y_avg y_avg_good yp_avg phi_avg phi_avg_r phi_avg_good w_avg "
    "w_avg_good x_sig x_sig_good xp_sig y_sig y_sig_good yp_sig phi_sig phi_sig_r phi_sig_good "
    "w_sig w_sig_good x_emit y_emit z_emit r_max abs_phi_max num_loss num_lloss num_good".split())}
# Beam::Update* selectors of hps_beam_update
_UPD_LOSS, _UPD_LLOSS, _UPD_GOOD, _UPD_AVG, _UPD_SIG, _UPD_EMIT, _UPD_RELPHI = 0, 1, 2, 3, 4, 5, 6
_UPD_STAT_SC, _UPD_AVGXY, _UPD_MAXR = 7, 8, 9
_PREC = {"fp64": 0, "fp32": 1}


def set_gpu(device_id):
    """set_gpu(device_id): choose the GPU (src/pywrapper/src/hpsim_module.cpp:39-53)."""
    call("hps_set_gpu", int(device_id))


class Beam:
    """Beam(mass=, charge=, current=, num=) or Beam(file=) (wrap_beam.cpp:26-49).

    Addition: ``precision='fp64'`` (default; the reference's FP64 semantics)
    or ``'fp32'`` (FP32 particle state about an FP64 synchronous particle)."""

    def __init__(self, mass=None, charge=None, current=0.0, num=0, file=None, precision="fp64"):
        self._h = C.c_void_p()
        if file:
            from .beam_io import read_beam_file
            mass, charge, current, freq, cols = read_beam_file(file)
            num = len(cols[0])
        if not num:
            raise ValueError("Beam constructor needs either a file name or num of particles as arg!")
        if mass is None or charge is None:
            raise ValueError("Beam(mass=, charge=, current=, num=) needs mass and charge")
        call("hps_beam_create", int(num), float(mass), float(charge), float(current),
             _PREC[precision], C.byref(self._h))
        self._n = int(num)
        if file:
            self.set_frequency(freq)
            x, xp, y, yp, phi, w, loss, lloss = cols
            # Beam::UpdateBeamFromFile: particle 0 on axis, design_w = w[0]
            self._set_dist_raw(x, xp, y, yp, phi, w, loss, lloss)
            self._design_w_from_file = float(w[0])
            call("hps_beam_set_ref_w", self._h, float(w[0]))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().hps_beam_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    # ---- initial distributions -------------------------------------------
    def _set_dist_raw(self, x, xp, y, yp, phi, w, loss=None, lloss=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, xp, y, yp, phi, w)]
        if any(len(a) != self._n for a in arrs):
            raise ValueError("provided distribution size doesn't match number of particles allocated")
        lo = None if loss is None else np.ascontiguousarray(loss, dtype=np.uint32)
        ll = None if lloss is None else np.ascontiguousarray(lloss, dtype=np.uint32)
        call("hps_beam_set_distribution", self._h, *[dptr(a) for a in arrs],
             uptr(lo) if lo is not None else None, uptr(ll) if ll is not None else None)

    def set_distribution(self, x, xp, y, yp, phi, w, loss=None, lloss=None):
        """set_distribution(x, xp, y, yp, phi, w, loss, lloss) (wrap_beam.cpp:61-123)."""
        self._set_dist_raw(x, xp, y, yp, phi, w, loss, lloss)

    def set_waterbag(self, ax, bx, ex, ay, by, ey, az, bz, ez, phi, w, freq, seed=0):
        """6D waterbag, PARMILA units (Beam::InitWaterbagBeam, beam.cpp:391-462)."""
        t = np.array([ax, bx, ex, ay, by, ey, az, bz, ez], dtype=np.float64)
        call("hps_beam_set_waterbag", self._h, dptr(t), float(phi), float(w), float(freq), int(seed))

    def set_dc(self, ax, bx, ex, ay, by, ey, dphi, phi, w, seed=0):
        """DC beam (Beam::InitDCBeam, beam.cpp:481-537)."""
        t = np.array([ax, bx, ex, ay, by, ey], dtype=np.float64)
        call("hps_beam_set_dc", self._h, dptr(t), float(dphi), float(phi), float(w), int(seed))

    def save_initial_beam(self):
        call("hps_beam_save", self._h, 0)

    def save_intermediate_beam(self):
        call("hps_beam_save", self._h, 1)

    def restore_initial_beam(self):
        call("hps_beam_restore", self._h, 0)

    def restore_intermediate_beam(self):
        call("hps_beam_restore", self._h, 1)

    def print_to(self, output_file, msg=""):
        """Text dump of Beam::PrintToFile (beam.cpp:670-707)."""
        from .beam_io import write_beam_file
        self._update(_UPD_LOSS)
        cols = [self._coord(k) for k in ("x", "xp", "y", "yp", "phi", "w")]
        write_beam_file(output_file, msg, self.get_charge(), self.get_mass(), self._scalar(2),
                        self.get_frequency(), cols, self._loss(0), self._loss(1))

    # ---- scalars -----------------------------------------------------------
    def _scalar(self, which):
        v = C.c_double()
        call("hps_beam_get_scalar", self._h, which, C.byref(v))
        return v.value

    def set_ref_w(self, w):
        call("hps_beam_set_ref_w", self._h, float(w))

    def set_ref_phi(self, phi):
        call("hps_beam_set_ref_phi", self._h, float(phi))

    def set_frequency(self, freq):
        call("hps_beam_set_frequency", self._h, float(freq))

    def get_mass(self):
        return self._scalar(0)

    def get_charge(self):
        return self._scalar(1)

    def get_frequency(self):
        return self._scalar(3)

    def get_ref_w(self):
        w, p = C.c_double(), C.c_double()
        call("hps_beam_get_ref", self._h, C.byref(w), C.byref(p))
        return w.value

    def get_ref_phi(self):
        w, p = C.c_double(), C.c_double()
        call("hps_beam_get_ref", self._h, C.byref(w), C.byref(p))
        return p.value

    def get_size(self):
        return self._n

    # ---- device statistics (Beam::Update* then Beam::Get*) -----------------
    def _update(self, op, coord=0, good=0):
        call("hps_beam_update", self._h, op, coord, int(good))

    def _stat(self, name):
        v = C.c_double()
        call("hps_beam_get_stat", self._h, _ST[name], C.byref(v))
        return v.value

    def _coord(self, name):
        out = np.empty(self._n, dtype=np.float64)
        call("hps_beam_get_coord", self._h, _COORD[name] if name in _COORD else 6, dptr(out))
        return out

    def _loss(self, longitudinal):
        out = np.empty(self._n, dtype=np.uint32)
        call("hps_beam_get_loss", self._h, int(longitudinal), uptr(out))
        return out

    def _select(self, arr, option):
        if option not in ("good", "lost", "all"):
            raise ValueError(f"invalid option: {option}, pick from ('good', 'lost', 'all')")
        if option == "all":
            return arr
        loss = self._loss(0)
        return arr[loss == 0] if option == "good" else arr[loss != 0]

    def _get(self, name, option):
        self._update(_UPD_LOSS)
        return self._select(self._coord(name), option)

    def get_x(self, option="good"):
        return self._get("x", option)

    def get_xp(self, option="good"):
        return self._get("xp", option)

    def get_y(self, option="good"):
        return self._get("y", option)

    def get_yp(self, option="good"):
        return self._get("yp", option)

    def get_w(self, option="good"):
        return self._get("w", option)

    def get_phi(self, option="good", option2="absolute"):
        """get_phi(option, 'absolute'|'relative') (wrap_beam.cpp:712-795)."""
        if option2 not in ("absolute", "relative"):
            raise ValueError(f"invalid 2nd option: {option2}, pick from ('absolute', 'relative')")
        self._update(_UPD_LOSS)
        if option2 == "relative":
            self._update(_UPD_RELPHI, good=0)
            return self._select(self._coord("phi_r"), option)
        return self._select(self._coord("phi"), option)

    def get_losses(self, option="t"):
        if option not in ("t", "l"):
            raise ValueError(f"invalid option: {option}, pick from ('t', 'l')")
        if option == "t":
            self._update(_UPD_LOSS)
            return self._loss(0)
        self._update(_UPD_LLOSS)
        return self._loss(1)

    def get_loss_num(self, option="t"):
        if option not in ("t", "l", "all"):
            raise ValueError(f"invalid option: {option}, pick from ('t', 'l', 'all')")
        if option == "t":
            self._update(_UPD_LOSS)
            return int(self._stat("num_loss"))
        if option == "l":
            self._update(_UPD_LLOSS)
            return int(self._stat("num_lloss"))
        self._update(_UPD_LOSS)
        self._update(_UPD_LLOSS)
        self._update(_UPD_GOOD)
        return self._n - int(self._stat("num_good"))

    def _avg_sig(self, coord, option, sig):
        self._update(_UPD_LOSS)
        good = option != "transverse_good"
        self._update(_UPD_SIG if sig else _UPD_AVG, _COORD[coord], good)
        key = f"{coord}_{'sig' if sig else 'avg'}{'_good' if good else ''}"
        return self._stat(key)

    def get_avg_x(self, option="transverse_good"):
        return self._avg_sig("x", option, False)

    def get_avg_y(self, option="transverse_good"):
        return self._avg_sig("y", option, False)

    def get_avg_w(self, option="transverse_good"):
        return self._avg_sig("w", option, False)

    def get_sig_x(self, option="transverse_good"):
        return self._avg_sig("x", option, True)

    def get_sig_y(self, option="transverse_good"):
        return self._avg_sig("y", option, True)

    def get_sig_w(self, option="transverse_good"):
        return self._avg_sig("w", option, True)

    def get_avg_phi(self, option="absolute"):
        """wrap_beam.cpp:978-1011"""
        self._update(_UPD_LOSS)
        if option == "absolute":
            self._update(_UPD_AVG, _COORD["phi"], 0)
            return self._stat("phi_avg")
        if option == "relative":
            self._update(_UPD_RELPHI, good=0)
            self._update(_UPD_AVG, 6, 0)
            return self._stat("phi_avg_r")
        self._update(_UPD_GOOD)
        self._update(_UPD_AVG, _COORD["phi"], 1)
        return self._stat("phi_avg_good")

    def get_sig_phi(self, option="absolute"):
        """wrap_beam.cpp:1116-1151"""
        self._update(_UPD_LOSS)
        if option == "absolute":
            self._update(_UPD_SIG, _COORD["phi"], 0)
            return self._stat("phi_sig")
        if option == "relative":
            self._update(_UPD_RELPHI, good=0)
            self._update(_UPD_SIG, 6, 0)
            return self._stat("phi_sig_r")
        self._update(_UPD_GOOD)
        self._update(_UPD_AVG, _COORD["phi"], 1)
        self._update(_UPD_RELPHI, good=1)
        self._update(_UPD_SIG, 6, 1)
        return self._stat("phi_sig_good")

    def _emit(self, name):
        self._update(_UPD_LOSS)
        self._update(_UPD_EMIT)
        return self._stat(name) if self._n >= 2 else 0.0

    def get_emittance_x(self):
        return self._emit("x_emit")

    def get_emittance_y(self):
        return self._emit("y_emit")

    def get_emittance_z(self):
        return self._emit("z_emit")

    def get_current(self):
        """Beam current reduced by the transverse losses (wrap_beam.cpp:1286-1298)."""
        self._update(_UPD_LOSS)
        return self._scalar(2) * (1.0 - self._stat("num_loss") / self._n)

    def apply_cut(self, axis, minval, maxval):
        call("hps_beam_apply_cut", self._h, C.c_char(axis.encode()[:1]), float(minval), float(maxval))

    def translate(self, axis, val):
        a = axis.lower()
        if a not in _COORD:
            return
        call("hps_beam_translate", self._h, _COORD[a], float(val))

    # ---- additions ---------------------------------------------------------
    def monitor(self):
        """Side-effect-free statistics record (HPS_MON_* of include/hps_layout.h)."""
        out = np.zeros(24)
        call("hps_beam_monitor", self._h, dptr(out))
        return out

    def get_stat(self, name):
        """Raw device scalar (no update), e.g. 'x_sig_good', 'num_good'."""
        return self._stat(name)


class DBConnection:
    """DBConnection(db_file) over Python's sqlite3 (wrap_dbconnection.cpp,
    sql_utility.cpp:211-367).  The lattice loader is hpsim_gb300/dbloader.py.

    ``load_lib`` records the SQL extension's name without loading it: the
    loader reads the ``*_model`` columns, which do not need it."""

    def __init__(self, db_addr):
        from .dbloader import open_connection
        self._conn, self.dbs = open_connection(db_addr)
        self.libs = []
        self.model_index = {}

    def attach_db(self, db_addr, db_name=None):
        from .dbloader import attach
        attach(self, db_addr, db_name)

    def load_lib(self, lib_name):
        self.libs.append(lib_name)

    def print_dbs(self):
        if not self.dbs:
            print("DBConnection is not connected to any db.")
        for name, path in self.dbs:
            print(f"{name} -> {path}")

    def print_libs(self):
        if not self.libs:
            print("No lib is loaded for this DBConnection.")
        for name in self.libs:
            print(name)

    def clear_model_index(self):
        from .dbloader import clear_model_index
        clear_model_index(self)

    def get_epics_channels(self):
        from .dbloader import epics_channels
        return epics_channels(self)


def _db_args(dbconnection, beamline=None, what=""):
    if not isinstance(dbconnection, DBConnection):
        raise TypeError(f"{what}: needs a DBConnection")
    if beamline is not None and not isinstance(beamline, BeamLine):
        raise TypeError(f"{what}: needs a BeamLine")


def get_db_model(record_name, field_name, dbconnection):
    """get_db_model(record_name, field_name, DBConnection) -> the model
    parameter's value in the database as text, or None (hpsim_module.cpp:
    307-360)."""
    from .dbloader import get_db_model as _get
    _db_args(dbconnection, what="get_db_model")
    return _get(str(record_name), str(field_name), dbconnection)


def set_db_model(record_name, field_name, value, dbconnection, beamline):
    """set_db_model(record_name, field_name, value, DBConnection, BeamLine):
    set a model parameter in the database and hand the recomputed model
    values to the beamline's elements (hpsim_module.cpp:86-267; the lattice
    loader's dbloader.set_db_model)."""
    from .dbloader import set_db_model as _set
    _db_args(dbconnection, beamline, "set_db_model")
    _set(str(record_name), str(field_name), value, dbconnection, beamline)


def get_db_epics(pv_name, dbconnection):
    """get_db_epics(pv_name, DBConnection) -> the channel's value in the
    database as text, or None (hpsim_module.cpp:269-305)."""
    from .dbloader import get_db_epics as _get
    _db_args(dbconnection, what="get_db_epics")
    return _get(str(pv_name), dbconnection)


def set_db_epics(pv_name, value, dbconnection, beamline):
    """set_db_epics(pv_name, value, DBConnection, BeamLine)
    (hpsim_module.cpp:52-84) drives the EPICS server's PV observers
    (src/server), which this package does not include: it raises.  Model
    parameters are set with set_db_model."""
    raise NotImplementedError("set_db_epics: the EPICS server's PV observers are not part of this package; "
                              "set model parameters with set_db_model")


class BeamLine:
    """BeamLine(DBConnection) (wrap_beamline.cpp:24-41).

    Addition: ``BeamLine()`` or ``BeamLine(elements=[(type, name, params)...])``
    builds a lattice without a database; ``add_element`` appends one."""

    def __init__(self, dbconnection=None, elements=None):
        self._h = C.c_void_p()
        call("hps_beamline_create", C.byref(self._h))
        if dbconnection is not None:
            from .dbloader import generate_beamline
            elements = generate_beamline(dbconnection)
        for e in elements or ():
            self.add_element(*e)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().hps_beamline_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def add_element(self, etype, name=None, params=None, **kw):
        """add_element(type, name, params) or add_element(type, name, length=...,)."""
        if params is None:
            code, name, params = _lat.element(etype, name, **kw)
        else:
            code = _lat.TYPE_CODES[etype.lower()] if isinstance(etype, str) else int(etype)
        p = np.ascontiguousarray(params, dtype=np.float64)
        if p.shape != (_lat.NPARAM,):
            raise ValueError(f"element parameters must have {_lat.NPARAM} slots")
        call("hps_beamline_add", self._h, int(code), name.encode(), dptr(p))

    def __len__(self):
        v = C.c_uint32()
        call("hps_beamline_size", self._h, C.byref(v))
        return v.value

    def index(self, name):
        """BeamLine::GetElementModelIndex (case-insensitive)."""
        v = C.c_uint32()
        st = lib().hps_beamline_find(self._h, name.encode(), C.byref(v))
        if st != 0:
            raise KeyError(f"Invalid beamline element name, please check it! ({name})")
        return v.value

    def element(self, i):
        t = C.c_int()
        buf = C.create_string_buffer(256)
        p = np.zeros(_lat.NPARAM)
        call("hps_beamline_get", self._h, int(i), C.byref(t), buf, 256, dptr(p))
        return t.value, buf.value.decode(), p

    def set_param(self, name_or_index, key, value):
        """Element setter (RFGap::SetRFAmplitude, Quad::SetGradient, ...)."""
        i = self.index(name_or_index) if isinstance(name_or_index, str) else int(name_or_index)
        t, _, _ = self.element(i)
        call("hps_beamline_set_param", self._h, i, _lat.param_index(t, key), float(value))

    def get_element_names(self, start="", end="", type=""):  # noqa: A002
        """wrap_beamline.cpp:92-110: names in [start, end] (inclusive), by type."""
        n = len(self)
        i0 = self.index(start) if start else 0
        i1 = self.index(end) if end else n - 1
        out = []
        for i in range(i0, i1 + 1):
            t, nm, _ = self.element(i)
            if not type or _lat.TYPE_NAMES[t] == type:
                out.append(nm)
        return out or None

    def print_out(self):
        for i in range(len(self)):
            t, nm, p = self.element(i)
            print(f"{nm}: {_lat.TYPE_NAMES[t]}, length = {p[0]}, aperture = {p[1]}")

    def print_range(self, start_element, end_element):
        for i in range(self.index(start_element), self.index(end_element) + 1):
            t, nm, p = self.element(i)
            print(f"{nm}: {_lat.TYPE_NAMES[t]}, length = {p[0]}, aperture = {p[1]}")


class SpaceCharge:
    """SpaceCharge(nr, nz, interval=0.01, adj_bunch=0, type='scheff')
    (wrap_spacecharge.cpp:31-54)."""

    _P = {"interval": 0, "adj_bunch": 1, "adj_bunch_cutoff_w": 2, "mesh_size_cutoff_w": 3,
          "remesh_threshold": 4, "fraction": 5, "nr": 6, "nz": 7}

    def __init__(self, nr, nz, interval=0.01, adj_bunch=0, type="scheff"):  # noqa: A002
        if type != "scheff":
            raise ValueError(f"SpaceCharge type: {type} is not supported.")
        self._h = C.c_void_p()
        call("hps_scheff_create", int(nr), int(nz), int(adj_bunch), C.byref(self._h))
        self.set_interval(interval)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().hps_scheff_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def _set(self, k, v):
        call("hps_scheff_set", self._h, self._P[k], float(v))

    def _get(self, k):
        v = C.c_double()
        call("hps_scheff_get", self._h, self._P[k], C.byref(v))
        return v.value

    def set_mesh_size(self, nr, nz):
        call("hps_scheff_set_mesh_size", self._h, int(nr), int(nz))

    def get_mesh_size(self):
        return [int(self._get("nr")), int(self._get("nz"))]

    def get_interval(self):
        return self._get("interval")

    def set_interval(self, v):
        self._set("interval", v)

    def get_adj_bunch(self):
        return int(self._get("adj_bunch"))

    def set_adj_bunch(self, v):
        self._set("adj_bunch", int(v))

    def get_adj_bunch_cutoff_w(self):
        return self._get("adj_bunch_cutoff_w")

    def set_adj_bunch_cutoff_w(self, v):
        self._set("adj_bunch_cutoff_w", v)

    def get_mesh_size_cutoff_w(self):
        return self._get("mesh_size_cutoff_w")

    def set_mesh_size_cutoff_w(self, v):
        self._set("mesh_size_cutoff_w", v)

    def get_remesh_threshold(self):
        return self._get("remesh_threshold")

    def set_remesh_threshold(self, v):
        self._set("remesh_threshold", v)

    def get_counter(self, name):
        """Counters and flags kept on the device (not in the reference's API):
        'solves' (field solves since creation), 'stat_sweeps' (kicks of an
        FP32 beam whose statistics took the loss-test and moments sweeps),
        'tensor_cores' (1: FP32 beams' contractions run on the tensor cores),
        'tc_error' (1: a bounded wait of that kernel gave up),
        'surrogate_tc_layers' (layers of the attached network on the tensor
        cores), 'surrogate_tc_error' (1: a bounded wait of one gave up)."""
        out = C.c_double()
        call("hps_scheff_get", self._h, {"solves": 8, "stat_sweeps": 9, "tensor_cores": 11, "tc_error": 12,
                                         "surrogate_tc_layers": 14, "surrogate_tc_error": 15}[name], C.byref(out))
        return int(out.value)

    def set_contraction(self, kernel):
        """Contraction kernel of FP32 beams (not in the reference's API):
        'tensor' (the default: split-BF16 tcgen05 products where the mesh
        allows) or 'cuda' (the FP32 ring convolution on CUDA cores)."""
        call("hps_scheff_set", self._h, 10, {"tensor": 0.0, "cuda": 1.0}[kernel])

    def set_surrogate_kernel(self, kernel):
        """Kernel of the attached surrogate's layers (not in the reference's
        API): 'cuda' (the default: the CUDA-core convolution, slightly faster
        on the one plane a solver evaluates) or 'tensor' (tcgen05 BF16 MMA
        where the layer's shape allows; what training uses for its batches)."""
        call("hps_scheff_set", self._h, 13, {"tensor": 0.0, "cuda": 1.0}[kernel])

    def set_surrogate(self, net, tol=0.02, n_samples=64):
        """Attach a trained field surrogate (not in the reference's API):
        `net` is a surrogate.Network or its saved state (dict / npz).  Kicks
        on the network's mesh (FP64 and FP32 beams) then take the network's
        field when its relative residual against the plain sum at n_samples
        spot points is <= tol, and the plain Green's table and contraction
        otherwise."""
        from . import surrogate
        ex = surrogate.export(net.state() if hasattr(net, "state") else net)
        n = len(ex["weights"])
        arch = np.ascontiguousarray(ex["arch"], np.int32).reshape(-1)
        skip = np.ascontiguousarray(ex["skip"], np.int32)
        wts = [np.ascontiguousarray(w, np.uint16) for w in ex["weights"]]
        bis = [np.ascontiguousarray(b, np.float32) for b in ex["biases"]]
        wp = (C.c_void_p * n)(*[w.ctypes.data for w in wts])
        bp = (C.c_void_p * n)(*[b.ctypes.data for b in bis])
        call("hps_scheff_set_surrogate", self._h, n, arch.ctypes.data_as(C.POINTER(C.c_int)), int(ex["gmean_after"]),
             skip.ctypes.data_as(C.POINTER(C.c_int)), wp, bp, int(ex["nr"]), int(ex["nz"]), float(ex["out_scale"]),
             float(tol), int(n_samples))

    def clear_surrogate(self):
        call("hps_scheff_clear_surrogate", self._h)

    def surrogate_stats(self):
        """(kicks whose field the surrogate gave, kicks that fell back to the
        plain contraction, the last spot residual)."""
        a, r, res = C.c_double(), C.c_double(), C.c_double()
        call("hps_scheff_surrogate_stats", self._h, C.byref(a), C.byref(r), C.byref(res))
        return int(a.value), int(r.value), res.value


class Simulator:
    """Simulator(beam=, beamline=, spch=None) (wrap_simulator.cpp:27-54).

    Holds references to its beam, beamline and solver (the reference kept
    raw pointers)."""

    def __init__(self, beam, beamline, spch=None):
        self.beam, self.beamline, self.spch = beam, beamline, spch
        self._h = C.c_void_p()
        call("hps_sim_create", beam.handle, beamline.handle, spch.handle if spch is not None else None,
             C.byref(self._h))
        self._mon = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().hps_sim_destroy(h)
            except Exception:
                pass
            self._h = None

    def simulate(self, start=None, end=None):
        """simulate() or simulate(start_element, end_element), inclusive.

        Element names as in the reference; integer indices are accepted too."""
        s = -1 if start is None else (self.beamline.index(start) if isinstance(start, str) else int(start))
        e = -1 if end is None else (self.beamline.index(end) if isinstance(end, str) else int(end))
        call("hps_sim_simulate", self._h, s, e)

    def reset(self):
        call("hps_sim_reset", self._h)

    def set_space_charge(self, on_off):
        call("hps_sim_set_space_charge", self._h, 1 if on_off.lower() == "on" else 0)

    # ---- additions ---------------------------------------------------------
    def enable_monitor(self, on=True):
        """Record HPS_NMON statistics after every element into ``self.monitor``."""
        if on:
            self._mon = np.zeros((len(self.beamline), 24))
            call("hps_sim_set_monitor", self._h, dptr(self._mon), len(self.beamline))
        else:
            self._mon = None
            call("hps_sim_set_monitor", self._h, None, 0)

    @property
    def monitor(self):
        return self._mon

    def use_graph(self, on=True):
        call("hps_sim_use_graph", self._h, 1 if on else 0)

    PHASES = ("drift", "quad", "gap1", "gap2", "other", "sc_stats", "sc_mesh", "sc_kick", "monitor")

    def profile(self, on=True):
        """Per-phase CUDA-event timers (launches go direct, not through a graph)."""
        call("hps_sim_profile", self._h, 1 if on else 0)

    def profile_read(self, reset=True):
        """{phase: (milliseconds, phase count)} accumulated since the last reset."""
        ms = np.zeros(len(self.PHASES))
        cnt = np.zeros(len(self.PHASES), dtype=np.uint64)
        call("hps_sim_profile_read", self._h, dptr(ms), cnt.ctypes.data_as(C.POINTER(C.c_uint64)), int(reset))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.PHASES)}

    def last_time_ms(self):
        v = C.c_double()
        call("hps_sim_last_time_ms", self._h, C.byref(v))
        return v.value

    SHAPE_KEYS = ("contraction", "deposit_blocks_per_sm", "sweep_blocks_per_sm", "deposit_aggregate",
                  "deposit_threads")

    def autotune(self, start=None, end=None, reps=3):
        """Pick the launch shape of this simulation by timing candidates on
        the GPU (no reference counterpart): returns {"shape": {...}, "ms":
        [candidate times]}; the beam, solver and engine state are left as
        they were.  A shape found before for the same device, mesh, size
        class and precision is reused without timing ("ms" empty)."""
        return _autotune("hps_sim_autotune", self._h, self.beamline, start, end, reps)

    def get_shape(self):
        sh = np.zeros(len(self.SHAPE_KEYS), np.int32)
        call("hps_sim_get_shape", self._h, sh.ctypes.data_as(C.POINTER(C.c_int)))
        return dict(zip(self.SHAPE_KEYS, (int(v) for v in sh)))

    def set_shape(self, shape):
        sh = np.array([int(shape.get(k, 0)) for k in self.SHAPE_KEYS], np.int32)
        call("hps_sim_set_shape", self._h, sh.ctypes.data_as(C.POINTER(C.c_int)))


def _autotune(fn, handle, bl, start, end, reps):
    s = -1 if start is None else (bl.index(start) if isinstance(start, str) else int(start))
    e = -1 if end is None else (bl.index(end) if isinstance(end, str) else int(end))
    sh = np.zeros(len(Simulator.SHAPE_KEYS), np.int32)
    ms = np.zeros(64)
    n = C.c_uint32()
    call(fn, handle, s, e, int(reps), sh.ctypes.data_as(C.POINTER(C.c_int)), dptr(ms), len(ms), C.byref(n))
    return {"shape": dict(zip(Simulator.SHAPE_KEYS, (int(v) for v in sh))), "ms": ms[:n.value].tolist()}


def kernel_launch_count():
    return int(lib().hps_kernel_launch_count())


class Batch:
    """Addition (no reference counterpart): several simulators, each with its
    own beam and SpaceCharge, advanced by one graph launch of per-simulator
    child graphs (or, with set_lockstep, one launch per kernel for all
    beams when their launch sequences match).  ``simulate`` takes the same start/end as
    Simulator.simulate; the results are those of running each simulator
    alone."""

    def __init__(self, simulators):
        self._sims = list(simulators)  # keep the simulators (and their beams) alive
        arr = (C.c_void_p * len(self._sims))(*[s._h.value for s in self._sims])
        self._h = C.c_void_p()
        call("hps_batch_create", C.cast(arr, C.POINTER(C.c_void_p)), len(self._sims), C.byref(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().hps_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def simulate(self, start=None, end=None):
        """Element names resolve in the first simulator's beamline."""
        bl = self._sims[0].beamline
        s = -1 if start is None else (bl.index(start) if isinstance(start, str) else int(start))
        e = -1 if end is None else (bl.index(end) if isinstance(end, str) else int(end))
        call("hps_batch_simulate", self._h, s, e)

    def last_time_ms(self):
        v = C.c_double()
        call("hps_batch_last_time_ms", self._h, C.byref(v))
        return v.value

    def set_lockstep(self, on=True):
        """Lockstep form on or off (the default): one launch per kernel for
        every beam when the simulators issue the same launch sequence, else a
        graph of per-simulator child graphs (results agree to FP32
        rounding)."""
        call("hps_batch_set_lockstep", self._h, 1 if on else 0)

    def last_mode(self):
        """("lockstep", "") or ("graphs", why) for the last simulate."""
        on = C.c_int()
        why = C.create_string_buffer(256)
        call("hps_batch_last_mode", self._h, C.byref(on), why, 256)
        return ("lockstep", "") if on.value else ("graphs", why.value.decode())

    def autotune(self, start=None, end=None, reps=3):
        """Simulator.autotune for the whole batch (objective: the batch's
        launch; the shape is applied to every simulator)."""
        return _autotune("hps_batch_autotune", self._h, self._sims[0].beamline, start, end, reps)
