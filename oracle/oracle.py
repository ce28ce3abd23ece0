"""ctypes binding of the FP64 CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The product (hpsim_gb300/) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
NPARAM = 32
NMON = 24
NSTAT = 27
ST = {n: i for i, n in enumerate(
    "x_avg x_avg_good xp_avg y_avg y_avg_good yp_avg phi_avg phi_avg_r phi_avg_good "
    "w_avg w_avg_good x_sig x_sig_good xp_sig y_sig y_sig_good yp_sig phi_sig phi_sig_r "
    "phi_sig_good w_sig w_sig_good x_emit y_emit z_emit r_max abs_phi_max".split())}


def build(quiet=True):
    """Compile oracle/liboracle.so (and oracle/_ref when the reference tree is
    present) with the Makefile beside this file."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, d, u32, i32 = C.c_void_p, C.c_double, C.c_uint32, C.c_int
        dp, up, ip = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_int)
        sig = {
            "orc_beam_create": (vp, [u32, d, d, d]),
            "orc_beam_free": (None, [vp]),
            "orc_beam_set_distribution": (None, [vp, dp, dp, dp, dp, dp, dp, up, up]),
            "orc_beam_set_waterbag": (None, [vp] + [d] * 12 + [u32]),
            "orc_beam_set_dc": (None, [vp] + [d] * 9 + [u32]),
            "orc_beam_set_ref_w": (None, [vp, d]),
            "orc_beam_set_ref_phi": (None, [vp, d]),
            "orc_beam_save": (None, [vp, i32]),
            "orc_beam_restore": (i32, [vp, i32]),
            "orc_beam_update_loss": (None, [vp]),
            "orc_beam_update_longitudinal_loss": (None, [vp]),
            "orc_beam_update_good_count": (None, [vp]),
            "orc_beam_update_avg": (None, [vp, i32, i32]),
            "orc_beam_update_sig": (None, [vp, i32, i32]),
            "orc_beam_update_emittance": (None, [vp]),
            "orc_beam_update_relative_phi": (None, [vp, i32]),
            "orc_beam_update_stat_for_sc": (None, [vp]),
            "orc_beam_monitor": (None, [vp, dp]),
            "orc_beam_apply_cut": (None, [vp, C.c_char, d, d]),
            "orc_beam_shift": (None, [vp, i32, d]),
            "orc_scheff_create": (vp, [u32, u32, u32]),
            "orc_scheff_free": (None, [vp]),
            "orc_scheff_set_interval": (None, [vp, d]),
            "orc_scheff_green_table": (None, [vp, d, d, u32, d, u32]),
            "orc_scheff_deposit": (None, [vp, vp, d, d]),
            "orc_scheff_contract": (None, [vp]),
            "orc_scheff_start": (None, [vp, vp, d]),
            "orc_sim_create": (vp, [vp, u32, ip, dp, vp]),
            "orc_sim_free": (None, [vp]),
            "orc_sim_reset": (None, [vp]),
            "orc_sim_simulate": (i32, [vp, i32, i32]),
            "orc_sim_set_monitor": (None, [vp, dp]),
            "orc_num_threads": (i32, []),
            "orc_set_threads": (None, [i32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class _BeamStruct(C.Structure):
    _fields_ = [("n", C.c_uint32), ("mass", C.c_double), ("charge", C.c_double),
                ("current", C.c_double), ("freq", C.c_double), ("design_w", C.c_double),
                ("grid_size", C.c_uint32), ("blck_size", C.c_uint32),
                ("x", C.POINTER(C.c_double)), ("xp", C.POINTER(C.c_double)),
                ("y", C.POINTER(C.c_double)), ("yp", C.POINTER(C.c_double)),
                ("phi", C.POINTER(C.c_double)), ("phi_r", C.POINTER(C.c_double)),
                ("w", C.POINTER(C.c_double)), ("loss", C.POINTER(C.c_uint32)),
                ("lloss", C.POINTER(C.c_uint32)), ("st", C.c_double * NSTAT),
                ("num_loss", C.c_uint32), ("num_lloss", C.c_uint32), ("num_good", C.c_uint32)]


class _ScheffStruct(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("nz", C.c_uint32), ("nx_init", C.c_uint32),
                ("nz_init", C.c_uint32), ("adj_bunch", C.c_uint32),
                ("fraction", C.c_double), ("interval", C.c_double),
                ("interval_init", C.c_double), ("adj_bunch_w", C.c_double),
                ("mesh_w", C.c_double), ("sigr_old", C.c_double), ("sigz_old", C.c_double),
                ("gm_old", C.c_double), ("good_cnt_old", C.c_uint32),
                ("remesh_val", C.c_double), ("dr", C.c_double), ("dz", C.c_double),
                ("num_on_mesh", C.c_uint32), ("bin", C.POINTER(C.c_double)),
                ("fld1", C.POINTER(C.c_double)), ("fld2", C.POINTER(C.c_double))]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class Beam:
    def __init__(self, num, mass=939.294, charge=-1.0, current=0.015):
        self.h = lib().orc_beam_create(int(num), mass, charge, current)
        self.s = C.cast(self.h, C.POINTER(_BeamStruct)).contents
        self.n = int(num)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_beam_free(self.h)
            self.h = None

    def set_waterbag(self, twiss, sync_phi, sync_w, freq, seed):
        lib().orc_beam_set_waterbag(self.h, *[float(t) for t in twiss], float(sync_phi),
                                    float(sync_w), float(freq), int(seed))

    def set_dc(self, twiss6, dphi, sync_phi, sync_w, seed):
        lib().orc_beam_set_dc(self.h, *[float(t) for t in twiss6], float(dphi),
                              float(sync_phi), float(sync_w), int(seed))

    def set_distribution(self, x, xp, y, yp, phi, w, loss=None, lloss=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, xp, y, yp, phi, w)]
        lo = np.ascontiguousarray(loss, dtype=np.uint32) if loss is not None else None
        ll = np.ascontiguousarray(lloss, dtype=np.uint32) if lloss is not None else None
        lib().orc_beam_set_distribution(self.h, *[_dp(a) for a in arrs],
                                        _up(lo) if lo is not None else None,
                                        _up(ll) if ll is not None else None)

    def set_ref_w(self, w):
        lib().orc_beam_set_ref_w(self.h, float(w))

    def set_ref_phi(self, p):
        lib().orc_beam_set_ref_phi(self.h, float(p))

    def set_frequency(self, f):
        self.s.freq = float(f)

    def arr(self, name):
        if name in ("loss", "lloss"):
            return np.ctypeslib.as_array(getattr(self.s, name), shape=(self.n,)).copy()
        return np.ctypeslib.as_array(getattr(self.s, name), shape=(self.n,)).copy()

    def coords(self):
        return {k: self.arr(k) for k in ("x", "xp", "y", "yp", "phi", "w", "loss", "lloss")}

    def stat(self, name):
        return self.s.st[ST[name]]

    def monitor(self):
        out = np.zeros(NMON)
        lib().orc_beam_monitor(self.h, _dp(out))
        return out


class Scheff:
    def __init__(self, nr, nz, interval=0.01, adj_bunch=0):
        self.h = lib().orc_scheff_create(int(nr), int(nz), int(adj_bunch))
        self.s = C.cast(self.h, C.POINTER(_ScheffStruct)).contents
        lib().orc_scheff_set_interval(self.h, float(interval))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scheff_free(self.h)
            self.h = None

    def set(self, **kw):
        for k, v in kw.items():
            setattr(self.s, {"remesh_threshold": "remesh_val", "adj_bunch_cutoff_w": "adj_bunch_w",
                             "mesh_size_cutoff_w": "mesh_w"}.get(k, k), v)

    def tables(self):
        nx, nz = self.s.nx, self.s.nz
        bin_ = np.ctypeslib.as_array(self.s.bin, shape=(nz * nx,)).copy()
        fld1 = np.ctypeslib.as_array(self.s.fld1, shape=((nx + 1) * nx * nz * 2,)).copy()
        fld2 = np.ctypeslib.as_array(self.s.fld2, shape=((nz + 1) * (nx + 1) * 2,)).copy()
        return bin_, fld1, fld2


class Sim:
    def __init__(self, beam: Beam, types, params, spch: Scheff | None = None):
        self.beam, self.spch = beam, spch
        self.types = np.ascontiguousarray(types, dtype=np.int32)
        self.params = np.ascontiguousarray(params, dtype=np.float64)
        self.n = len(self.types)
        self.mon = np.zeros((self.n, NMON))
        self.h = lib().orc_sim_create(beam.h, self.n, self.types.ctypes.data_as(C.POINTER(C.c_int)),
                                      _dp(self.params), spch.h if spch else None)
        lib().orc_sim_set_monitor(self.h, _dp(self.mon))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_free(self.h)
            self.h = None

    def simulate(self, start=-1, end=-1):
        rc = lib().orc_sim_simulate(self.h, int(start), int(end))
        if rc != 0:
            raise ValueError("oracle: malformed lattice")
        return self.mon


def run(elems, num, spch_args=None, spch_set=None, seed=12345, twiss=None, w0=0.75, phi0=0.0,
        freq=201.25, start=-1, end=-1, late=False):
    """Build a waterbag beam, run the lattice, return (monitor, coords).
    late: the beam is configured after the simulator is created."""
    from hpsim_gb300 import lattices as L
    types, params, _ = L.lattice_arrays(elems)
    b = Beam(num)

    def configure():
        b.set_waterbag(twiss or L.waterbag_twiss(), phi0, w0, freq, seed)
        b.set_ref_w(w0)
        b.set_ref_phi(phi0)

    if not late:
        configure()
    sp = None
    if spch_args is not None:
        sp = Scheff(*spch_args)
        if spch_set:
            sp.set(**spch_set)
    sim = Sim(b, types, params, sp)
    if late:
        configure()
    mon = sim.simulate(start, end).copy()
    return mon, b.coords()
