"""ctypes driver for oracle/_ref/libhpsref.so: the reference's own tracking
code compiled for the host CPU (see ref_harness.cpp).

TEST INFRASTRUCTURE ONLY.  Available only where the reference tree exists at
build time; tests that use it skip elsewhere and fall back to the golden
fixtures it produced (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libhpsref.so")
NMON = 24
_lib = None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        vp, d, u32, i32 = C.c_void_p, C.c_double, C.c_uint32, C.c_int
        dp, up = C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        sig = {
            "ref_beam_create": (vp, [u32, d, d, d]),
            "ref_beam_free": (None, [vp]),
            "ref_beam_set_waterbag": (None, [vp, dp, d, d, d, u32]),
            "ref_beam_set_distribution": (None, [vp, dp, dp, dp, dp, dp, dp, up, up]),
            "ref_beam_set_dc": (None, [vp] + [d] * 9 + [u32]),
            "ref_scheff_tables": (None, [dp, dp, dp]),
            "ref_scheff_mesh_params": (None, [dp]),
            "ref_beam_set_ref_w": (None, [vp, d]),
            "ref_beam_set_ref_phi": (None, [vp, d]),
            "ref_beam_set_frequency": (None, [vp, d]),
            "ref_beam_get": (None, [vp, dp, dp, dp, dp, dp, dp, up, up]),
            "ref_beam_monitor": (None, [vp, dp]),
            "ref_beamline_create": (vp, []),
            "ref_beamline_free": (None, [vp]),
            "ref_beamline_add": (i32, [vp, i32, C.c_char_p, dp]),
            "ref_scheff_create": (vp, [u32, u32, i32, d, d, d, d]),
            "ref_scheff_free": (None, [vp]),
            "ref_sim_create": (vp, [vp, vp, vp]),
            "ref_sim_free": (None, [vp]),
            "ref_sim_simulate": (i32, [vp, vp, i32, i32, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def run(elems, num, spch=None, seed=12345, twiss=None, w0=0.75, phi0=0.0, freq=201.25,
        dist=None, mass=939.294, charge=-1.0, current=0.015, late=False):
    """Run the reference on a waterbag (or given) beam; return (monitor, coords).

    spch: None or dict(nr, nz, interval, adj_bunch, remesh_threshold,
    adj_bunch_cutoff_w, mesh_size_cutoff_w).  late: the beam's distribution
    and reference energy / phase are set after the simulator is created."""
    from hpsim_gb300 import lattices as L
    lb = lib()
    b = lb.ref_beam_create(int(num), mass, charge, current)

    def configure():
        if dist is None:
            tw = np.ascontiguousarray(twiss or L.waterbag_twiss(), dtype=np.float64)
            lb.ref_beam_set_waterbag(b, _dp(tw), phi0, w0, freq, int(seed))
        else:
            arrs = [np.ascontiguousarray(dist[k], dtype=np.float64) for k in ("x", "xp", "y", "yp", "phi", "w")]
            lo = np.ascontiguousarray(dist["loss"], dtype=np.uint32) if "loss" in dist else None
            ll = np.ascontiguousarray(dist["lloss"], dtype=np.uint32) if "lloss" in dist else None
            lb.ref_beam_set_distribution(b, *[_dp(a) for a in arrs], _up(lo) if lo is not None else None,
                                         _up(ll) if ll is not None else None)
            lb.ref_beam_set_frequency(b, freq)
        lb.ref_beam_set_ref_w(b, w0)
        lb.ref_beam_set_ref_phi(b, phi0)

    if not late:
        configure()
    bl = lb.ref_beamline_create()
    for t, name, p in elems:
        pp = np.ascontiguousarray(p, dtype=np.float64)
        if lb.ref_beamline_add(bl, int(t), name.encode(), _dp(pp)) != 0:
            raise ValueError(f"element {name}")
    sp = None
    if spch is not None:
        s = dict(interval=0.01, adj_bunch=0, remesh_threshold=0.05, adj_bunch_cutoff_w=0.0,
                 mesh_size_cutoff_w=0.0)
        s.update(spch)
        sp = lb.ref_scheff_create(s["nr"], s["nz"], s["adj_bunch"], s["interval"],
                                  s["remesh_threshold"], s["adj_bunch_cutoff_w"], s["mesh_size_cutoff_w"])
    sim = lb.ref_sim_create(b, bl, sp)
    if late:
        configure()
    mon = np.zeros((len(elems), NMON))
    rc = lb.ref_sim_simulate(sim, b, -1, -1, _dp(mon))
    out = {k: np.zeros(num) for k in ("x", "xp", "y", "yp", "phi", "w")}
    out["loss"] = np.zeros(num, dtype=np.uint32)
    out["lloss"] = np.zeros(num, dtype=np.uint32)
    lb.ref_beam_get(b, *[_dp(out[k]) for k in ("x", "xp", "y", "yp", "phi", "w")], _up(out["loss"]),
                    _up(out["lloss"]))
    lb.ref_sim_free(sim)
    if sp:
        lb.ref_scheff_free(sp)
    lb.ref_beamline_free(bl)
    lb.ref_beam_free(b)
    if rc != 0:
        raise ValueError("reference: malformed lattice")
    return mon, out
