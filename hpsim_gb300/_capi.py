"""ctypes binding of libhpsim_gb300.so (the C ABI of include/hpsim_gb300.h).

The library is built in-tree by hpsim_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback for the tracking path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

HPS_OK = 0
_lib = None


class HPSimError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


def library_path():
    return _build.LIB


def lib():
    """Load libhpsim_gb300.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python hpsim_gb300/build.py)")
    L = C.CDLL(path)
    vp, d, u32, i32, u64 = C.c_void_p, C.c_double, C.c_uint32, C.c_int, C.c_uint64
    dp, up, ip, pvp = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_int), C.POINTER(C.c_void_p)
    cp = C.c_char_p
    st = C.c_int
    sig = {
        "hps_abi_version": (i32, []),
        "hps_last_error": (cp, []),
        "hps_status_string": (cp, [i32]),
        "hps_set_gpu": (st, [i32]),
        "hps_kernel_launch_count": (u64, []),
        "hps_beam_create": (st, [u32, d, d, d, i32, pvp]),
        "hps_beam_destroy": (st, [vp]),
        "hps_beam_info": (st, [vp, up, ip]),
        "hps_beam_set_distribution": (st, [vp, dp, dp, dp, dp, dp, dp, up, up]),
        "hps_beam_set_waterbag": (st, [vp, dp, d, d, d, u32]),
        "hps_beam_set_dc": (st, [vp, dp, d, d, d, u32]),
        "hps_beam_get_coord": (st, [vp, i32, dp]),
        "hps_beam_get_loss": (st, [vp, i32, up]),
        "hps_beam_save": (st, [vp, i32]),
        "hps_beam_restore": (st, [vp, i32]),
        "hps_beam_set_ref_w": (st, [vp, d]),
        "hps_beam_set_ref_phi": (st, [vp, d]),
        "hps_beam_get_ref": (st, [vp, dp, dp]),
        "hps_beam_set_frequency": (st, [vp, d]),
        "hps_beam_get_scalar": (st, [vp, i32, dp]),
        "hps_beam_update": (st, [vp, i32, i32, i32]),
        "hps_beam_get_stat": (st, [vp, i32, dp]),
        "hps_beam_apply_cut": (st, [vp, C.c_char, d, d]),
        "hps_beam_translate": (st, [vp, i32, d]),
        "hps_beam_monitor": (st, [vp, dp]),
        "hps_plot_points": (st, [vp, i32, i32, vp, i32]),
        "hps_plot_maxmin": (st, [vp, i32, i32, i32, dp]),
        "hps_plot_histogram": (st, [vp, i32, u32, d, d, vp, i32]),
        "hps_plot_histogram2d": (st, [vp, i32, i32, u32, u32, dp, vp, i32]),
        "hps_beamline_create": (st, [pvp]),
        "hps_beamline_destroy": (st, [vp]),
        "hps_beamline_add": (st, [vp, i32, cp, dp]),
        "hps_beamline_size": (st, [vp, up]),
        "hps_beamline_find": (st, [vp, cp, up]),
        "hps_beamline_get": (st, [vp, u32, ip, C.c_char_p, C.c_size_t, dp]),
        "hps_beamline_set_param": (st, [vp, u32, i32, d]),
        "hps_scheff_create": (st, [u32, u32, u32, pvp]),
        "hps_scheff_destroy": (st, [vp]),
        "hps_scheff_set": (st, [vp, i32, d]),
        "hps_scheff_get": (st, [vp, i32, dp]),
        "hps_scheff_set_mesh_size": (st, [vp, u32, u32]),
        "hps_scheff_snapshot": (st, [vp, i32, dp, dp, dp]),
        "hps_scheff_set_surrogate": (st, [vp, i32, ip, i32, ip, C.POINTER(vp), C.POINTER(vp), u32, u32, d, d, u32]),
        "hps_scheff_clear_surrogate": (st, [vp]),
        "hps_scheff_surrogate_stats": (st, [vp, dp, dp, dp]),
        "hps_scheff_field": (st, [u32, u32, dp, dp, dp]),
        "hps_scheff_field_noalloc": (st, [u32, u32, vp, dp, vp, vp]),
        "hps_scheff_field_f32": (st, [u32, u32, dp, dp, dp]),
        "hps_scheff_field_f32_kernel": (st, [u32, u32, dp, dp, dp, i32]),
        "hps_sim_create": (st, [vp, vp, vp, pvp]),
        "hps_sim_destroy": (st, [vp]),
        "hps_sim_simulate": (st, [vp, i32, i32]),
        "hps_sim_reset": (st, [vp]),
        "hps_sim_set_space_charge": (st, [vp, i32]),
        "hps_sim_set_monitor": (st, [vp, dp, u32]),
        "hps_sim_use_graph": (st, [vp, i32]),
        "hps_sim_synchronize": (st, [vp]),
        "hps_sim_last_time_ms": (st, [vp, dp]),
        "hps_sim_profile": (st, [vp, i32]),
        "hps_sim_profile_read": (st, [vp, dp, C.POINTER(C.c_uint64), i32]),
        "hps_nn_conv_forward": (st, [ip, vp, vp, vp, i32, vp, vp, vp]),
        "hps_nn_conv_forward_tc": (st, [ip, vp, vp, vp, i32, vp, vp, vp]),
        "hps_nn_conv_tc_tile_bytes": (st, [ip, C.POINTER(C.c_uint64)]),
        "hps_nn_conv_tc_prepare": (st, [ip, vp, vp, vp]),
        "hps_nn_conv_forward_tiles": (st, [ip, vp, vp, vp, i32, vp, vp, vp, vp]),
        "hps_nn_conv_backward": (st, [ip, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]),
        "hps_nn_gmean_forward": (st, [vp, i32, i32, vp]),
        "hps_nn_gmean_backward": (st, [vp, i32, i32, vp]),
        "hps_nn_mse": (st, [vp, vp, C.c_int64, vp, C.c_int64, vp, vp, i32, vp]),
        "hps_nn_add": (st, [vp, vp, vp, C.c_int64, i32, vp]),
        "hps_nn_adam": (st, [vp, vp, vp, vp, vp, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, i32, vp]),
        "hps_nn_convert": (st, [vp, vp, C.c_int64, i32, vp]),
        "hps_batch_create": (st, [pvp, u32, pvp]),
        "hps_batch_destroy": (st, [vp]),
        "hps_batch_simulate": (st, [vp, i32, i32]),
        "hps_batch_last_time_ms": (st, [vp, dp]),
        "hps_batch_set_lockstep": (st, [vp, i32]),
        "hps_batch_last_mode": (st, [vp, ip, C.c_char_p, C.c_size_t]),
        "hps_sim_autotune": (st, [vp, i32, i32, i32, ip, dp, u32, C.POINTER(u32)]),
        "hps_batch_autotune": (st, [vp, i32, i32, i32, ip, dp, u32, C.POINTER(u32)]),
        "hps_sim_get_shape": (st, [vp, ip]),
        "hps_sim_set_shape": (st, [vp, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status, what=""):
    if status != HPS_OK:
        msg = lib().hps_last_error().decode(errors="replace")
        raise HPSimError(status, f"{what}: {msg}" if what else msg)


def call(name, *args):
    check(getattr(lib(), name)(*args), name)


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))
