"""Headless plot data of a beam (the reference's online-mode graphics
kernels, src/graphics/inc/graphics_kernel.cu, computed into plain memory):
phase-space points, the max/min that frames a plot, and 1D / 2D histograms.

Each function returns numpy arrays; ``device_ptr=`` writes into caller
device memory instead (an integer address of a buffer on the beam's GPU,
e.g. ``torch_tensor.data_ptr()``) and returns None."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import call, dptr

COORDS = {"x": 0, "xp": 1, "y": 2, "yp": 3, "phi": 4, "w": 5, "phi_r": 6}


def _c(name):
    if name not in COORDS:
        raise ValueError(f"unknown coordinate {name!r}, pick from {tuple(COORDS)}")
    return COORDS[name]


def phase_space(beam, cx="x", cy="xp", device_ptr=None):
    """(n, 2) float32 points; lost particles at the origin."""
    if device_ptr is not None:
        call("hps_plot_points", beam.handle, _c(cx), _c(cy), C.c_void_p(device_ptr), 1)
        return None
    out = np.empty((beam.get_size(), 2), dtype=np.float32)
    call("hps_plot_points", beam.handle, _c(cx), _c(cy), out.ctypes.data_as(C.c_void_p), 0)
    return out


def maxmin(beam, cx="x", cy="xp", live_only=True):
    """(xmax, xmin, ymax, ymin)."""
    out = np.empty(4, dtype=np.float64)
    call("hps_plot_maxmin", beam.handle, _c(cx), _c(cy), int(bool(live_only)), dptr(out))
    return tuple(float(v) for v in out)


def histogram(beam, coord, nbins, vmin, vmax, device_ptr=None):
    """uint32 counts of live particles in nbins bins over [vmin, vmax]."""
    if device_ptr is not None:
        call("hps_plot_histogram", beam.handle, _c(coord), int(nbins), float(vmin), float(vmax),
             C.c_void_p(device_ptr), 1)
        return None
    out = np.empty(int(nbins), dtype=np.uint32)
    call("hps_plot_histogram", beam.handle, _c(coord), int(nbins), float(vmin), float(vmax),
         out.ctypes.data_as(C.c_void_p), 0)
    return out


def histogram2d(beam, cx, cy, nx, ny, frame=None, device_ptr=None):
    """(ny, nx) uint32 counts of live particles; frame = (xmax, xmin, ymax,
    ymin), by default maxmin(beam, cx, cy)."""
    mm = np.ascontiguousarray(frame if frame is not None else maxmin(beam, cx, cy), dtype=np.float64)
    if device_ptr is not None:
        call("hps_plot_histogram2d", beam.handle, _c(cx), _c(cy), int(nx), int(ny), dptr(mm),
             C.c_void_p(device_ptr), 1)
        return None
    out = np.empty((int(ny), int(nx)), dtype=np.uint32)
    call("hps_plot_histogram2d", beam.handle, _c(cx), _c(cy), int(nx), int(ny), dptr(mm),
         out.ctypes.data_as(C.c_void_p), 0)
    return out


def bin_centres_2d(frame, nx, ny):
    """SetHistogram2DCoordinateDataKernel (graphics_kernel.cu:313-330): the
    (x, y) centre of every 2D bin, row iy."""
    xmax, xmin, ymax, ymin = frame
    dx, dy = (xmax - xmin) / nx, (ymax - ymin) / ny
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny))
    return np.stack([(xmin + dx * (0.5 + ix)).astype(np.float32), (ymin + dy * (0.5 + iy)).astype(np.float32)], -1)
