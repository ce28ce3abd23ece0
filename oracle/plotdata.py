"""Test infrastructure: numpy restatement of the reference's plot-data
kernels (src/graphics/inc/graphics_kernel.cu), the oracle for
hpsim_gb300's headless plot kernels (csrc/plot.cu).  Never used by the
library.

Parity of this restatement is pinned to the kernels' source, not to runs of
them: their only caller is the reference's OpenGL online mode (it needs a
graphics stack, which this project does not use), and a host build of the kernels would change the
float-to-unsigned conversion they rely on (the GPU's saturates; a host
conversion of a negative float is undefined).
"""
from __future__ import annotations

import numpy as np


def _sat_u32(f):
    """cvt.rzi.u32.f32: NaN and negatives to 0, above 2^32 - 1 to 2^32 - 1."""
    f = np.asarray(f, dtype=np.float64)
    out = np.where(np.isnan(f) | (f <= 0), 0.0, np.minimum(np.trunc(f), 4294967295.0))
    return out.astype(np.uint64).astype(np.uint32)


def points(x, y, loss):
    """Set2dPhaseSpaceDataKernel (:52-75): (float)(x, y), lost at (0, 0)."""
    out = np.stack([np.asarray(x, np.float64).astype(np.float32), np.asarray(y, np.float64).astype(np.float32)], -1)
    out[np.asarray(loss) != 0] = 0.0
    return out


def _nmax(a, b):
    return a if np.isnan(b) else (b if (np.isnan(a) or a < b) else a)


def _nmin(a, b):
    return a if np.isnan(b) else (b if (np.isnan(a) or a > b) else a)


def maxmin(x, y, loss=None):
    """BlockMaxMin2DKernel (:86-165) + FindMaxMin2D: (xmax, xmin, ymax,
    ymin); lost particles' seats hold particle 0's values; NaN skipped."""
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    if loss is not None:
        lost = np.asarray(loss) != 0
        x = np.where(lost, x[0], x)
        y = np.where(lost, y[0], y)
    out = []
    for v in (x, y):
        good = v[~np.isnan(v)]
        out += [float(good.max()), float(good.min())] if good.size else [float("nan")] * 2
    return tuple(out)


def histogram(x, loss, nbins, vmin, vmax):
    """HistogramKernel (:229-252) + HistogramReduceKernel: the bin is
    (int)(uint)floorf((float)((x - min) / w)); bins 0 .. nbins-2 count,
    negative ints count in bin 0, above nbins-1 in the last bin, and
    exactly nbins-1 is skipped."""
    x = np.asarray(x, np.float64)[np.asarray(loss) == 0]
    w = (vmax - vmin) / nbins
    q = ((x - vmin) / w).astype(np.float32)
    b = _sat_u32(np.floor(q)).view(np.int32).astype(np.int64)
    hist = np.zeros(nbins, dtype=np.uint32)
    inside = (b >= 0) & (b < nbins - 1)
    np.add.at(hist, b[inside], 1)
    hist[0] += np.count_nonzero(b < 0)
    hist[nbins - 1] += np.count_nonzero(b > nbins - 1)
    return hist


def histogram2d(x, y, loss, nx, ny, frame):
    """Histogram2DKernel (:272-299): live particles in the frame (xmax, xmin,
    ymax, ymin), bins (uint)floorf((float)((v - min) / d)) clamped to the
    last; returns (ny, nx)."""
    xmax, xmin, ymax, ymin = frame
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    keep = (np.asarray(loss) == 0) & (x >= xmin) & (x <= xmax) & (y >= ymin) & (y <= ymax)
    x, y = x[keep], y[keep]
    dx, dy = (xmax - xmin) / nx, (ymax - ymin) / ny
    ix = np.minimum(_sat_u32(np.floor(((x - xmin) / dx).astype(np.float32))), nx - 1).astype(np.int64)
    iy = np.minimum(_sat_u32(np.floor(((y - ymin) / dy).astype(np.float32))), ny - 1).astype(np.int64)
    hist = np.zeros((ny, nx), dtype=np.uint32)
    np.add.at(hist, (iy, ix), 1)
    return hist
