"""The plot-data oracle (oracle/plotdata.py) on hand-worked cases of the
reference kernels' rules (src/graphics/inc/graphics_kernel.cu)."""
import numpy as np

from oracle import plotdata as P


def test_histogram_bin_rules():
    # 4 bins over [0, 4): width 1
    x = np.array([0.5, 1.5, 2.5,      # bins 0, 1, 2
                  3.5, 3.0,           # inside the last bin: skipped
                  4.0, 7.0,           # at / above the maximum: last bin
                  -0.5, -3.0,         # below the minimum: bin 0 (saturating conversion)
                  np.nan,             # NaN: bin 0
                  1.0])               # a lost particle
    loss = np.zeros(len(x), np.uint32)
    loss[-1] = 7
    assert P.histogram(x, loss, 4, 0.0, 4.0).tolist() == [4, 1, 1, 2]


def test_histogram_quotient_is_rounded_to_fp32():
    # (x - min) / w just below 1 in FP64 rounds to 1.0f: bin 1, not 0
    w = 1.0
    x = np.array([1.0 - 2.0 ** -30])
    assert P.histogram(x, np.zeros(1, np.uint32), 4, 0.0, 4.0 * w).tolist() == [0, 1, 0, 0]


def test_histogram_huge_values_wrap_to_bin_zero():
    # (uint)floorf(q) >= 2^31 reads as a negative int: the reference counts it in bin 0
    x = np.array([3.0e9, 5.0e9])
    assert P.histogram(x, np.zeros(2, np.uint32), 8, 0.0, 8.0).tolist() == [2, 0, 0, 0, 0, 0, 0, 0]


def test_maxmin_uses_particle_zero_for_lost_seats_and_skips_nan():
    x = np.array([0.5, 2.0, -1.0, np.nan, 9.0])
    y = np.array([0.1, 0.2, 0.3, 0.4, np.nan])
    loss = np.array([1, 0, 0, 0, 5], np.uint32)  # particle 0 lost: its value still counts
    assert P.maxmin(x, y, loss) == (2.0, -1.0, 0.4, 0.1)
    assert P.maxmin(x, y, None) == (9.0, -1.0, 0.4, 0.1)


def test_histogram2d_frame_and_clamp():
    x = np.array([0.0, 1.0, 0.99, 0.5, 2.0])
    y = np.array([0.0, 1.0, 0.0, 0.5, 0.5])
    loss = np.zeros(5, np.uint32)
    h = P.histogram2d(x, y, loss, 2, 2, (1.0, 0.0, 1.0, 0.0))
    # (0,0) -> bin (0,0); (1,1) on the edge -> clamped (1,1); (0.99, 0) -> (1,0);
    # (0.5, 0.5) -> (1,1); x = 2 outside the frame
    assert h.tolist() == [[1, 1], [0, 2]]


def test_points_put_lost_particles_at_the_origin():
    p = P.points([1.5, 2.5], [3.5, 4.5], np.array([0, 3], np.uint32))
    assert p.dtype == np.float32 and p.tolist() == [[1.5, 3.5], [0.0, 0.0]]
