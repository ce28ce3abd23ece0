"""Headless plot kernels (csrc/plot.cu through hpsim_gb300.plotdata) against
the numpy restatement of the reference's graphics kernels (oracle/plotdata.py),
on FP64 and FP32 beams after a lattice that loses particles; plus hand-made
values on the rules' edges and output into device memory."""
import numpy as np
import pytest

from oracle import plotdata as P

pytestmark = pytest.mark.gpu
COORDS = ("x", "xp", "y", "yp", "phi", "w")


def tracked_beam(precision):
    from hpsim_gb300 import HPSim, lattices as L
    elems = L.small_fodo(aperture=0.004)
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=50000, precision=precision)
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 9)
    beam.set_ref_w(0.75)
    sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=elems), HPSim.SpaceCharge(32, 128, 0.1))
    sim.simulate()
    return beam


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_plot_data_matches_oracle(precision):
    from hpsim_gb300 import plotdata as G
    beam = tracked_beam(precision)
    c = {k: beam._coord(k) for k in COORDS}  # FP64 values (FP32: offset + synchronous particle)
    loss = beam._loss(0)
    assert 0 < np.count_nonzero(loss) < len(loss)
    for cx, cy in (("x", "xp"), ("y", "yp"), ("phi", "w")):
        assert np.array_equal(G.phase_space(beam, cx, cy), P.points(c[cx], c[cy], loss)), (cx, cy)
        mm = G.maxmin(beam, cx, cy)
        assert mm == P.maxmin(c[cx], c[cy], loss), (cx, cy)
        assert G.maxmin(beam, cx, cy, live_only=False) == P.maxmin(c[cx], c[cy], None)
        for nb in (1, 2, 64, 1000):
            lo, hi = mm[1], mm[0]
            assert np.array_equal(G.histogram(beam, cx, nb, lo, hi), P.histogram(c[cx], loss, nb, lo, hi)), (cx, nb)
        assert np.array_equal(G.histogram2d(beam, cx, cy, 64, 48, mm),
                              P.histogram2d(c[cx], c[cy], loss, 64, 48, mm)), (cx, cy)


def test_rule_edges_on_a_hand_made_beam():
    from hpsim_gb300 import HPSim, plotdata as G
    x = np.array([0.5, 0.5, 1.5, 2.5, 3.5, 3.0, 4.0, 7.0, -0.5, -3.0, 1.0, 1.0 - 2.0 ** -30])
    n = len(x)
    z = np.zeros(n)
    loss = np.zeros(n, np.uint32)
    loss[10] = 3
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.0, num=n)
    beam.set_distribution(x, z, z, z, z, z + 0.75, loss, None)
    xs = beam._coord("x")  # particle 0 is put on axis
    h = G.histogram(beam, "x", 4, 0.0, 4.0)
    assert np.array_equal(h, P.histogram(xs, loss, 4, 0.0, 4.0))
    assert G.maxmin(beam, "x", "w") == P.maxmin(xs, beam._coord("w"), loss)


def test_output_into_device_memory():
    torch = pytest.importorskip("torch")
    from hpsim_gb300 import plotdata as G
    beam = tracked_beam("fp32")
    n = beam.get_size()
    pts = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    G.phase_space(beam, "x", "xp", device_ptr=pts.data_ptr())
    hist = torch.empty(100, dtype=torch.int32, device="cuda")
    lo, hi = -0.004, 0.004
    G.histogram(beam, "x", 100, lo, hi, device_ptr=hist.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(pts.cpu().numpy(), G.phase_space(beam, "x", "xp"))
    assert np.array_equal(hist.cpu().numpy().view(np.uint32), G.histogram(beam, "x", 100, lo, hi))
