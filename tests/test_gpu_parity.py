"""CUDA path (FP64 beams) against the reference's own results (golden
fixtures) and the FP64 oracle.

Bar: loss flags and transmitted counts exact; coordinates within rtol 1e-8
(the CUDA and host math libraries differ in the last bits, nvcc fuses
multiply-adds, and the deposit accumulates 2^-36 fixed-point weights);
monitor statistics within 1e-6 relative."""
import numpy as np
import pytest

from tests import golden_cases as G
from tests.gpu_runs import COORDS, run_gpu

pytestmark = pytest.mark.gpu
CASES = G.case_names()


@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_fixture(name):
    z, meta = G.load(name)
    elems = G.elems_of(z, meta)
    mon, c, _ = run_gpu(elems, meta["n"], spch=meta["spch"], seed=meta["seed"], twiss=tuple(meta["twiss"]),
                        w0=meta["w0"], phi0=meta["phi0"], freq=meta["freq"])
    assert np.array_equal(c["loss"], z["loss"]), (name, np.flatnonzero(c["loss"] != z["loss"])[:10])
    assert np.array_equal(c["lloss"], z["lloss"]), name
    alive = z["loss"] == 0
    for k in COORDS:
        a, b = c[k][alive], z[k][alive]
        assert np.allclose(a, b, rtol=1e-8, atol=1e-11), (name, k, np.max(np.abs(a - b)))
    ok = G.monitor_close(mon, z["mon"], 1e-6)
    assert ok.all(), (name, np.argwhere(~ok)[:5])


def test_gpu_matches_oracle_dtl_long(oracle):
    """48 gaps of the DTL-like lattice with a full SCHEFF solve at every gap
    and quad, 8192 particles: transmission exact, statistics at 1e-6."""
    from hpsim_gb300 import lattices as L
    elems = L.dtl_like(n_gaps=48)
    spch = dict(nr=32, nz=128, remesh_threshold=0.0)
    mon, c, _ = run_gpu(elems, 8192, spch=spch)
    mo, co = oracle.run(elems, 8192, spch_args=(32, 128, 0.01, 0), spch_set={"remesh_threshold": 0.0})
    assert np.array_equal(c["loss"], co["loss"])
    assert np.array_equal(c["lloss"], co["lloss"])
    ok = G.monitor_close(mon, mo, 1e-6)
    assert ok.all(), np.argwhere(~ok)[:5]


def test_graph_replay_is_bit_identical():
    """Captured-graph replay, direct launches and a second run agree bitwise
    (every reduction and the deposit are order-independent)."""
    from hpsim_gb300 import lattices as L
    elems = L.small_fodo()
    spch = dict(nr=32, nz=128, interval=0.1, remesh_threshold=0.0)
    _, a, _ = run_gpu(elems, 20000, spch=spch, graph=True, monitor=False)
    _, b, _ = run_gpu(elems, 20000, spch=spch, graph=False, monitor=False)
    _, c, _ = run_gpu(elems, 20000, spch=spch, graph=True, monitor=False)
    for k in COORDS + ("loss", "lloss"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


def test_repeated_simulate_replays_graph():
    """A second simulate() of the same range from the same host state reuses
    the captured graph and gives the same result as the first."""
    from hpsim_gb300 import HPSim, lattices as L
    elems = L.small_fodo()
    n = 8192
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=n)
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 5)
    beam.set_ref_w(0.75)
    beam.save_initial_beam()
    bl = HPSim.BeamLine(elements=elems)
    sc = HPSim.SpaceCharge(32, 128, 0.1, 0)
    sim = HPSim.Simulator(beam, bl, sc)
    sim.simulate()
    x1 = beam.get_x("all")
    beam.restore_initial_beam()
    sc2 = HPSim.SpaceCharge(32, 128, 0.1, 0)
    sim2 = HPSim.Simulator(beam, bl, sc2)
    sim2.simulate()
    x2 = beam.get_x("all")
    assert np.array_equal(x1, x2)
