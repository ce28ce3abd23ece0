"""Batches (hps_batch_*, HPSim.Batch): beams of uneven sizes and perturbed
set points advanced in one graph launch give, beam by beam, the results of
simulating each alone (bit-identical: every kernel is deterministic), and
one of them matches the FP64 oracle."""
import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu
COORDS = ("x", "xp", "y", "yp", "phi", "w")


def make(sb, precision, monitor=False):
    from hpsim_gb300 import HPSim, lattices as L
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=sb.num, precision=precision)
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, sb.seed)
    beam.set_ref_w(0.75)
    beam.set_ref_phi(0.0)
    bl = HPSim.BeamLine(elements=L.scan_lattice(sb, aperture=0.006))
    sc = HPSim.SpaceCharge(32, 128, 0.1, 0)
    sc.set_remesh_threshold(0.0)
    sim = HPSim.Simulator(beam, bl, sc)
    if monitor:
        sim.enable_monitor(True)
    return beam, bl, sc, sim


def state(beam):
    out = {k: beam._coord(k) for k in COORDS}
    out["loss"], out["lloss"] = beam._loss(0), beam._loss(1)
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_equals_each_beam_alone(precision):
    from hpsim_gb300 import HPSim, lattices as L
    scan = L.batched_scan(12, seed=5, n_min=2048, n_max=65536)
    objs = [make(sb, precision, monitor=True) for sb in scan]
    batch = HPSim.Batch([o[3] for o in objs])
    batch.simulate()
    assert batch.last_time_ms() > 0
    for sb, (beam, _, _, sim) in zip(scan, objs):
        ref = make(sb, precision, monitor=True)
        ref[3].simulate()
        a, b = state(beam), state(ref[0])
        for k in a:
            assert np.array_equal(a[k], b[k]), (sb, k)
        assert np.array_equal(np.nan_to_num(sim.monitor), np.nan_to_num(ref[3].monitor))
    # a rewound range resets the simulators and captures them again
    batch.simulate(0, 10)
    for sb, (beam, *_) in zip(scan, objs):
        ref = make(sb, precision)
        ref[3].simulate()
        ref[3].simulate(0, 10)
        assert np.array_equal(beam._coord("x"), ref[0]._coord("x")), sb


def test_batch_beam_matches_oracle(oracle):
    from hpsim_gb300 import HPSim, lattices as L
    scan = L.batched_scan(4, seed=11, n_min=4096, n_max=8192)
    objs = [make(sb, "fp64", monitor=True) for sb in scan]
    HPSim.Batch([o[3] for o in objs]).simulate()
    sb = scan[2]
    mo, co = oracle.run(L.scan_lattice(sb, aperture=0.006), sb.num, spch_args=(32, 128, 0.1, 0),
                        spch_set={"remesh_threshold": 0.0}, seed=sb.seed)
    c = state(objs[2][0])
    assert np.array_equal(c["loss"], co["loss"])
    ok = G.monitor_close(objs[2][3].monitor, mo, 1e-6)
    assert ok.all(), np.argwhere(~ok)[:5]


def test_batch_rejects_shared_beams():
    from hpsim_gb300 import HPSim, lattices as L
    sb = L.batched_scan(1, seed=3, n_min=1024, n_max=1024)[0]
    beam, bl, sc, sim = make(sb, "fp32")
    sim2 = HPSim.Simulator(beam, bl, HPSim.SpaceCharge(32, 128, 0.1, 0))
    with pytest.raises(Exception):
        HPSim.Batch([sim, sim2])


def test_autotune_leaves_no_trace_and_its_shape_reproduces():
    """The autotuner times candidate launch shapes on the simulator's own
    run and restores the beam, solver and engine state: a simulation after
    tuning equals, bit for bit, a fresh simulator of the same beam run with
    the chosen shape set by hand; a second tuning of the same configuration
    comes from the cache (nothing timed)."""
    import numpy as np
    from hpsim_gb300 import HPSim, lattices as L

    def make():
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=65536, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 5)
        beam.set_ref_w(0.75)
        beam.set_ref_phi(0.0)
        sc = HPSim.SpaceCharge(32, 128)
        sc.set_remesh_threshold(0.0)
        return beam, sc, HPSim.Simulator(beam, HPSim.BeamLine(elements=L.dtl_like(n_gaps=10)), sc)

    beam, sc, sim = make()
    res = sim.autotune(reps=2)
    assert len(res["ms"]) >= 4 and all(t > 0 for t in res["ms"])
    assert sim.get_shape() == res["shape"]
    assert res["shape"]["contraction"] in (0, 1) and 1 <= res["shape"]["deposit_blocks_per_sm"] <= 4
    assert res["shape"]["deposit_threads"] * res["shape"]["deposit_blocks_per_sm"] <= 1024
    sim.enable_monitor(True)
    sim.simulate()
    tuned = sim.monitor.copy(), beam._coord("xp")
    beam2, sc2, sim2 = make()
    sim2.set_shape(res["shape"])
    sim2.enable_monitor(True)
    sim2.simulate()
    assert np.array_equal(tuned[0], sim2.monitor)
    assert np.array_equal(tuned[1], beam2._coord("xp"))
    beam3, sc3, sim3 = make()
    again = sim3.autotune(reps=2)
    assert again["ms"] == [] and again["shape"] == res["shape"]


def test_batch_autotune():
    from hpsim_gb300 import HPSim, lattices as L
    objs = []
    for sb in L.batched_scan(6, n_min=16384, n_max=65536):
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=sb.num, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, sb.seed)
        beam.set_ref_w(0.75)
        sc = HPSim.SpaceCharge(32, 128, 0.10, 0)
        objs.append((beam, sc, HPSim.Simulator(beam, HPSim.BeamLine(elements=L.scan_lattice(sb)), sc)))
    batch = HPSim.Batch([o[2] for o in objs])
    res = batch.autotune(reps=1)
    assert len(res["ms"]) >= 4
    for o in objs:
        assert o[2].get_shape() == res["shape"]
    batch.simulate()


def test_aggregated_deposit_adds_give_the_same_table():
    """The deposit's warp-aggregated histogram adds (launch-shape knob
    deposit_aggregate) sum the same integer weights in another order: the
    simulation is bit for bit the one with one atomic per particle and bin,
    on the CUDA-core and the tensor-core contraction."""
    import numpy as np
    from hpsim_gb300 import HPSim, lattices as L
    for contraction in (0, 1):
        out = []
        for agg in (0, 1):
            beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=65536, precision="fp32")
            beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 21)
            beam.set_ref_w(0.75)
            beam.set_ref_phi(0.0)
            sc = HPSim.SpaceCharge(32, 128)
            sc.set_remesh_threshold(0.0)
            sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=L.dtl_like(n_gaps=10)), sc)
            sim.set_shape({"contraction": contraction, "deposit_blocks_per_sm": 3, "sweep_blocks_per_sm": 0,
                           "deposit_aggregate": agg})
            assert sim.get_shape()["deposit_aggregate"] == agg
            sim.enable_monitor(True)
            sim.simulate()
            out.append((sim.monitor.copy(), [beam._coord(k) for k in ("x", "xp", "y", "yp", "phi", "w")]))
        assert np.array_equal(out[0][0], out[1][0])
        for a, b in zip(out[0][1], out[1][1]):
            assert np.array_equal(a, b)


def test_deposit_block_sizes_agree():
    """The deposit's block size (launch-shape knob deposit_threads: 256, 512,
    1024 threads) changes the fixed-point scale of the per-block histograms,
    not the physics: the same transmission and loss flags, emittances within
    1e-4 relative at every element."""
    import numpy as np
    from hpsim_gb300 import HPSim, lattices as L
    runs = {}
    for threads, per_sm in ((256, 3), (512, 1), (1024, 1)):
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=65536, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 33)
        beam.set_ref_w(0.75)
        beam.set_ref_phi(0.0)
        sc = HPSim.SpaceCharge(64, 256)
        sc.set_remesh_threshold(0.0)
        sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=L.dtl_like(n_gaps=8)), sc)
        sim.set_shape({"contraction": 0, "deposit_blocks_per_sm": per_sm, "sweep_blocks_per_sm": 0,
                       "deposit_aggregate": 0, "deposit_threads": threads})
        sim.enable_monitor(True)
        sim.simulate()
        runs[threads] = (sim.monitor.copy(), beam._loss(0), beam._loss(1))
    ref = runs[256]
    for threads in (512, 1024):
        mon, loss, lloss = runs[threads]
        assert np.array_equal(loss, ref[1]) and np.array_equal(lloss, ref[2])
        assert np.array_equal(mon[:, 0], ref[0][:, 0])
        for i in (6, 11, 16):
            assert np.max(np.abs(mon[:, i] / ref[0][:, i] - 1.0)) <= 1e-4, (threads, i)
