"""Batches in lockstep (hps_batch_set_lockstep / hps_batch_last_mode): when
every simulator of a batch issues the same FP32 launch sequence, each kernel
runs once for all beams (particle kernels over the beams' blocks laid end to
end, mesh kernels with a grid dimension over the beams).  Every beam keeps the
block count and reduction order it has alone; the lockstep kernels are
separate compilations of the same source, and the compiler fuses some
multiply-adds differently in them, so a beam's coordinates agree with the
child-graph form to FP32 rounding (bit for bit when both are compiled without
multiply-add fusion), not bit for bit.  The lockstep form is itself
deterministic run to run.  It is off by default (the child-graph form is
faster on the batch workloads measured).  Ranges with a launch that has no lockstep form
fall back to child graphs and say why."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
COORDS = ("x", "xp", "y", "yp", "phi", "w")


def state(beam):
    out = {k: beam._coord(k) for k in COORDS}
    out["loss"], out["lloss"] = beam._loss(0), beam._loss(1)
    return out


def scan_sims(n, precision="fp32", mesh=(32, 128), seed=5, n_min=2048, n_max=65536, contraction=None,
              monitor=False):
    from hpsim_gb300 import HPSim, lattices as L
    objs = []
    for sb in L.batched_scan(n, seed=seed, n_min=n_min, n_max=n_max):
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=sb.num, precision=precision)
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, sb.seed)
        beam.set_ref_w(0.75)
        beam.set_ref_phi(0.0)
        bl = HPSim.BeamLine(elements=L.scan_lattice(sb, aperture=0.006))
        sc = HPSim.SpaceCharge(mesh[0], mesh[1], 0.1, 0)
        sc.set_remesh_threshold(0.0)
        if contraction:
            sc.set_contraction(contraction)
        sim = HPSim.Simulator(beam, bl, sc)
        if monitor:
            sim.enable_monitor(True)
        objs.append((beam, bl, sc, sim))
    return objs


def dtl_sims(n, num, mesh, contraction, seed=7):
    from hpsim_gb300 import HPSim, lattices as L
    objs = []
    for sb in L.perturbed_beams(n, num, seed):
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=num, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, sb.seed)
        beam.set_ref_w(0.75)
        beam.set_ref_phi(0.0)
        bl = HPSim.BeamLine(elements=L.perturbed(L.dtl_like(n_gaps=6), sb))
        sc = HPSim.SpaceCharge(mesh[0], mesh[1], 0.1, 0)
        sc.set_remesh_threshold(0.0)
        sc.set_contraction(contraction)
        objs.append((beam, bl, sc, HPSim.Simulator(beam, bl, sc)))
    return objs


def run_both(make, calls):
    """The same calls on a lockstep batch and a child-graph batch of equal
    simulators: the beams' states and the lockstep batch's modes."""
    from hpsim_gb300 import HPSim
    out, modes = [], []
    for lock in (True, False):
        objs = make()
        batch = HPSim.Batch([o[3] for o in objs])
        batch.set_lockstep(lock)
        m = []
        for start, end in calls:
            batch.simulate(start, end)
            m.append(batch.last_mode())
        out.append([state(o[0]) for o in objs])
        if lock:
            modes = m
        else:
            assert all(x == ("graphs", "lockstep switched off") for x in m), m
    return out[0], out[1], modes


def assert_same(a, b):
    """Bit for bit."""
    for k, (sa, sb) in enumerate(zip(a, b)):
        for key in sa:
            assert np.array_equal(sa[key], sb[key]), (k, key)


def assert_close(a, b, rel=1e-4):
    """FP32 rounding apart: the same particles survive (up to one in ten
    thousand flipped at an aperture edge), and every coordinate's mean and rms
    over the particles both keep agree to `rel` of the rms."""
    for k, (sa, sb) in enumerate(zip(a, b)):
        n = sa["loss"].size
        both = (sa["loss"] == 0) & (sb["loss"] == 0)
        flipped = int(np.count_nonzero((sa["loss"] == 0) != (sb["loss"] == 0)))
        assert flipped <= max(1, n // 10000), (k, flipped)
        for key in COORDS:
            u, v = sa[key][both], sb[key][both]
            scale = max(float(np.std(v)), 1e-30)
            assert abs(float(np.mean(u) - np.mean(v))) <= rel * scale, (k, key)
            assert abs(float(np.std(u) - np.std(v))) <= rel * scale, (k, key)


def test_lockstep_equals_child_graphs():
    """Uneven beams (2k..64k particles), perturbed set points: a whole run, a
    second run over the same range (the cached lockstep graph, replayed from
    the beams' new state), and a run split in two ranges."""
    a, b, modes = run_both(lambda: scan_sims(6), [(None, None), (None, None)])
    assert modes == [("lockstep", "")] * 2
    assert_close(a, b)
    again, _, _ = run_both(lambda: scan_sims(6), [(None, None), (None, None)])
    assert_same(a, again)  # deterministic
    a, b, modes = run_both(lambda: scan_sims(5, seed=9), [(0, 17), (18, None)])
    assert modes == [("lockstep", "")] * 2
    assert_close(a, b)


@pytest.mark.parametrize("mesh,contraction", [((32, 128), "cuda"), ((64, 256), "tensor"), ((32, 128), "tensor")])
def test_lockstep_mesh_kernels(mesh, contraction):
    """DTL gaps and quads with the CUDA-core and the tensor-core contraction:
    mesh kernels with a grid dimension over the beams."""
    a, b, modes = run_both(lambda: dtl_sims(3, 32768, mesh, contraction), [(None, None)])
    assert modes == [("lockstep", "")]
    assert_close(a, b)
    assert any(np.count_nonzero(s["loss"] == 0) > 0 for s in a)


def test_lockstep_falls_back():
    from hpsim_gb300 import HPSim
    # monitors record per element: child graphs
    objs = scan_sims(3)
    batch = HPSim.Batch([o[3] for o in objs])
    batch.simulate()
    assert batch.last_mode() == ("graphs", "lockstep switched off")  # the default
    objs = scan_sims(3, monitor=True)
    batch = HPSim.Batch([o[3] for o in objs])
    batch.set_lockstep(True)
    batch.simulate()
    mode, why = batch.last_mode()
    assert mode == "graphs" and "monitor" in why
    # FP64 beams have no lockstep form
    objs = scan_sims(3, precision="fp64")
    batch = HPSim.Batch([o[3] for o in objs])
    batch.set_lockstep(True)
    batch.simulate()
    mode, why = batch.last_mode()
    assert mode == "graphs" and why
    # different meshes cannot share a mesh launch
    objs = scan_sims(2) + scan_sims(1, mesh=(64, 128), seed=3)
    batch = HPSim.Batch([o[3] for o in objs])
    batch.set_lockstep(True)
    batch.simulate()
    mode, why = batch.last_mode()
    assert mode == "graphs" and "differ" in why
    # and the fallback's results are those of each beam alone
    for beam, bl, sc, sim in objs[:1]:
        ref = scan_sims(2)[0]
        ref[3].simulate()
        assert np.array_equal(beam._coord("x"), ref[0]._coord("x"))
