"""FP32 particle path against the reference's own results (golden fixtures)
and the FP64 oracle.

FP32 beams keep x, x', y, y' in FP32 and phi, W as FP32 offsets from a
synchronous particle advanced in FP64 on the host.  Stated tolerances:
  * loss and longitudinal-loss flags: exact (hence transmission exact);
  * rms emittances: relative error <= 1e-3 (the stated accuracy target);
    a collapsed plane (emittance below 1e-3 sigma sigma', e.g. two
    particles, true value 0) is held to an absolute 1e-3 sigma sigma', the
    noise of the difference of products that forms it in FP32;
  * rms sizes: relative error <= 5e-4;
  * centroids (x, x', y, y', phi_r, W): |error| <= 5e-4 sigma of that
    coordinate;
  * particle 0's energy and phase: relative error <= 1e-6.
Typical errors after 165 DTL gaps are a few 1e-6.  A particle that sits on
a mesh-cell or mesh-edge boundary can land on the other side of it in FP32;
with 32k particles one such event moves a size or centroid by up to ~1e-4,
which is what the 5e-4 bounds leave room for."""
import numpy as np
import pytest

from tests import golden_cases as G
from tests.gpu_runs import COORDS, run_gpu

pytestmark = pytest.mark.gpu
CASES = G.case_names()

# monitor columns (include/hps_layout.h)
COUNTS = (0, 1)
CENTROIDS = {2: 3, 4: 5, 7: 8, 9: 10, 12: 13, 14: 15}  # avg column -> its sigma column
SIGMAS = (3, 5, 8, 10, 13, 15)
EMITS = {6: (3, 5), 11: (8, 10), 16: (13, 15)}
SYNC = (17, 18)


def fp32_monitor_errors(m, ref):
    """Largest error of each group of monitor quantities, in the units the
    tolerances are stated in."""
    m, ref = np.asarray(m, float), np.asarray(ref, float)
    out = {"counts": float(np.max(np.abs(m[:, COUNTS] - ref[:, COUNTS])))}
    e = 0.0
    for a, s in CENTROIDS.items():
        sig = np.abs(ref[:, s])
        ok = sig > 0
        if ok.any():
            e = max(e, float(np.max(np.abs(m[ok, a] - ref[ok, a]) / sig[ok])))
    out["centroid"] = e
    e = 0.0
    for s in SIGMAS:
        ok = np.abs(ref[:, s]) > 0
        if ok.any():
            e = max(e, float(np.max(np.abs(m[ok, s] - ref[ok, s]) / np.abs(ref[ok, s]))))
    out["sigma"] = e
    e = 0.0
    for c, (s1, s2) in EMITS.items():
        ss = np.abs(ref[:, s1] * ref[:, s2])
        em = np.abs(np.nan_to_num(ref[:, c]))
        d = np.abs(np.nan_to_num(m[:, c]) - np.nan_to_num(ref[:, c]))
        collapsed = em < 1e-3 * ss
        rel = np.where(collapsed, np.where(d <= 1e-3 * ss, 0.0, 1.0), d / np.maximum(em, 1e-300))
        e = max(e, float(np.max(rel)))
    out["emittance"] = e
    out["sync"] = float(np.max(np.abs(m[:, SYNC] - ref[:, SYNC]) / np.maximum(np.abs(ref[:, SYNC]), 1e-300)))
    return out


def assert_fp32_close(m, ref, what):
    e = fp32_monitor_errors(m, ref)
    assert e["counts"] == 0, (what, e)
    assert e["centroid"] <= 5e-4, (what, e)
    assert e["sigma"] <= 5e-4, (what, e)
    assert e["emittance"] <= 1e-3, (what, e)
    assert e["sync"] <= 1e-6, (what, e)


@pytest.mark.parametrize("name", CASES)
def test_fp32_matches_reference_fixture(name):
    z, meta = G.load(name)
    elems = G.elems_of(z, meta)
    mon, c, _ = run_gpu(elems, meta["n"], spch=meta["spch"], seed=meta["seed"], twiss=tuple(meta["twiss"]),
                        w0=meta["w0"], phi0=meta["phi0"], freq=meta["freq"], precision="fp32")
    assert np.array_equal(c["loss"], z["loss"]), (name, np.flatnonzero(c["loss"] != z["loss"])[:10])
    assert np.array_equal(c["lloss"], z["lloss"]), name
    assert_fp32_close(mon, z["mon"], name)
    alive = z["loss"] == 0
    for k in COORDS:  # per particle: FP32 rounding of O(1e-6) relative to the spread
        a, b = c[k][alive], z[k][alive]
        spread = np.std(b) if b.size > 1 else 1.0
        assert np.max(np.abs(a - b), initial=0.0) <= 1e-4 * max(spread, 1e-12) + 1e-6 * np.max(np.abs(b), initial=0.0), k


def test_fp32_dtl_165_gaps_matches_oracle(oracle):
    """The full DTL-like lattice (165 gaps, 331 elements, SCHEFF 32 x 128 at
    every gap and quad) with 32768 particles: transmission exact against the
    FP64 oracle, statistics at every element within the stated tolerances."""
    from hpsim_gb300 import lattices as L
    elems = L.dtl_like()
    mon, c, _ = run_gpu(elems, 32768, spch=dict(nr=32, nz=128), precision="fp32")
    mo, co = oracle.run(elems, 32768, spch_args=(32, 128, 0.01, 0))
    assert np.array_equal(c["loss"], co["loss"])
    assert np.array_equal(c["lloss"], co["lloss"])
    assert_fp32_close(mon, mo, "dtl165")


def test_fp32_ccl_matches_oracle(oracle):
    from hpsim_gb300 import lattices as L
    elems = L.ccl_like(modules=1, tanks=8)
    mon, c, _ = run_gpu(elems, 8192, spch=dict(nr=32, nz=128), w0=100.0, freq=805.0, precision="fp32")
    mo, co = oracle.run(elems, 8192, spch_args=(32, 128, 0.01, 0), w0=100.0, freq=805.0)
    assert np.array_equal(c["loss"], co["loss"])
    assert np.array_equal(c["lloss"], co["lloss"])
    assert_fp32_close(mon, mo, "ccl")


def test_fp32_ccl_64x256_tensor_cores_match_oracle(oracle):
    """The large configuration's shape: FP32 push, CCL gaps at 805 MHz from
    100 MeV, SCHEFF 64 x 256 at every element with the contraction on the
    tensor cores, against the FP64 oracle: loss flags exact, statistics at
    every element within the stated tolerances; the solver ran its
    tensor-core kernels and no bounded wait gave up."""
    from hpsim_gb300 import lattices as L
    elems = L.ccl_like(modules=1, tanks=2)
    mon, c, objs = run_gpu(elems, 16384, spch=dict(nr=64, nz=256), w0=100.0, freq=805.0, precision="fp32")
    sc = objs[2]
    assert sc.get_counter("tensor_cores") == 1 and sc.get_counter("tc_error") == 0
    mo, co = oracle.run(elems, 16384, spch_args=(64, 256, 0.01, 0), w0=100.0, freq=805.0)
    assert np.array_equal(c["loss"], co["loss"])
    assert np.array_equal(c["lloss"], co["lloss"])
    assert_fp32_close(mon, mo, "ccl 64x256")


def test_fp32_contraction_kernels_agree():
    """The same FP32 DTL run with the contraction on the tensor cores and on
    CUDA cores: identical loss flags, statistics within the FP32 tolerances
    of each other."""
    from hpsim_gb300 import HPSim, lattices as L
    mons, losses = [], []
    for kernel in ("tensor", "cuda"):
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=16384, precision="fp32")
        beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 31)
        beam.set_ref_w(0.75)
        beam.set_ref_phi(0.0)
        sc = HPSim.SpaceCharge(32, 128)
        sc.set_contraction(kernel)
        assert sc.get_counter("tensor_cores") == (kernel == "tensor")
        sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=L.dtl_like(n_gaps=40)), sc)
        sim.enable_monitor(True)
        sim.simulate()
        mons.append(sim.monitor.copy())
        losses.append(beam._loss(0))
    assert np.array_equal(losses[0], losses[1])
    assert_fp32_close(mons[0], mons[1], "tensor vs cuda cores")


def test_fp32_uncertified_statistics_match_oracle(oracle):
    """Kicks whose statistics the element map before them cannot certify:
    particles more than 3 pi behind the bunch are flagged by the
    longitudinal-loss test at the first kick (the good set changes, so the
    moments are swept again about the new <phi>_good) and particles sit
    near the relative-phase wrap.  The fallback sweep runs (the solver's
    counter says so) and flags, counts and statistics still match the FP64
    oracle on the same distribution."""
    import numpy as np
    from hpsim_gb300 import HPSim, lattices as L
    n = 4096
    rng = np.random.default_rng(8)
    b0 = oracle.Beam(n)
    b0.set_waterbag(L.waterbag_twiss(), 0.0, 0.75, 201.25, 77)
    x, xp, y, yp, phi, w = (b0.arr(k).copy() for k in ("x", "xp", "y", "yp", "phi", "w"))
    late = rng.choice(np.arange(1, n), 24, replace=False)
    phi[late[:12]] += 4.0 * np.pi          # beyond <phi> + 3 pi: longitudinal loss
    phi[late[12:]] += np.pi * 0.999        # next to the wrap of the relative phase
    elems = L.small_fodo()[:7]
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=n, precision="fp32")
    beam.set_distribution(x, xp, y, yp, phi, w)
    beam.set_ref_w(0.75)
    beam.set_frequency(201.25)
    sc = HPSim.SpaceCharge(32, 128, 0.10, 0)
    sc.set_remesh_threshold(0.0)
    sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=elems), sc)
    sim.enable_monitor(True)
    sim.simulate()
    assert sc.get_counter("stat_sweeps") > 0
    ob = oracle.Beam(n)
    ob.set_distribution(x, xp, y, yp, phi, w)
    ob.set_ref_w(0.75)
    ob.set_frequency(201.25)
    types, params, _ = L.lattice_arrays(elems)
    sp = oracle.Scheff(32, 128, 0.10, 0)
    sp.set(remesh_threshold=0.0)
    mo = oracle.Sim(ob, types, params, sp).simulate().copy()
    assert np.array_equal(beam._loss(0), ob.arr("loss"))
    assert np.array_equal(beam._loss(1), ob.arr("lloss"))
    assert int(ob.arr("lloss").sum()) >= 12
    assert_fp32_close(sim.monitor, mo, "uncertified")


def test_fp32_graph_replay_is_bit_identical():
    from hpsim_gb300 import lattices as L
    elems = L.small_fodo()
    spch = dict(nr=32, nz=128, interval=0.1, remesh_threshold=0.0)
    _, a, _ = run_gpu(elems, 20000, spch=spch, graph=True, monitor=False, precision="fp32")
    _, b, _ = run_gpu(elems, 20000, spch=spch, graph=False, monitor=False, precision="fp32")
    _, c, _ = run_gpu(elems, 20000, spch=spch, graph=True, monitor=False, precision="fp32")
    for k in COORDS + ("loss", "lloss"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


def test_fp32_restore_and_replay():
    """Save the initial beam, simulate, restore, simulate again (graph
    replay with the synchronous particle restored): identical results."""
    from hpsim_gb300 import HPSim, lattices as L
    elems = L.dtl_like(n_gaps=12)
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=8192, precision="fp32")
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 7)
    beam.set_ref_w(0.75)
    beam.set_ref_phi(0.0)
    beam.save_initial_beam()
    sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=elems), HPSim.SpaceCharge(32, 128))
    sim.simulate()
    first = {k: beam._coord(k) for k in COORDS}
    w_end = beam.get_ref_w()
    beam.restore_initial_beam()
    sim.simulate()
    for k in COORDS:
        assert np.array_equal(beam._coord(k), first[k]), k
    assert beam.get_ref_w() == w_end
