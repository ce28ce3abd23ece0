"""The accuracy gate the bench line reports (bench.accuracy): a pass of the
FP64 oracle over the DTL-like lattice (512 particles, its first 25
elements: 13 quads around 12 gaps, SCHEFF at every element) against itself
passes with zero error, and mistakes planted in a copy of the oracle's
records -- an emittance off by more than the 1e-3 gate, a flipped loss
flag, a transmission count -- fail it.  CPU only."""
import argparse

import numpy as np
import pytest


@pytest.fixture(scope="module")
def oracle_pass():
    import bench
    from oracle import oracle as O
    O.build()
    args = argparse.Namespace(workload="dtl_like", particles=512, precision=None, gaps=bench.GAPS, elements=25)
    bench.resolve(args)
    elems = bench.workload(args)
    b, sim = bench.oracle_sim(args, elems)
    for i in range(len(elems)):
        sim.simulate(i, i)
    return sim.mon.copy(), b.arr("loss").copy(), b.arr("lloss").copy()


def test_identical_passes_meet_the_gate(oracle_pass):
    import bench
    mon, loss, lloss = oracle_pass
    assert mon.shape[0] == 25 and np.all(mon[:, 0] > 0)
    acc = bench.accuracy(mon, mon.copy(), loss, loss.copy(), lloss, lloss.copy())
    assert acc["gate"]["pass"]
    assert acc["transmission_equal"] and acc["loss_flags_equal"] and acc["lloss_equal"]
    assert all(v == 0.0 for v in acc["max_rel_err"].values())


@pytest.mark.parametrize("col", ["eps_x", "eps_y", "eps_z"])
def test_emittance_errors_against_the_gate(oracle_pass, col):
    import bench
    mon, loss, lloss = oracle_pass
    c = bench.MON_EMITS[col]
    k = int(np.argmax(np.abs(mon[:, c])))
    for rel, ok in ((5e-4, True), (2e-3, False)):
        ref = mon.copy()
        ref[k, c] = mon[k, c] / (1.0 + rel)  # the GPU's value is off by rel of the reference
        acc = bench.accuracy(mon, ref, loss, loss, lloss, lloss)
        assert acc["max_rel_err"][col] == pytest.approx(rel, rel=1e-9)
        assert acc["worst_element"][col] == k
        assert acc["gate"]["pass"] is ok


def test_flags_and_transmission_must_be_exact(oracle_pass):
    import bench
    mon, loss, lloss = oracle_pass
    ref_loss = loss.copy()
    ref_loss[7] = 1 if ref_loss[7] == 0 else 0
    acc = bench.accuracy(mon, mon, loss, ref_loss, lloss, lloss)
    assert not acc["loss_flags_equal"] and not acc["gate"]["pass"]
    ref_lloss = lloss.copy()
    ref_lloss[9] = 1 if ref_lloss[9] == 0 else 0
    acc = bench.accuracy(mon, mon, loss, loss, lloss, ref_lloss)
    assert not acc["lloss_equal"] and not acc["gate"]["pass"]
    ref = mon.copy()
    ref[-1, 0] -= 1
    acc = bench.accuracy(mon, ref, loss, loss, lloss, lloss)
    assert not acc["transmission_equal"] and not acc["gate"]["pass"]
