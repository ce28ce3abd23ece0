"""The batched-scan workload (hpsim_gb300.lattices.batched_scan): seeded,
particle counts log-uniform in the stated range, set points within their
stated spreads, lattices that differ only in those set points."""
import math

import numpy as np

from hpsim_gb300 import lattices as L


def test_scan_is_seeded_and_in_range():
    a = L.batched_scan(256, seed=7)
    b = L.batched_scan(256, seed=7)
    assert a == b and a != L.batched_scan(256, seed=8)
    nums = np.array([s.num for s in a])
    assert nums.min() >= 16384 and nums.max() <= 524288
    # log-uniform: about half below the geometric midpoint
    mid = math.sqrt(16384 * 524288)
    assert 0.35 < np.mean(nums < mid) < 0.65
    assert all(0.95 <= s.rf_scale <= 1.05 and 0.97 <= s.quad_scale <= 1.03 for s in a)
    assert all(abs(s.phase_offset) <= math.radians(3.0) for s in a)
    assert len({s.seed for s in a}) == 256


def test_scan_lattice_perturbs_only_the_set_points():
    sb = L.ScanBeam(num=1000, seed=1, rf_scale=1.02, phase_offset=0.01, quad_scale=0.98)
    base, pert = L.small_fodo(), L.scan_lattice(sb)
    assert [e[:2] for e in base] == [e[:2] for e in pert]
    for (code, _, p0), (_, _, p1) in zip(base, pert):
        if code == L.BUNCHER:
            v, ph = L.param_index(L.BUNCHER, "voltage"), L.param_index(L.BUNCHER, "phase")
            assert p1[v] == p0[v] * 1.02 and p1[ph] == p0[ph] + 0.01
        elif code == L.QUAD:
            g = L.param_index(L.QUAD, "gradient")
            assert p1[g] == p0[g] * 0.98
        else:
            assert np.array_equal(p0, p1)


def test_ccl_batch_perturbs_gaps_and_quads():
    beams = L.ccl_batch(16)
    assert beams == L.ccl_batch(16) and len(beams) == 16
    assert all(b.num == 1 << 20 and 0.99 <= b.rf_scale <= 1.01 and 0.97 <= b.quad_scale <= 1.03 and
               abs(b.phase_offset) <= np.radians(1.0) for b in beams)
    assert len({b.seed for b in beams}) == 16
    sb = L.ScanBeam(num=10, seed=1, rf_scale=1.01, phase_offset=0.002, quad_scale=0.99)
    base = L.ccl_like(modules=1, tanks=2, cells=2)
    pert = L.perturbed(base, sb)
    assert [e[:2] for e in base] == [e[:2] for e in pert]
    for (code, _, p0), (_, _, p1) in zip(base, pert):
        if code == L.RFGAP_CCL:
            a, s = L.param_index(code, "amplitude"), L.param_index(code, "phase_shift")
            assert p1[a] == p0[a] * 1.01 and p1[s] == p0[s] + 0.002
            rest = [k for k in range(len(p0)) if k not in (a, s)]
            assert np.array_equal(p0[rest], p1[rest])
        elif code == L.QUAD:
            g = L.param_index(L.QUAD, "gradient")
            assert p1[g] == p0[g] * 0.99
        else:
            assert np.array_equal(p0, p1)
