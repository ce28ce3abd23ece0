"""Synthetic lattices: synchronous-particle design and element records."""
import math

import numpy as np

from hpsim_gb300 import lattices as L


def test_element_records():
    t, name, p = L.element("Quad", "Q1", length=0.05, gradient=18.0)
    assert t == L.QUAD and p[0] == 0.05 and p[2] == 18.0 and p.shape == (32,)
    t, _, p = L.element(L.RFGAP_DTL, "G1", amplitude=2.5, fit_s5=0.3)
    assert p[4] == 2.5 and p[25] == 0.3 and p[3] == 1.0
    try:
        L.element(L.DRIFT, "D", gradient=1.0)
        raise AssertionError("unknown parameter accepted")
    except ValueError:
        pass


def test_dtl_like_shape_and_design():
    el = L.dtl_like()
    types = [e[0] for e in el]
    assert types.count(L.RFGAP_DTL) == 165 and types.count(L.QUAD) == 166 and len(el) == 331
    assert all(types[i] == L.QUAD for i in range(0, 331, 2))
    names = [e[1] for e in el]
    assert len(set(names)) == len(names)
    w = [e[2][7] for e in el if e[0] == L.RFGAP_DTL]
    assert all(b > a for a, b in zip(w, w[1:])) and w[0] > 0.75
    # cell length = beta_center * lambda (no cell-length phase correction)
    lam = L.CLIGHT / 201.25
    for t, _, p in el:
        if t == L.RFGAP_DTL:
            assert abs(p[0] + 0.04 - p[8] * lam) < 1e-12


def test_waterbag_twiss_rms():
    tw = L.waterbag_twiss()
    bg = L.betagamma_of(0.75, 939.294)
    # total emittance = 8 x rms, unnormalised, cm rad
    assert math.isclose(tw[2], 0.02 / bg / 1000 * 8)
    assert tw[1] == 20.0 and tw[0] == 0.0


def test_ccl_like_shape():
    el = L.ccl_like(modules=1, tanks=2, cells=4)
    types = [e[0] for e in el]
    assert types.count(L.RFGAP_CCL) == 8 and types.count(L.QUAD) == 4 and types.count(L.DRIFT) == 2
    assert np.all(np.diff([e[2][7] for e in el if e[0] == L.RFGAP_CCL]) > 0)
