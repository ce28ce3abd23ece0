"""The FP64 oracle against fixtures generated by the reference's own code
(oracle/_ref, tests/golden/make_golden.py), and against that build directly
where it exists."""
import numpy as np
import pytest

from tests import golden_cases as G

CASES = G.case_names()


def run_oracle(O, z, meta):
    elems = G.elems_of(z, meta)
    sa, extra = G.spch_args(meta)
    return O.run(elems, meta["n"], spch_args=sa, spch_set=extra, seed=meta["seed"],
                 twiss=tuple(meta["twiss"]), w0=meta["w0"], phi0=meta["phi0"], freq=meta["freq"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(oracle, name):
    z, meta = G.load(name)
    mon, c = run_oracle(oracle, z, meta)
    # loss flags: exact
    assert np.array_equal(c["loss"], z["loss"]), name
    assert np.array_equal(c["lloss"], z["lloss"]), name
    alive = z["loss"] == 0
    if meta["spch"] is None:
        # no reduction enters the particle update: bit-identical
        for k in G.COORDS:
            assert np.array_equal(c[k], z[k]), (name, k)
    else:
        for k in G.COORDS:
            # summation order of the moments differs; coordinates agree to ~1e-13
            a, b = c[k][alive], z[k][alive]
            assert np.allclose(a, b, rtol=1e-10, atol=1e-12), (name, k, np.abs(a - b).max())
    ok = G.monitor_close(mon, z["mon"], 1e-7)
    assert ok.all(), (name, np.argwhere(~ok)[:5])


def test_fixture_set_exercises_losses():
    z, meta = G.load("loss_mix_sc")
    lost = z["loss"][z["loss"] != 0]
    kinds = set(np.unique(lost).tolist())
    assert len(lost) > 20 and len(kinds) >= 4, kinds


def test_initial_distributions(oracle):
    z = np.load(f"{G.GOLDEN}/initial_distributions.npz")
    n = len(z["waterbag_x"])
    b = oracle.Beam(n)
    b.set_waterbag(z["twiss"], 0.1, 0.75, 201.25, 777)
    c = b.coords()
    for k in G.COORDS:
        assert np.array_equal(c[k], z[f"waterbag_{k}"]), k
    d = oracle.Beam(n)
    a = z["dc_args"]
    d.set_dc(a[:6], a[6], a[7], a[8], int(a[9]))
    c = d.coords()
    for k in G.COORDS:
        assert np.array_equal(c[k], z[f"dc_{k}"]), k


def test_scheff_tables(oracle):
    z = np.load(f"{G.GOLDEN}/scheff_tables_8x64.npz")
    from hpsim_gb300 import lattices as L
    elems = [L.element(L.DRIFT, "D1", length=0.02)]
    types, params, _ = L.lattice_arrays(elems)
    b = oracle.Beam(2048)
    b.set_waterbag(L.waterbag_twiss(), 0.0, 0.75, 201.25, 99)
    b.set_ref_w(0.75)
    b.set_ref_phi(0.0)
    s = oracle.Scheff(8, 64, 0.02, 0)
    s.set(remesh_threshold=0.0)
    sim = oracle.Sim(b, types, params, s)
    sim.simulate()
    bin_, fld1, fld2 = s.tables()
    assert np.allclose(bin_, z["bin"], rtol=1e-12, atol=1e-12)
    assert np.allclose(fld1, z["fld1"], rtol=1e-12, atol=1e-13 * np.abs(z["fld1"]).max())
    assert np.allclose(fld2, z["fld2"], rtol=1e-10, atol=1e-12 * np.abs(z["fld2"]).max())
    # the 8x64 mesh is smaller than one 1024-thread block: the reference
    # leaves the (nz, nr) corner of the field table at zero
    assert z["fld2"][-2:].tolist() == [0.0, 0.0] and fld2[-2:].tolist() == [0.0, 0.0]


def test_oracle_against_reference_build(oracle):
    from oracle import refimpl as R
    if not R.available():
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    from hpsim_gb300 import lattices as L
    elems = L.dtl_like(n_gaps=8, seed=7)
    mr, cr = R.run(elems, 700, spch=dict(nr=16, nz=64, remesh_threshold=0.02), seed=31)
    mo, co = oracle.run(elems, 700, spch_args=(16, 64, 0.01, 0), spch_set={"remesh_threshold": 0.02}, seed=31)
    assert np.array_equal(cr["loss"], co["loss"])
    for k in G.COORDS:
        assert np.allclose(cr[k], co[k], rtol=1e-10, atol=1e-12), k


def test_field_from_charge_table(oracle):
    """The table stage alone: the reference's charge table and mesh
    parameters through the oracle's Green's table and contraction give the
    reference's field table."""
    import ctypes as C
    z = np.load(f"{G.GOLDEN}/scheff_tables_8x64.npz")
    m = z["mesh"]
    s = oracle.Scheff(8, 64, 0.02, 0)
    s.s.dr, s.s.dz = m[0], m[1]
    oracle.lib().orc_scheff_green_table(s.h, m[2], m[3], int(m[4]), m[5], int(m[6]))
    bins = np.ascontiguousarray(z["bin"])  # every z[...] reads a new array: keep this one alive
    C.memmove(s.s.bin, bins.ctypes.data, bins.nbytes)
    C.memset(s.s.fld2, 0, z["fld2"].nbytes)
    oracle.lib().orc_scheff_contract(s.h)
    _, fld1, fld2 = s.tables()
    assert np.allclose(fld1, z["fld1"], rtol=1e-12, atol=1e-13 * np.abs(z["fld1"]).max())
    assert np.allclose(fld2, z["fld2"], rtol=1e-11, atol=1e-13 * np.abs(z["fld2"]).max())


def test_first_simulate_keeps_the_engine_state_of_its_creation(oracle):
    """SimulationEngine's previous end index is an int holding UINT_MAX (-1),
    so its first Simulate call does not reset: a beam configured after the
    simulator was created keeps the creation-time design energy and
    wavelength (zero frequency: the phase does not advance through the first
    quad), and the reference build does the same.  (Its RF gaps then run
    with a design energy of zero, where the reference's arithmetic gives
    non-finite phases and loses every particle; that degenerate input is not
    restated.)"""
    from hpsim_gb300 import lattices as L
    from oracle import refimpl as R
    elems = L.dtl_like(n_gaps=2, seed=3)
    m0, _ = oracle.run(elems, 500, seed=5)
    m1, _ = oracle.run(elems, 500, seed=5, late=True)
    assert m0[0, 18] != 0.0 and m1[0, 18] == 0.0  # particle 0's phase after the first quad
    if R.available():
        mr, _ = R.run(elems, 500, seed=5, late=True)
        assert mr[0, 18] == 0.0 and np.allclose(mr[0], m1[0], rtol=1e-10, atol=0.0)


def test_oracle_against_reference_build_ccl_64x256(oracle):
    """The large configuration's mesh and elements: CCL gaps at 805 MHz from
    100 MeV, a doublet and a drift, SCHEFF 64 x 256 with a solve at every
    element, 2048 particles -- the oracle against the reference's own code."""
    from oracle import refimpl as R
    if not R.available():
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    from hpsim_gb300 import lattices as L
    elems = L.ccl_like(modules=1, tanks=1, cells=2)
    kw = dict(seed=9, w0=100.0, freq=805.0, twiss=L.waterbag_twiss(w0=100.0, freq=805.0))
    mr, cr = R.run(elems, 2048, spch=dict(nr=64, nz=256, remesh_threshold=0.0), **kw)
    mo, co = oracle.run(elems, 2048, spch_args=(64, 256, 0.01, 0), spch_set={"remesh_threshold": 0.0}, **kw)
    assert np.array_equal(cr["loss"], co["loss"])
    for k in G.COORDS:
        assert np.allclose(cr[k], co[k], rtol=1e-10, atol=1e-12 * np.abs(co[k]).max()), k
    assert G.monitor_close(mo, mr, 1e-7).all()
